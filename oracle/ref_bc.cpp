// ref_bc.cpp -- TEST INFRASTRUCTURE ONLY.  Drives the reference's own
// boundary routine intialise() (Flow_Initialisation.cpp, built from the copy
// under oracle/_ref/) on arrays in the reference layout, to pin the oracle's
// restatement (oracle_boundary_fill).  sing (may be null) is the
// singular-node table, six slots per row.
#include <cstdint>

#include "bc_ref_shim.h"

vector<MNODE> node;
vector<singul> singular;
vector<FLOW_VARIABLES> FLOW;
vector<int> inlet_node, outlet_node, wall_node, boundary_node;
vector<int> sd_inlet_node, sd_outlet_node, sd_wall_node, sd_boundary_node;
int out_node, inl_node, wal_node, bou_node, sd_out_node, sd_inl_node, sd_wal_node, sd_bou_node;
int initial, i, h, sd_node;
double Mach;

#pragma pack(push, 1)
struct ref_grid_row { double x, y, z; int32_t N[6]; int32_t ID, loc; };
#pragma pack(pop)

extern "C" void ref_boundary_fill(const ref_grid_row *grid, FLOW_VARIABLES *flow, int n_rows,
                                  const int32_t *outlet, int n_outlet, const int32_t *inlet, int n_inlet,
                                  const int32_t *boundary, int n_boundary, const int32_t *wall, int n_wall,
                                  double mach, int initial_flag, int n_owned, const int32_t *sing)
{
    node.assign(n_rows, MNODE{});
    singular.assign(n_rows, singul{});
    if (sing)
        for (int r = 0; r < n_rows; ++r)
            for (int s = 0; s < 6; ++s) singular[r].n_n[s] = sing[(size_t)r * 6 + s];
    FLOW.assign(flow, flow + n_rows);
    for (int r = 0; r < n_rows; ++r) {
        for (int s = 0; s < 6; ++s) node[r].n_n[s] = grid[r].N[s];
        node[r].loc = grid[r].loc;
        node[r].ID = grid[r].ID;
    }
    outlet_node.assign(outlet, outlet + n_outlet);
    inlet_node.assign(inlet, inlet + n_inlet);
    boundary_node.assign(boundary, boundary + n_boundary);
    wall_node.assign(wall, wall + n_wall);
    out_node = n_outlet;
    inl_node = n_inlet;
    bou_node = n_boundary;
    wal_node = n_wall;
    sd_out_node = sd_inl_node = sd_bou_node = sd_wal_node = 0;
    initial = initial_flag;
    sd_node = n_owned;
    Mach = mach;
    intialise(0);
    for (int r = 0; r < n_rows; ++r) flow[r] = FLOW[r];
}

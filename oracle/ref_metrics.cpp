// ref_metrics.cpp -- TEST INFRASTRUCTURE ONLY.  Drives the reference's own
// geometry routines -- metric_term() (Grid_Transformation.cpp) and the
// half-point block of Main.cpp:2369-2440 (ref_half_points_body, cut out by
// build_ref.sh) -- on a node table in the reference layout, to pin the
// oracle's restatement and the library's producer.
#include <cstdint>

#include "metric_ref_shim.h"

vector<MNODE> node;
vector<JACOB> jacobian;
vector<JAC> jac;
vector<TEMP_JAC> jaco;
vector<ELEM> CD;
vector<TRANSFORMED> metric;
vector<DETERM> deter;
vector<double> det;
vector<int> all_boundary_nodes;
int all_bou_node, NUMNP, h, i, sd_node;
double del_zeta = 1.0, del_eta = 1.0;

#pragma pack(push, 1)
struct ref_grid_row { double x, y, z; int32_t N[6]; int32_t ID, loc; };
#pragma pack(pop)

static void load_nodes(const ref_grid_row *grid, int n_rows)
{
    node.assign(n_rows, MNODE{});
    for (int r = 0; r < n_rows; ++r) {
        node[r].x = grid[r].x;
        node[r].y = grid[r].y;
        node[r].z = grid[r].z;
        for (int s = 0; s < 6; ++s) node[r].n_n[s] = grid[r].N[s];
        node[r].ID = grid[r].ID;
        node[r].loc = grid[r].loc;
    }
}

// metric_term() on rows 1..n_rows-1: its boundary-node list is every row
// with a missing neighbour, in row order (the lines start there).
extern "C" void ref_compact_metrics(const ref_grid_row *grid, int n_rows, double *det_out, double *metric_out)
{
    load_nodes(grid, n_rows);
    jacobian.assign(n_rows, JACOB{});
    jac.assign(n_rows, JAC{});
    jaco.assign(n_rows, TEMP_JAC{});
    CD.assign(1, ELEM{});
    metric.assign(n_rows, TRANSFORMED{});
    det.assign(n_rows, 0.0);
    all_boundary_nodes.clear();
    for (int r = 1; r < n_rows; ++r)
        for (int s = 0; s < 6; ++s)
            if (grid[r].N[s] == 0) {
                all_boundary_nodes.push_back(r);
                break;
            }
    all_bou_node = (int)all_boundary_nodes.size();
    NUMNP = n_rows - 1;
    metric_term();
    for (int r = 0; r < n_rows; ++r) {
        det_out[r] = det[r];
        std::memcpy(metric_out + 63 * (size_t)r, &metric[r], 9 * sizeof(double));
    }
}

// The half-point block of Main.cpp on rows 1..n_owned (metric and det as
// given; face blocks of metric and deter written).
extern "C" void ref_half_point_metrics(const ref_grid_row *grid, int n_rows, int n_owned, const double *det_in,
                                       double *metric_io, double *deter_out)
{
    load_nodes(grid, n_rows);
    metric.assign(n_rows, TRANSFORMED{});
    deter.assign(n_rows, DETERM{});
    det.assign(det_in, det_in + n_rows);
    std::memcpy(metric.data(), metric_io, sizeof(TRANSFORMED) * (size_t)n_rows);
    sd_node = n_owned;
    ref_half_points_body();
    std::memcpy(metric_io, metric.data(), sizeof(TRANSFORMED) * (size_t)n_rows);
    std::memcpy(deter_out, deter.data(), sizeof(DETERM) * (size_t)n_rows);
}

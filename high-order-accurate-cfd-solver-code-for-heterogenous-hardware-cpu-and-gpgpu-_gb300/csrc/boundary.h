// boundary.h -- the reference's boundary routine intialise()
// (Flow_Initialisation.cpp:23-1394) as device work: plan entries resolved
// on the host, applied by one thread per entry (or in list order when the
// entries of a list touch each other's rows).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "cfd_rhs.h"
#include "lattice.cuh"

namespace cfd {

// The four lists in the order the routine visits them, then the trailing-
// edge tip rows the solver fixes after the routine (Solver.cpp:660-683).
enum { BC_OUTLET = 0, BC_INLET = 1, BC_BOUNDARY = 2, BC_WALL = 3, BC_TIP = 4, BC_NTYPES = 5 };
// Entry classes (low byte of BcEntry::cls).  BC_CONT marks an entry that
// continues the group of the entry before it: the singular-node branches of
// one wall node (its face or edge rule, then node rules and mirror passes
// from the singular table) are a group that one thread applies in order.
enum { BC_FACE = 0, BC_EDGE = 1, BC_MIRROR = 2, BC_CONT = 0x100 };

// One list entry with its node chains resolved: the boundary node b; for a
// face code (1..6) the three inward nodes s[0..2] along the interior slot
// and the three ghosts g[0..2] along the missing slot; for a node rule
// (edge or corner codes 7..26, the singular branches' node rules, tips) the
// source s[0]; for a singular mirror pass the three ghosts g[0..2] along the
// ghost slot of b and the three nodes s[0..2] along the singular slot from
// the singular neighbour.  Indices are reference rows, or lattice nodes
// after remapping.
struct BcEntry {
    int32_t b, cls;
    int32_t s[3];
    int32_t g[3];
};

__host__ __device__ __forceinline__ int bc_class(const BcEntry &e) { return e.cls & 0xff; }
__host__ __device__ __forceinline__ bool bc_cont(const BcEntry &e) { return (e.cls & BC_CONT) != 0; }
// Lists whose node rules are the wall's (zero velocity).
__host__ __device__ __forceinline__ bool bc_no_slip(int type) { return type == BC_WALL || type == BC_TIP; }

// Host plan of the lists (reference rows).  independent: no list touches a
// row that another list writes, and no list needs its own order, so all
// entries may run in one launch in any order.
struct BcPlan {
    std::vector<BcEntry> list[BC_NTYPES];
    bool sequential[BC_NTYPES] = {};
    bool independent = false;
};

// Offsets of the lists in the concatenated entry array of one launch:
// list t holds entries [o[t], o[t + 1]).
struct BcOffsets {
    int o[BC_NTYPES + 1];
};

// List of entry q of the concatenated array.
__host__ __device__ __forceinline__ int bc_type_of(const BcOffsets &off, int q)
{
    return (q >= off.o[1]) + (q >= off.o[2]) + (q >= off.o[3]) + (q >= off.o[4]);
}

// f(entry, m) for target m (0 <= m < NM) of entry q of a list ending at
// end; when entry q heads a group, the m == 0 thread applies every target
// of every entry of the group in order and the others return; a
// continuation entry returns (its head applies it).  A group never crosses
// a list: the first entry of a list is never a continuation.
template <int NM, class F>
__device__ __forceinline__ void bc_for_group(const BcEntry *E, int q, int end, int m, const F &f)
{
    if (bc_cont(E[q])) return;
    if (!(q + 1 < end && bc_cont(E[q + 1]))) {
        f(E[q], m);
        return;
    }
    if (m != 0) return;
    for (int r = q; r < end && (r == q || bc_cont(E[r])); ++r)
        for (int k = 0; k < NM; ++k) f(E[r], k);
}

// Resolves the lists against the neighbour table.  singular (rows x 6, may
// be null) is the reference's singular-node table; tips (n_tips rows) get
// the tip rule after the lists.  Fails (with a message) on an index outside
// [0, n_rows), on wall nodes that need the singular table when none is
// given (ID 10, codes 29/30, 33..52), and on wall codes 53..56 (the routine
// leaves their mirror slots unset); entries with codes the routine has no
// branch for are dropped.
bool bc_make_plan(const cfd_grid_t *grid, int32_t n_rows, const int32_t *const rows[BC_NTYPES],
                  const int32_t n[BC_NTYPES], const int32_t *singular, BcPlan &plan, std::string &err);

// The same plan with every index mapped through n_of (reference row ->
// lattice node); false if an index has no node.
bool bc_remap(const BcPlan &in, const std::vector<int32_t> &n_of, BcPlan &out);

// Device copy of a plan: the lists back to back in one array (list t at
// d[t] = all + off.o[t]); a plan with independent lists runs as one launch.
struct BcDevice {
    BcEntry *all = nullptr;
    BcEntry *d[BC_NTYPES] = {};
    int n[BC_NTYPES] = {};
    int seq[BC_NTYPES] = {};
    BcOffsets off{};
    bool fused = false;
    int total() const { return off.o[BC_NTYPES]; }
    int launches() const
    {
        if (fused) return total() > 0 ? 1 : 0;
        int k = 0;
        for (int t = 0; t < BC_NTYPES; ++t) k += n[t] > 0;
        return k;
    }
};
cudaError_t bc_upload(const BcPlan &plan, BcDevice &dev, cudaStream_t st);
void bc_free(BcDevice &dev);

// The routine on FLOW in the reference layout (rows of 9 doubles) or on the
// lattice's SoA FLOW fields [9][N] (boundary.cu, reference evaluation order).
void bc_apply_aos(cudaStream_t st, const BcDevice &bc, double *flow_rows, double mach);
void bc_apply_soa(cudaStream_t st, const BcDevice &bc, double *prim9, int N, double mach);
// Free stream on rows 1..sd_node (the routine's initial == 0 branch).
void bc_free_stream_aos(cudaStream_t st, double *flow_rows, int sd_node, double mach);
// The mixed form: targets from the hi/lo state of U slot q (mixed.cu).
void bc_apply_mixed(cudaStream_t st, const BcDevice &bc, const LatView &g, int q, double mach);
// The split form: targets from the FP64 state of U slot q (split.cu).
void bc_apply_split(cudaStream_t st, const BcDevice &bc, const LatView &g, int q, double mach);

// Target m of one entry of the routine on a lattice state held in a
// precision form's own representation: m = 0 the boundary node, m = 1..3
// its ghosts (face codes; node rules have only m = 0, mirror passes only
// m = 1..3).  The same rules on (rho, u, v, w, p), the fields the next stage
// reads (U_Q.cl takes rho, u, v, w, p of FLOW): outlet copies the first
// inward node into the node and its ghosts, inlet writes the free stream
// (Flow_Initialisation.cpp:35-48), boundary mirrors inward node m into
// ghost m, wall sets zero velocity at the node and mirrors with the velocity
// negated; node rules copy their source (zero velocity on walls and tips);
// a singular mirror pass writes ghost m from singular-chain node m with the
// velocity negated.  Outside a group each target depends only on nodes the
// entry does not write.  St provides prims(n, rho, u, v, w, p, t) and
// set(n, rho, u, v, w, p).
template <class St>
__device__ __forceinline__ void bc_target_rules(const St &S, int type, const BcEntry &e, int m, double mach)
{
    const double gm2 = 1.4 * mach * mach;
    double rho, u, v, w, p, t;
    const int cls = bc_class(e);
    if (cls == BC_EDGE) {
        if (m != 0) return;
        S.prims(e.s[0], rho, u, v, w, p, t);
        if (bc_no_slip(type)) u = v = w = 0.0;
        S.set(e.b, gm2 * (p / t), u, v, w, p);
        return;
    }
    if (cls == BC_MIRROR) {
        if (m == 0) return;
        const int node = e.g[m - 1];
        for (int k = m; k < 3; ++k)
            if (e.g[k] == node) return;
        S.prims(e.s[m - 1], rho, u, v, w, p, t);
        S.set(node, rho, -u, -v, -w, p);
        return;
    }
    const int node = m == 0 ? e.b : e.g[m - 1];
    // the routine writes the targets in order: when a collapsed chain names a
    // node twice, the later target's write stands
    for (int k = m; k < 3; ++k)
        if (e.g[k] == node) return;
    if (type == BC_INLET || type == BC_OUTLET) {   // node and ghosts alike
        if (type == BC_INLET) {
            u = 1.0;
            v = w = 0.0;
            p = 1.0 / gm2;
            t = 1.0;
        } else {
            S.prims(e.s[0], rho, u, v, w, p, t);
        }
        S.set(node, gm2 * (p / t), u, v, w, p);
        return;
    }
    // boundary (mirror copy) and wall (no slip): ghost m from inward node m,
    // the node itself from the first inward node
    S.prims(e.s[m == 0 ? 0 : m - 1], rho, u, v, w, p, t);
    if (m == 0 && type == BC_WALL)
        S.set(node, gm2 * (p / t), 0.0, 0.0, 0.0, p);
    else if (type == BC_WALL)
        S.set(node, rho, -u, -v, -w, p);
    else
        S.set(node, rho, u, v, w, p);
}

}  // namespace cfd

// Library object behind cfd_bc_t.
struct cfd_bc {
    cfd_ctx_t *ctx = nullptr;
    int32_t n_rows = 0;
    cfd::BcPlan plan;
    cfd::BcDevice dev;
};

// boundary.cu -- the reference's boundary routine intialise()
// (Flow_Initialisation.cpp:23-1394) on the device.
//
// Per list (outlet, inlet, boundary, wall, in that order) and per entry:
//   face code 1..6 (loc names the missing neighbour, :55-89): the node and
//     its three ghost layers along the missing slot,
//       outlet   node <- first inward node (u,v,w,p,t), rho/e/a derived;
//                ghosts <- node                              (:92-137)
//       inlet    node <- free stream; ghosts <- node        (:385-419)
//       boundary node <- first inward node; ghost m <- inward node m
//                                                            (:667-704)
//       wall     node: u=v=w=0, p and t of the first inward node, rho/e/a
//                derived; ghost m <- inward node m with u,v,w negated
//                                                            (:953-990)
//   edge/corner code 7..26: the node <- a diagonal inward node (u,v,w,p,t;
//     u=v=w=0 on walls), rho and e derived (:139-340 and the same chains in
//     the other three lists).
//   wall nodes with the singular-node table (:1194-1392), after the rule of
//     their code, as one group applied in order by one thread:
//       code 29/30  node rule from the node beyond singular[b][3] along
//                   slot 4 / 5 (in place of a face or edge rule)
//       ID 10       node rule from singular[b][3], then three mirror passes
//                   (ghost slot, singular slot) = (2,0), (0,2), (1,3)
//       code 33..52 node rule from singular[b][0], then per pass (two or
//                   three by code) the node rule from singular[b][k] and a
//                   mirror pass (l, k)
//     a mirror pass: the three nodes along slot l from b <- the three nodes
//     along slot k from singular[b][k], velocity negated, a of b.
//   tips, after the lists (Solver.cpp:660-683): the wall node rule from the
//     tip's slot-3 neighbour.
// mu is never touched; `a` is not updated by node rules.
// Compiled with --fmad=false: the arithmetic (rho, e, a, free stream) is the
// reference's expression for expression, so results are bit-identical.
#include <algorithm>
#include <cmath>
#include <unordered_map>

#include "boundary.h"
#include "internal.h"

namespace cfd {

namespace {

constexpr int kFaceL[7] = {-1, 0, 1, 2, 3, 5, 4};   // missing (ghost) slot of face codes 1..6
constexpr int kFaceK[7] = {-1, 2, 3, 0, 1, 4, 5};   // inward slot
constexpr int kEdgeChain[20][3] = {
    {1, 5, 2}, {1, 4, 2}, {3, 4, 2}, {3, 5, 2}, {1, 5, 0}, {1, 4, 0}, {3, 4, 0}, {3, 5, 0},
    {5, 0, -1}, {1, 0, -1}, {4, 0, -1}, {3, 0, -1}, {5, 2, -1}, {1, 2, -1}, {4, 2, -1}, {3, 2, -1},
    {1, 5, -1}, {1, 4, -1}, {3, 4, -1}, {3, 5, -1}};

enum { F_U = 0, F_V = 1, F_W = 2, F_P = 3, F_T = 4, F_RHO = 5, F_MU = 6, F_A = 7, F_E = 8 };

struct AosFlow {
    double *f;
    __device__ double &at(int r, int c) const { return f[(size_t)r * 9 + c]; }
};

struct SoaFlow {
    double *f;
    int N;
    __device__ double &at(int n, int c) const { return f[(size_t)c * N + n]; }
};

template <class A>
__device__ __forceinline__ void rho_e(const A &F, int b, double mach)
{
    F.at(b, F_RHO) = (1.4 * mach * mach) * (F.at(b, F_P) / F.at(b, F_T));
    F.at(b, F_E) = F.at(b, F_P) / (0.4 * F.at(b, F_RHO));
}

template <class A>
__device__ __forceinline__ void copy8(const A &F, int dst, int src)
{
    F.at(dst, F_U) = F.at(src, F_U);
    F.at(dst, F_V) = F.at(src, F_V);
    F.at(dst, F_W) = F.at(src, F_W);
    F.at(dst, F_P) = F.at(src, F_P);
    F.at(dst, F_RHO) = F.at(src, F_RHO);
    F.at(dst, F_T) = F.at(src, F_T);
    F.at(dst, F_A) = F.at(src, F_A);
    F.at(dst, F_E) = F.at(src, F_E);
}

template <class A>
__device__ void apply_entry(const A &F, int type, const BcEntry &e, double mach)
{
    const int b = e.b;
    const int cls = bc_class(e);
    if (cls == BC_MIRROR) {
        for (int m = 0; m < 3; ++m) {
            const int gm = e.g[m], sm = e.s[m];
            F.at(gm, F_U) = (-1.0) * F.at(sm, F_U);
            F.at(gm, F_V) = (-1.0) * F.at(sm, F_V);
            F.at(gm, F_W) = (-1.0) * F.at(sm, F_W);
            F.at(gm, F_P) = F.at(sm, F_P);
            F.at(gm, F_RHO) = F.at(sm, F_RHO);
            F.at(gm, F_T) = F.at(sm, F_T);
            F.at(gm, F_A) = F.at(b, F_A);
            F.at(gm, F_E) = F.at(sm, F_E);
        }
        return;
    }
    if (cls == BC_EDGE) {
        const int s = e.s[0];
        if (bc_no_slip(type)) {
            F.at(b, F_U) = 0.0;
            F.at(b, F_V) = 0.0;
            F.at(b, F_W) = 0.0;
        } else {
            F.at(b, F_U) = F.at(s, F_U);
            F.at(b, F_V) = F.at(s, F_V);
            F.at(b, F_W) = F.at(s, F_W);
        }
        F.at(b, F_P) = F.at(s, F_P);
        F.at(b, F_T) = F.at(s, F_T);
        rho_e(F, b, mach);
        return;
    }
    const int s1 = e.s[0];
    if (type == BC_OUTLET || type == BC_INLET) {
        if (type == BC_OUTLET) {
            F.at(b, F_U) = F.at(s1, F_U);
            F.at(b, F_V) = F.at(s1, F_V);
            F.at(b, F_W) = F.at(s1, F_W);
            F.at(b, F_P) = F.at(s1, F_P);
            F.at(b, F_T) = F.at(s1, F_T);
        } else {
            F.at(b, F_U) = 1.0;
            F.at(b, F_V) = 0.0;
            F.at(b, F_W) = 0.0;
            F.at(b, F_P) = 1.0 / (1.4 * mach * mach);
            F.at(b, F_T) = 1.0;
        }
        rho_e(F, b, mach);
        F.at(b, F_A) = sqrt(1.4 * F.at(b, F_P) / F.at(b, F_RHO));
        for (int m = 0; m < 3; ++m) copy8(F, e.g[m], b);
    } else if (type == BC_BOUNDARY) {
        copy8(F, b, s1);
        for (int m = 0; m < 3; ++m) copy8(F, e.g[m], e.s[m]);
    } else {
        F.at(b, F_U) = 0.0;
        F.at(b, F_V) = 0.0;
        F.at(b, F_W) = 0.0;
        F.at(b, F_P) = F.at(s1, F_P);
        F.at(b, F_T) = F.at(s1, F_T);
        rho_e(F, b, mach);
        F.at(b, F_A) = sqrt(1.4 * F.at(b, F_P) / F.at(b, F_RHO));
        for (int m = 0; m < 3; ++m) {
            const int gm = e.g[m], sm = e.s[m];
            F.at(gm, F_U) = (-1.0) * F.at(sm, F_U);
            F.at(gm, F_V) = (-1.0) * F.at(sm, F_V);
            F.at(gm, F_W) = (-1.0) * F.at(sm, F_W);
            F.at(gm, F_P) = F.at(sm, F_P);
            F.at(gm, F_RHO) = F.at(sm, F_RHO);
            F.at(gm, F_T) = F.at(sm, F_T);
            F.at(gm, F_A) = F.at(sm, F_A);
            F.at(gm, F_E) = F.at(sm, F_E);
        }
    }
}

// one thread per entry (per group), or (sequential) one thread walking the
// list in order
template <class A>
__global__ void k_bc(A F, const BcEntry *__restrict__ E, int n, int type, double mach, int sequential)
{
    if (sequential) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            for (int q = 0; q < n; ++q) apply_entry(F, type, E[q], mach);
        return;
    }
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) bc_for_group<1>(E, q, n, 0, [&](const BcEntry &e, int) { apply_entry(F, type, e, mach); });
}

// every entry of independent lists in one launch, one thread per entry
template <class A>
__global__ void k_bc_fused(A F, const BcEntry *__restrict__ E, BcOffsets off, double mach)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= off.o[BC_NTYPES]) return;
    const int type = bc_type_of(off, q);
    bc_for_group<1>(E, q, off.o[BC_NTYPES], 0, [&](const BcEntry &e, int) { apply_entry(F, type, e, mach); });
}

__global__ void k_free_stream(AosFlow F, int sd_node, double mach)
{
    const int r = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (r > sd_node) return;
    F.at(r, F_U) = 1.0;
    F.at(r, F_V) = 0.0;
    F.at(r, F_W) = 0.0;
    F.at(r, F_P) = 1.0 / (1.4 * mach * mach);
    F.at(r, F_T) = 1.0;
    F.at(r, F_RHO) = (1.4 * mach * mach) * (F.at(r, F_P) / F.at(r, F_T));
    F.at(r, F_E) = F.at(r, F_P) / (0.4 * F.at(r, F_RHO));
    F.at(r, F_A) = sqrt(1.4 * F.at(r, F_P) / F.at(r, F_RHO));
}

template <class A>
void launch_lists(cudaStream_t st, const BcDevice &bc, const A &F, double mach)
{
    if (bc.fused) {
        if (bc.total() > 0) k_bc_fused<<<blocks_for(bc.total(), 128), 128, 0, st>>>(F, bc.all, bc.off, mach);
        return;
    }
    for (int t = 0; t < BC_NTYPES; ++t) {
        if (bc.n[t] == 0) continue;
        const unsigned blocks = bc.seq[t] ? 1u : blocks_for(bc.n[t], 128);
        k_bc<<<blocks, bc.seq[t] ? 1 : 128, 0, st>>>(F, bc.d[t], bc.n[t], t, mach, bc.seq[t]);
    }
}

int nb(const cfd_grid_t &g, int slot)
{
    switch (slot) {
    case 0: return g.N0;
    case 1: return g.N1;
    case 2: return g.N2;
    case 3: return g.N3;
    case 4: return g.N4;
    default: return g.N5;
    }
}

// Rows an entry writes and reads (for the order checks).
void entry_rows(int type, const BcEntry &e, std::vector<int32_t> &w, std::vector<int32_t> &r)
{
    w.clear();
    r.clear();
    if (bc_class(e) == BC_MIRROR) {
        for (int m = 0; m < 3; ++m) {
            w.push_back(e.g[m]);
            r.push_back(e.s[m]);
        }
        r.push_back(e.b);
        return;
    }
    w.push_back(e.b);
    if (bc_class(e) == BC_EDGE) {
        r.push_back(e.s[0]);
        return;
    }
    if (type != BC_INLET) r.push_back(e.s[0]);
    if (type == BC_BOUNDARY || type == BC_WALL) {
        r.push_back(e.s[1]);
        r.push_back(e.s[2]);
    }
    for (int m = 0; m < 3; ++m) w.push_back(e.g[m]);
}

// True when some group's reads or writes meet another group's writes: the
// list must then run in its order.  (A group -- an entry and the
// continuation entries after it -- runs in order on one thread, so the rows
// its own entries share do not count.)
bool needs_order(int type, const std::vector<BcEntry> &list)
{
    std::unordered_map<int32_t, int> writer;   // row -> group (index of its head)
    std::vector<int32_t> w, r;
    int head = 0;
    for (size_t q = 0; q < list.size(); ++q) {
        if (!bc_cont(list[q])) head = (int)q;
        entry_rows(type, list[q], w, r);
        for (int32_t x : w) {
            auto it = writer.find(x);
            if (it != writer.end() && it->second != head) return true;
            writer[x] = head;
        }
    }
    head = 0;
    for (size_t q = 0; q < list.size(); ++q) {
        if (!bc_cont(list[q])) head = (int)q;
        entry_rows(type, list[q], w, r);
        for (int32_t x : r) {
            auto it = writer.find(x);
            if (it != writer.end() && it->second != head) return true;
        }
    }
    return false;
}

// True when no row written by one list is read or written by another.
bool lists_independent(const BcPlan &plan)
{
    std::unordered_map<int32_t, int> writer;   // row -> list
    std::vector<int32_t> w, r;
    for (int t = 0; t < BC_NTYPES; ++t)
        for (const BcEntry &e : plan.list[t]) {
            entry_rows(t, e, w, r);
            for (int32_t x : w) {
                auto it = writer.find(x);
                if (it != writer.end() && it->second != t) return false;
                writer[x] = t;
            }
        }
    for (int t = 0; t < BC_NTYPES; ++t)
        for (const BcEntry &e : plan.list[t]) {
            entry_rows(t, e, w, r);
            for (int32_t x : r) {
                auto it = writer.find(x);
                if (it != writer.end() && it->second != t) return false;
            }
        }
    return true;
}

}  // namespace

namespace {

// The mirror passes (ghost slot l, singular slot k) of the singular wall
// codes 33..52 (Flow_Initialisation.cpp:1285-1342): two for 33..36, 41..44
// and 49..52, three for 37..40 and 45..48.  Returns the count.
int multi_pass(int loc, int lk[3][2])
{
    auto set = [&](int h, int l, int k) {
        lk[h][0] = l;
        lk[h][1] = k;
    };
    if (loc >= 33 && loc <= 40) set(0, 2, 0);
    else if (loc >= 41 && loc <= 48) set(0, 0, 2);
    else if (loc == 49 || loc == 52) set(0, 5, 4);
    else set(0, 4, 5);   // 50, 51
    switch (loc) {
    case 33: case 43: case 51: case 52: case 39: case 40: case 47: case 48: set(1, 3, 1); break;
    case 35: case 41: case 49: case 50: case 37: case 38: case 45: case 46: set(1, 1, 3); break;
    case 34: case 44: set(1, 5, 4); break;
    default: set(1, 4, 5); break;   // 36, 42
    }
    if ((loc >= 37 && loc <= 40) || (loc >= 45 && loc <= 48)) {
        if (loc == 37 || loc == 40 || loc == 48 || loc == 45) set(2, 5, 4);
        else set(2, 4, 5);
        return 3;
    }
    return 2;
}

}  // namespace

bool bc_make_plan(const cfd_grid_t *grid, int32_t n_rows, const int32_t *const rows[BC_NTYPES],
                  const int32_t n[BC_NTYPES], const int32_t *singular, BcPlan &plan, std::string &err)
{
    auto in_range = [&](int r) { return r >= 0 && r < n_rows; };
    // slot s of row r in the singular table, or -1
    auto sing = [&](int r, int s) { return singular[(size_t)r * 6 + s]; };
    for (int t = 0; t < BC_NTYPES; ++t) {
        plan.list[t].clear();
        for (int32_t q = 0; q < n[t]; ++q) {
            const int b = rows[t][q];
            if (!in_range(b)) {
                err = "boundary list row outside [0, n_rows)";
                return false;
            }
            const cfd_grid_t &gb = grid[b];
            const int loc = gb.loc;
            if (t == BC_TIP) {   // Solver.cpp:660-683
                BcEntry e{};
                e.b = b;
                e.cls = BC_EDGE;
                e.s[0] = e.s[1] = e.s[2] = gb.N3;
                e.g[0] = e.g[1] = e.g[2] = b;
                if (!in_range(gb.N3)) {
                    err = "tip neighbour outside the table";
                    return false;
                }
                plan.list[t].push_back(e);
                continue;
            }
            const bool singular_node =
                t == BC_WALL && (loc == 29 || loc == 30 || (loc >= 33 && loc <= 56) || gb.ID == 10);
            if (singular_node && loc >= 53 && loc <= 56) {
                err = "wall codes 53-56: the reference leaves their singular mirror slots unset";
                return false;
            }
            if (singular_node && !singular) {
                err = "wall node needs the reference's singular-node table (ID 10 or loc 29/30/33-52)";
                return false;
            }
            const size_t first = plan.list[t].size();
            BcEntry e{};
            e.b = b;
            if (loc >= 1 && loc <= 6) {
                e.cls = BC_FACE;
                int r = b;
                for (int m = 0; m < 3; ++m) {
                    r = nb(grid[r], kFaceL[loc]);
                    if (!in_range(r)) {
                        err = "ghost chain leaves the table";
                        return false;
                    }
                    e.g[m] = r;
                }
                r = b;
                for (int m = 0; m < 3; ++m) {
                    r = nb(grid[r], kFaceK[loc]);
                    if (!in_range(r)) {
                        err = "inward chain leaves the table";
                        return false;
                    }
                    e.s[m] = r;
                }
            } else if (loc >= 7 && loc <= 26) {
                e.cls = BC_EDGE;
                int r = b;
                for (int m = 0; m < 3 && kEdgeChain[loc - 7][m] >= 0; ++m) {
                    r = nb(grid[r], kEdgeChain[loc - 7][m]);
                    if (!in_range(r)) {
                        err = "diagonal chain leaves the table";
                        return false;
                    }
                }
                e.s[0] = r;
                e.s[1] = e.s[2] = r;
                e.g[0] = e.g[1] = e.g[2] = b;
            }
            if ((loc >= 1 && loc <= 26)) plan.list[t].push_back(e);
            // other codes: the routine has no branch for them (besides the
            // singular branches below)
            if (singular_node) {
                bool ok = true;
                auto node_rule = [&](int src) {
                    BcEntry x{};
                    x.b = b;
                    x.cls = BC_EDGE;
                    ok = ok && in_range(src);
                    x.s[0] = x.s[1] = x.s[2] = src;
                    x.g[0] = x.g[1] = x.g[2] = b;
                    plan.list[t].push_back(x);
                };
                auto mirror = [&](int l, int k) {
                    BcEntry x{};
                    x.b = b;
                    x.cls = BC_MIRROR;
                    int gr = b, sr = sing(b, k);
                    for (int m = 0; m < 3 && ok; ++m) {
                        gr = nb(grid[gr], l);
                        if (m > 0) sr = nb(grid[sr], k);
                        ok = in_range(gr) && in_range(sr);
                        x.g[m] = gr;
                        x.s[m] = sr;
                    }
                    plan.list[t].push_back(x);
                };
                auto sing_ok = [&](int s) {
                    ok = ok && in_range(sing(b, s));
                    return ok;
                };
                if (loc == 29 || loc == 30) {   // :1194-1213
                    if (sing_ok(3)) node_rule(nb(grid[sing(b, 3)], loc == 29 ? 4 : 5));
                }
                if (gb.ID == 10 && loc != 29 && loc != 30 && sing_ok(3)) {   // :1215-1272
                    static const int lk10[3][2] = {{2, 0}, {0, 2}, {1, 3}};
                    node_rule(sing(b, 3));
                    for (int h = 0; h < 3 && ok; ++h)
                        if (sing_ok(lk10[h][1])) mirror(lk10[h][0], lk10[h][1]);
                }
                if (loc >= 33 && loc <= 52 && sing_ok(0)) {   // :1276-1390
                    int lk[3][2];
                    const int np = multi_pass(loc, lk);
                    node_rule(sing(b, 0));
                    for (int h = 0; h < np && ok; ++h)
                        if (sing_ok(lk[h][1])) {
                            node_rule(sing(b, lk[h][1]));
                            mirror(lk[h][0], lk[h][1]);
                        }
                }
                if (!ok) {
                    err = "singular-node chain leaves the table";
                    return false;
                }
                for (size_t x = first + 1; x < plan.list[t].size(); ++x) plan.list[t][x].cls |= BC_CONT;
            }
        }
        plan.sequential[t] = needs_order(t, plan.list[t]);
    }
    plan.independent = lists_independent(plan);
    for (int t = 0; t < BC_NTYPES; ++t) plan.independent = plan.independent && !plan.sequential[t];
    return true;
}

bool bc_remap(const BcPlan &in, const std::vector<int32_t> &n_of, BcPlan &out)
{
    auto map = [&](int32_t r, int32_t &o) {
        if (r < 0 || r >= (int32_t)n_of.size() || n_of[r] < 0) return false;
        o = n_of[r];
        return true;
    };
    out.independent = in.independent;   // the map is one to one
    for (int t = 0; t < BC_NTYPES; ++t) {
        out.list[t] = in.list[t];
        out.sequential[t] = in.sequential[t];
        for (BcEntry &e : out.list[t]) {
            if (!map(e.b, e.b)) return false;
            for (int m = 0; m < 3; ++m)
                if (!map(e.s[m], e.s[m]) || !map(e.g[m], e.g[m])) return false;
        }
    }
    return true;
}

cudaError_t bc_upload(const BcPlan &plan, BcDevice &dev, cudaStream_t st)
{
    bc_free(dev);
    std::vector<BcEntry> all;
    for (int t = 0; t < BC_NTYPES; ++t) {
        dev.n[t] = (int)plan.list[t].size();
        dev.seq[t] = plan.sequential[t] ? 1 : 0;
        dev.off.o[t] = (int)all.size();
        all.insert(all.end(), plan.list[t].begin(), plan.list[t].end());
    }
    dev.off.o[BC_NTYPES] = (int)all.size();
    dev.fused = plan.independent;
    if (all.empty()) return cudaSuccess;
    cudaError_t e = cudaMalloc(&dev.all, all.size() * sizeof(BcEntry));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dev.all, all.data(), all.size() * sizeof(BcEntry), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    for (int t = 0; t < BC_NTYPES; ++t) dev.d[t] = dev.n[t] ? dev.all + dev.off.o[t] : nullptr;
    return cudaStreamSynchronize(st);
}

void bc_free(BcDevice &dev)
{
    if (dev.all) cudaFree(dev.all);
    dev = BcDevice();
}

void bc_apply_aos(cudaStream_t st, const BcDevice &bc, double *flow_rows, double mach)
{
    launch_lists(st, bc, AosFlow{flow_rows}, mach);
}

void bc_apply_soa(cudaStream_t st, const BcDevice &bc, double *prim9, int N, double mach)
{
    launch_lists(st, bc, SoaFlow{prim9, N}, mach);
}

void bc_free_stream_aos(cudaStream_t st, double *flow_rows, int sd_node, double mach)
{
    if (sd_node > 0) k_free_stream<<<blocks_for(sd_node, 256), 256, 0, st>>>(AosFlow{flow_rows}, sd_node, mach);
}

}  // namespace cfd

using namespace cfd;

extern "C" {

cfd_status_t cfd_bc_create_singular(cfd_ctx_t *ctx, const cfd_grid_t *grid, int32_t n_rows, const int32_t *outlet,
                                    int32_t n_outlet, const int32_t *inlet, int32_t n_inlet, const int32_t *boundary,
                                    int32_t n_boundary, const int32_t *wall, int32_t n_wall, const int32_t *singular,
                                    const int32_t *tips, int32_t n_tips, cfd_bc_t **out)
{
    if (!ctx || !grid || !out || n_rows < 1 || n_outlet < 0 || n_inlet < 0 || n_boundary < 0 || n_wall < 0
        || n_tips < 0)
        return CFD_EINVAL;
    *out = nullptr;
    const int32_t *rows[BC_NTYPES] = {outlet, inlet, boundary, wall, tips};
    const int32_t n[BC_NTYPES] = {n_outlet, n_inlet, n_boundary, n_wall, n_tips};
    for (int t = 0; t < BC_NTYPES; ++t)
        if (n[t] > 0 && !rows[t]) return fail(ctx, CFD_EINVAL, "cfd_bc_create: null list with a nonzero count");
    cfd_status_t st = use_device(ctx);
    if (st != CFD_OK) return st;
    cfd_bc *bc = new cfd_bc();
    bc->ctx = ctx;
    bc->n_rows = n_rows;
    std::string err;
    if (!bc_make_plan(grid, n_rows, rows, n, singular, bc->plan, err)) {
        const bool unsupported = err.find("singular") != std::string::npos || err.find("53-56") != std::string::npos;
        delete bc;
        return fail(ctx, unsupported ? CFD_EUNSUPPORTED : CFD_EINVAL, "cfd_bc_create: " + err);
    }
    cudaError_t e = bc_upload(bc->plan, bc->dev, ctx->stream);
    if (e != cudaSuccess) {
        bc_free(bc->dev);
        delete bc;
        return cuda_fail(ctx, e, "cfd_bc_create upload");
    }
    *out = bc;
    return CFD_OK;
}

cfd_status_t cfd_bc_create(cfd_ctx_t *ctx, const cfd_grid_t *grid, int32_t n_rows, const int32_t *outlet,
                           int32_t n_outlet, const int32_t *inlet, int32_t n_inlet, const int32_t *boundary,
                           int32_t n_boundary, const int32_t *wall, int32_t n_wall, cfd_bc_t **out)
{
    return cfd_bc_create_singular(ctx, grid, n_rows, outlet, n_outlet, inlet, n_inlet, boundary, n_boundary, wall,
                                  n_wall, nullptr, nullptr, 0, out);
}

cfd_status_t cfd_bc_destroy(cfd_bc_t *bc)
{
    if (!bc) return CFD_EINVAL;
    use_device(bc->ctx);
    cudaStreamSynchronize(bc->ctx->stream);
    bc_free(bc->dev);
    delete bc;
    return CFD_OK;
}

cfd_status_t cfd_boundary_fill(cfd_ctx_t *ctx, const cfd_bc_t *bc, cfd_flow_t *FLOW, double Mach, int32_t initial,
                               int32_t sd_node)
{
    if (!ctx || !bc || !FLOW || !std::isfinite(Mach) || sd_node < 0 || sd_node >= bc->n_rows) return CFD_EINVAL;
    cfd_status_t st = use_device(ctx);
    if (st != CFD_OK) return st;
    BufArg a[] = {{FLOW, 72, true, bc->n_rows}};   // a device buffer, or the table's host FLOW rows
    if ((st = stage_in(ctx, a, 1, "cfd_boundary_fill")) != CFD_OK) return st;
    double *f = reinterpret_cast<double *>(a[0].dev);
    if (initial == 0) {
        bc_free_stream_aos(ctx->stream, f, sd_node, Mach);
        ctx->launches += sd_node > 0;
    }
    bc_apply_aos(ctx->stream, bc->dev, f, Mach);
    ctx->launches += bc->dev.launches() - 1;   // after_launch counts one
    return stage_out(ctx, a, 1, after_launch(ctx, "cfd_boundary_fill"));
}

}  // extern "C"

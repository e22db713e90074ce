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
// mu is never touched; `a` is not updated for edge and corner codes.
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
    if (e.cls == BC_EDGE) {
        const int s = e.s[0];
        if (type == BC_WALL) {
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

// one thread per entry, or (sequential) one thread walking the list in order
template <class A>
__global__ void k_bc(A F, const BcEntry *__restrict__ E, int n, int type, double mach, int sequential)
{
    if (sequential) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            for (int q = 0; q < n; ++q) apply_entry(F, type, E[q], mach);
        return;
    }
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) apply_entry(F, type, E[q], mach);
}

// every entry of independent lists in one launch, one thread per entry
template <class A>
__global__ void k_bc_fused(A F, const BcEntry *__restrict__ E, BcOffsets off, double mach)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < off.o[BC_NTYPES]) apply_entry(F, bc_type_of(off, q), E[q], mach);
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

// Rows an entry writes and reads (for the order check within a list).
void entry_rows(int type, const BcEntry &e, std::vector<int32_t> &w, std::vector<int32_t> &r)
{
    w.assign(1, e.b);
    r.clear();
    if (e.cls == BC_EDGE) {
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

// True when some entry's reads or writes meet another entry's writes: the
// list must then run in its order.
bool needs_order(int type, const std::vector<BcEntry> &list)
{
    std::unordered_map<int32_t, int> writer;   // row -> entry index (first)
    std::vector<int32_t> w, r;
    for (size_t q = 0; q < list.size(); ++q) {
        entry_rows(type, list[q], w, r);
        for (int32_t x : w) {
            auto it = writer.find(x);
            if (it != writer.end() && it->second != (int)q) return true;
            writer[x] = (int)q;
        }
    }
    for (size_t q = 0; q < list.size(); ++q) {
        entry_rows(type, list[q], w, r);
        for (int32_t x : r) {
            auto it = writer.find(x);
            if (it != writer.end() && it->second != (int)q) return true;
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

bool bc_make_plan(const cfd_grid_t *grid, int32_t n_rows, const int32_t *const rows[BC_NTYPES],
                  const int32_t n[BC_NTYPES], BcPlan &plan, std::string &err)
{
    auto in_range = [&](int r) { return r >= 0 && r < n_rows; };
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
            if (t == BC_WALL && (loc == 29 || loc == 30 || (loc >= 33 && loc <= 56) || gb.ID == 10)) {
                err = "wall node needs the reference's singular-node table (ID 10 or loc 29/30/33-56)";
                return false;
            }
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
            } else {
                continue;   // the routine has no branch for this code
            }
            plan.list[t].push_back(e);
        }
        plan.sequential[t] = needs_order(t, plan.list[t]);
    }
    plan.independent = !plan.sequential[0] && !plan.sequential[1] && !plan.sequential[2] && !plan.sequential[3]
                       && lists_independent(plan);
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

cfd_status_t cfd_bc_create(cfd_ctx_t *ctx, const cfd_grid_t *grid, int32_t n_rows, const int32_t *outlet,
                           int32_t n_outlet, const int32_t *inlet, int32_t n_inlet, const int32_t *boundary,
                           int32_t n_boundary, const int32_t *wall, int32_t n_wall, cfd_bc_t **out)
{
    if (!ctx || !grid || !out || n_rows < 1 || n_outlet < 0 || n_inlet < 0 || n_boundary < 0 || n_wall < 0)
        return CFD_EINVAL;
    *out = nullptr;
    const int32_t *rows[BC_NTYPES] = {outlet, inlet, boundary, wall};
    const int32_t n[BC_NTYPES] = {n_outlet, n_inlet, n_boundary, n_wall};
    for (int t = 0; t < BC_NTYPES; ++t)
        if (n[t] > 0 && !rows[t]) return fail(ctx, CFD_EINVAL, "cfd_bc_create: null list with a nonzero count");
    cfd_status_t st = use_device(ctx);
    if (st != CFD_OK) return st;
    cfd_bc *bc = new cfd_bc();
    bc->ctx = ctx;
    bc->n_rows = n_rows;
    std::string err;
    if (!bc_make_plan(grid, n_rows, rows, n, bc->plan, err)) {
        const bool singular = err.find("singular") != std::string::npos;
        delete bc;
        return fail(ctx, singular ? CFD_EUNSUPPORTED : CFD_EINVAL, "cfd_bc_create: " + err);
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

// split.cu -- the split-precision form of the structured (lattice) stage:
// the conserved state, the RK3 accumulation and the metric/Jacobian products
// of the face flux in FP64; the characteristic projection, WENO5, the LLF
// speed and dissipation and the viscous fluxes in FP32 (lattice_split.cuh
// says which operation runs in which precision).
//
// Kernels per stage, as in the mixed form (mixed.cu): k_visc_s (radius-2
// star on the hi/lo read copy of the state, FP32, on a side stream),
// k_face_tile_s<d> x3 (one thread per face, the FP32
// stencil lines staged in shared memory, the FP64 face flux written to Fh),
// k_update_s (FP64 flux difference and RK stage + the next stage's U_Q);
// k_init_s / k_prep_s supply U_Q when no update produced it.  Compiled with
// FMA contraction and approximate FP32 division/square root.
#include "boundary.h"
#include "face_tile.cuh"
#include "internal.h"
#include "lattice_split.cuh"
#include "structured.h"

namespace cfd {

namespace {

__device__ __forceinline__ int node_id() { return blockIdx.x * blockDim.x + threadIdx.x; }

__global__ void __launch_bounds__(256) k_init_s(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) sp::init_node(g, n, q);
}

__global__ void __launch_bounds__(256) k_prep_s(LatView g, int src, int dst)
{
    const int n = node_id();
    if (n < g.N) sp::prep_node(g, n, src, dst);
}

// The viscous pass is the mixed form's (FP32, the same launch bounds) on
// the hi/lo read copy of the state (sp::hilo_view).
#ifndef CFD_SVISC_MIN_BLOCKS
#define CFD_SVISC_MIN_BLOCKS 6
#endif
#ifndef CFD_SVISC_LOC_MIN_BLOCKS
#define CFD_SVISC_LOC_MIN_BLOCKS 4
#endif

template <bool LOC>
__global__ void __launch_bounds__(256, LOC ? CFD_SVISC_LOC_MIN_BLOCKS : CFD_SVISC_MIN_BLOCKS) k_visc_s(LatView g)
{
    const int n = node_id();
    if (n < g.N) mx::visc_node<LOC>(g, n, 0);
}

__global__ void __launch_bounds__(256) k_mu_s(LatView g)
{
    const int n = node_id();
    if (n < g.N) mx::mu_node(g, n, 0);
}

#ifndef CFD_SFACE_MIN_BLOCKS
#define CFD_SFACE_MIN_BLOCKS 6
#endif
// One instance per candidate tile width (face_tile.cuh): faces along i of
// 32, 64 or 128, along j or k of 8, 16 or 32; the solver times them when it
// is created and keeps the fastest per direction (the same arithmetic,
// only the staging differs).
template <int D, int TILE>
__global__ void __launch_bounds__(kFaceThreads, CFD_SFACE_MIN_BLOCKS) k_face_tile_s(LatView g)
{
    using T = FaceTile<D, TILE>;
    __shared__ float smem[tile_smem_floats<T>()];
    sp::face_tile<T, D>(g, tile_of_block<T>(), smem);
}

template <int D, int TILE>
void launch_tile_s(const LatView &g, cudaStream_t st)
{
    k_face_tile_s<D, TILE><<<FaceTile<D, TILE>::grid(g), kFaceThreads, 0, st>>>(g);
}

template <int D>
void launch_face_tile_s(const LatView &g, cudaStream_t st, int tile)
{
    if constexpr (D == 0) {
        if (tile == 32) launch_tile_s<0, 32>(g, st);
        else if (tile == 128) launch_tile_s<0, 128>(g, st);
        else launch_tile_s<0, 64>(g, st);
    } else {
        if (tile == 8) launch_tile_s<D, 8>(g, st);
        else if (tile == 32) launch_tile_s<D, 32>(g, st);
        else launch_tile_s<D, 16>(g, st);
    }
}

template <bool LOC>
__global__ void __launch_bounds__(256) k_update_s(LatView g, int jst)
{
    const int n = node_id();
    if (n < g.N) sp::update_node<LOC>(g, n, jst);
}

__global__ void k_bc_s(LatView g, const BcEntry *__restrict__ E, int n, int type, int q, double mach, int sequential)
{
    if (sequential) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            for (int e = 0; e < n; ++e)
                for (int m = 0; m < 4; ++m) sp::bc_target(g, type, E[e], m, q, mach);
        return;
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 4 * n)
        bc_for_group<4>(E, t >> 2, n, t & 3,
                        [&](const BcEntry &e, int m) { sp::bc_target(g, type, e, m, q, mach); });
}

__global__ void k_bc_s_fused(LatView g, const BcEntry *__restrict__ E, BcOffsets off, int q, double mach)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * off.o[BC_NTYPES]) return;
    const int type = bc_type_of(off, t >> 2);
    bc_for_group<4>(E, t >> 2, off.o[BC_NTYPES], t & 3,
                    [&](const BcEntry &e, int m) { sp::bc_target(g, type, e, m, q, mach); });
}

__global__ void k_flow_out_s(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) sp::flow_out_node(g, n, q);
}

__global__ void k_to_float_s(const double *__restrict__ a, float *__restrict__ b, long long n)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = (float)a[t];
}

// node32 = [9 node metrics, det, det^(-1/3)] in FP32; idet64 = 1/det
__global__ void k_node_geometry_s(const double *__restrict__ m9, const double *__restrict__ det, long long N,
                                  float *__restrict__ node32, double *__restrict__ idet64)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
#pragma unroll
    for (int c = 0; c < 9; ++c) node32[c * N + n] = (float)m9[c * N + n];
    node32[9 * N + n] = (float)det[n];
    node32[10 * N + n] = (float)(1.0 / cbrt(det[n]));
    idet64[n] = 1.0 / det[n];
}

}  // namespace

void split_geometry(const StructuredLaunch &S)
{
    const long long N = (long long)S.ni * S.nj * S.nk;
    k_to_float_s<<<blocks_for(9 * N, 256), 256, 0, S.stream>>>(S.fm, S.fm32, 9 * N);
    k_node_geometry_s<<<blocks_for(N, 256), 256, 0, S.stream>>>(S.m9, S.det, N, S.node32, S.idet64);
}

void bc_apply_split(cudaStream_t st, const BcDevice &bc, const LatView &g, int q, double mach)
{
    if (bc.fused) {
        if (bc.total() > 0) k_bc_s_fused<<<blocks_for(4LL * bc.total(), 128), 128, 0, st>>>(g, bc.all, bc.off, q, mach);
        return;
    }
    for (int t = 0; t < BC_NTYPES; ++t) {
        if (bc.n[t] == 0) continue;
        const unsigned blocks = bc.seq[t] ? 1u : blocks_for(4LL * bc.n[t], 128);
        k_bc_s<<<blocks, bc.seq[t] ? 1 : 128, 0, st>>>(g, bc.d[t], bc.n[t], t, q, mach, bc.seq[t]);
    }
}

void split_flow_out(const LatView &g, int q, cudaStream_t st)
{
    k_flow_out_s<<<blocks_for(g.N, 256), 256, 0, st>>>(g, q);
}

void split_prep(const LatView &g, int src, int dst, cudaStream_t st)
{
    if (src == kPrepFromFlow)
        k_init_s<<<blocks_for(g.N, 256), 256, 0, st>>>(g, dst);
    else
        k_prep_s<<<blocks_for(g.N, 256), 256, 0, st>>>(g, src, dst);
}

int split_stage(const StructuredLaunch &S, int jst, double dt, double *Lout, cudaEvent_t *ev, int prep_from,
                const char **names)
{
    const LatView g = make_view(S, dt, Lout);
    const unsigned nb256 = blocks_for(g.N, 256);
    cudaStream_t st = S.stream;
    int e = 0, k = 0;
    auto mark = [&]() {
        if (ev) cudaEventRecord(ev[e++], st);
    };
    auto name = [&](const char *nm) {
        if (names) names[k] = nm;
        ++k;
    };
    mark();
    if (prep_from != kPrepNone) {
        split_prep(g, prep_from, jst, st);
        name("prep");
        mark();
    }
    const bool loc = g.loc8 != nullptr;
    const bool side = S.side && !ev;   // viscous pass beside the face passes (not when timing each launch)
    cudaStream_t sv = side ? S.side : st;
    if (side) {
        cudaEventRecord(S.fork, st);
        cudaStreamWaitEvent(sv, S.fork, 0);
    }
    const LatView gh = sp::hilo_view(g);
    if (S.P.viscous) {
        if (loc)
            k_visc_s<true><<<nb256, 256, 0, sv>>>(gh);
        else
            k_visc_s<false><<<nb256, 256, 0, sv>>>(gh);
        name("viscous");
    } else {
        k_mu_s<<<nb256, 256, 0, sv>>>(gh);
        name("mu_only");
    }
    if (side) cudaEventRecord(S.join, sv);
    mark();
    const bool fside = side && S.face_side[0] && S.face_side[1];
    cudaStream_t sj = fside ? S.face_side[0] : st, sk = fside ? S.face_side[1] : st;
    if (fside) {
        cudaStreamWaitEvent(sj, S.fork, 0);
        cudaStreamWaitEvent(sk, S.fork, 0);
    }
    launch_face_tile_s<0>(g, st, S.tile_i);
    name("face_i");
    mark();
    launch_face_tile_s<1>(g, sj, S.tile_jk);
    name("face_j");
    mark();
    launch_face_tile_s<2>(g, sk, S.tile_jk);
    name("face_k");
    mark();
    if (fside) {
        cudaEventRecord(S.face_join[0], sj);
        cudaEventRecord(S.face_join[1], sk);
        cudaStreamWaitEvent(st, S.face_join[0], 0);
        cudaStreamWaitEvent(st, S.face_join[1], 0);
    }
    if (side) cudaStreamWaitEvent(st, S.join, 0);
    if (loc)
        k_update_s<true><<<nb256, 256, 0, st>>>(g, jst);
    else
        k_update_s<false><<<nb256, 256, 0, st>>>(g, jst);
    name("update+prep");
    mark();
    return k;
}

void split_face_pass(const StructuredLaunch &S, int d, int tile, cudaStream_t st)
{
    const LatView g = make_view(S, 0.0, nullptr);
    if (d == 0) launch_face_tile_s<0>(g, st, tile);
    else if (d == 1) launch_face_tile_s<1>(g, st, tile);
    else launch_face_tile_s<2>(g, st, tile);
}

}  // namespace cfd

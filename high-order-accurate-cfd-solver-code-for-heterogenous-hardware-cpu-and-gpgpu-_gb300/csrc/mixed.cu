// mixed.cu -- the mixed-precision form of the structured (lattice) stage.
//
// FP32: the characteristic projection, WENO5 weights and reconstruction, the
// LLF split and face fluxes, the viscous and SGS fluxes, the node fluxes used
// by the sixth-order correction, the right-hand side sum.  The conserved
// state U0/U1/U2 is carried as hi + lo FP32 pairs and the RK3 stage is
// accumulated in that arithmetic, so no stage kernel issues FP64 work; FP64
// appears only where FLOW enters (after an upload) and where FLOW/U leave.
// Stage intermediates are FP32 (half the bytes of the FP64 form).
//
// Kernels per stage: k_visc_m (radius-2 star), k_face_tile_m<d> x3 (one
// thread per face, stencil lines staged in shared memory), k_update_m (RK
// stage + the next stage's U_Q); k_init_m /
// k_prep_m supply U_Q when no update produced it.  The per-node operations
// are in lattice_mixed.cuh.  This file is compiled with FMA contraction on
// and approximate FP32 division/square root (the mixed form's error budget
// is 1e-6 relative L2 against the FP64 form).
#include "boundary.h"
#include "face_tile.cuh"
#include "internal.h"
#include "lattice_mixed.cuh"
#include "structured.h"

namespace cfd {

namespace {

__device__ __forceinline__ int node_id() { return blockIdx.x * blockDim.x + threadIdx.x; }

__global__ void __launch_bounds__(256) k_init_m(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) mx::init_node(g, n, q);
}

__global__ void __launch_bounds__(256) k_prep_m(LatView g, int src, int dst)
{
    const int n = node_id();
    if (n < g.N) mx::prep_node(g, n, src, dst);
}

// Blocks of 256 per SM that the viscous pass's registers must allow: 6 on
// periodic lattices (40 registers: latency bound, more warps help; 4, 5, 6,
// 8 measured 0.122, 0.114, 0.112, 0.145 ms on TGV 128^3), 4 with loc codes
// (64 registers; the branch code spills below that: 0.140 ms against 0.148
// and 0.175 at 5 and 6 on the NACA0012 O-grid).
#ifndef CFD_MVISC_MIN_BLOCKS
#define CFD_MVISC_MIN_BLOCKS 6
#endif
#ifndef CFD_MVISC_LOC_MIN_BLOCKS
#define CFD_MVISC_LOC_MIN_BLOCKS 4
#endif

template <bool LOC>
__global__ void __launch_bounds__(256, LOC ? CFD_MVISC_LOC_MIN_BLOCKS : CFD_MVISC_MIN_BLOCKS) k_visc_m(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) mx::visc_node<LOC>(g, n, q);
}

__global__ void __launch_bounds__(256) k_mu_m(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) mx::mu_node(g, n, q);
}

#ifndef CFD_MFACE_MIN_BLOCKS
#define CFD_MFACE_MIN_BLOCKS 8
#endif

// Faces per tile along D (a block of 128 threads covers kTile x 128/kTile
// faces; face_tile.cuh), StructuredLaunch::tile_i / tile_jk.  TGV 128^3: i
// tiles of 16 / 32 / 64 / 128 took 0.097 / 0.093 / 0.091 / 0.090 ms, j/k
// tiles of 4 / 8 / 16 / 32 took 0.098 / 0.094 / 0.092 / 0.102-0.146 ms; the
// defaults 64 and 16 keep small lattices' i lines from idling most of a
// block, and the solver's tuner picks per lattice.

// One instance per candidate tile width (face_tile.cuh): faces along i of
// 32, 64 or 128, along j or k of 8, 16 or 32; the solver times them when it
// is created and keeps the fastest per direction (the same arithmetic,
// only the staging differs).
template <int D, int TILE>
__global__ void __launch_bounds__(kFaceThreads, CFD_MFACE_MIN_BLOCKS) k_face_tile_m(LatView g)
{
    using T = FaceTile<D, TILE>;
    __shared__ float smem[tile_smem_floats<T>()];
    mx::face_tile<T, D>(g, tile_of_block<T>(), smem);
}

template <int D, int TILE>
void launch_tile_m(const LatView &g, cudaStream_t st)
{
    k_face_tile_m<D, TILE><<<FaceTile<D, TILE>::grid(g), kFaceThreads, 0, st>>>(g);
}

template <int D>
void launch_face_tile(const LatView &g, cudaStream_t st, int tile)
{
    if constexpr (D == 0) {
        if (tile == 32) launch_tile_m<0, 32>(g, st);
        else if (tile == 128) launch_tile_m<0, 128>(g, st);
        else launch_tile_m<0, 64>(g, st);
    } else {
        if (tile == 8) launch_tile_m<D, 8>(g, st);
        else if (tile == 32) launch_tile_m<D, 32>(g, st);
        else launch_tile_m<D, 16>(g, st);
    }
}

template <bool LOC>
__global__ void __launch_bounds__(256) k_update_m(LatView g, int jst)
{
    const int n = node_id();
    if (n < g.N) mx::update_node<LOC>(g, n, jst);
}

// one thread per (entry, target node), a group of entries (one singular
// wall node) on one thread in order; a list whose groups touch each other's
// rows runs in list order on one thread
__global__ void k_bc_m(LatView g, const BcEntry *__restrict__ E, int n, int type, int q, double mach, int sequential)
{
    if (sequential) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            for (int e = 0; e < n; ++e)
                for (int m = 0; m < 4; ++m) mx::bc_target(g, type, E[e], m, q, mach);
        return;
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 4 * n)
        bc_for_group<4>(E, t >> 2, n, t & 3,
                        [&](const BcEntry &e, int m) { mx::bc_target(g, type, e, m, q, mach); });
}

// every target of independent lists in one launch
__global__ void k_bc_m_fused(LatView g, const BcEntry *__restrict__ E, BcOffsets off, int q, double mach)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * off.o[BC_NTYPES]) return;
    const int type = bc_type_of(off, t >> 2);
    bc_for_group<4>(E, t >> 2, off.o[BC_NTYPES], t & 3,
                    [&](const BcEntry &e, int m) { mx::bc_target(g, type, e, m, q, mach); });
}

__global__ void k_flow_out_m(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) mx::flow_out_node(g, n, q);
}

__global__ void k_u_out_m(LatView g, int q, double *__restrict__ aos)
{
    const int n = node_id();
    if (n >= g.N) return;
    const float *W = lat_W(g, q);
    const size_t r = g.row_of ? (size_t)g.row_of[n] : (size_t)n + 1;
#pragma unroll
    for (int c = 0; c < 5; ++c) aos[r * 5 + c] = (double)W[c * g.N + n] + (double)W[(5 + c) * g.N + n];
}

__global__ void k_to_float(const double *__restrict__ a, float *__restrict__ b, long long n)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = (float)a[t];
}

// node32 = [9 node metrics, det, det^(-1/3)] in FP32; idet32 = 1/det as hi, lo
__global__ void k_node_geometry(const double *__restrict__ m9, const double *__restrict__ det, long long N,
                                float *__restrict__ node32, float *__restrict__ idet32)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
#pragma unroll
    for (int c = 0; c < 9; ++c) node32[c * N + n] = (float)m9[c * N + n];
    node32[9 * N + n] = (float)det[n];
    node32[10 * N + n] = (float)(1.0 / cbrt(det[n]));
    const double id = 1.0 / det[n];
    const float h = (float)id;
    idet32[n] = h;
    idet32[N + n] = (float)(id - (double)h);
}

}  // namespace

void mixed_geometry(const StructuredLaunch &S)
{
    const long long N = (long long)S.ni * S.nj * S.nk;
    k_to_float<<<blocks_for(9 * N, 256), 256, 0, S.stream>>>(S.fm, S.fm32, 9 * N);
    k_to_float<<<blocks_for(3 * N, 256), 256, 0, S.stream>>>(S.fdet, S.fdet32, 3 * N);
    k_node_geometry<<<blocks_for(N, 256), 256, 0, S.stream>>>(S.m9, S.det, N, S.node32, S.idet32);
}

void bc_apply_mixed(cudaStream_t st, const BcDevice &bc, const LatView &g, int q, double mach)
{
    if (bc.fused) {
        if (bc.total() > 0) k_bc_m_fused<<<blocks_for(4LL * bc.total(), 128), 128, 0, st>>>(g, bc.all, bc.off, q, mach);
        return;
    }
    for (int t = 0; t < BC_NTYPES; ++t) {
        if (bc.n[t] == 0) continue;
        const unsigned blocks = bc.seq[t] ? 1u : blocks_for(4LL * bc.n[t], 128);
        k_bc_m<<<blocks, bc.seq[t] ? 1 : 128, 0, st>>>(g, bc.d[t], bc.n[t], t, q, mach, bc.seq[t]);
    }
}

void mixed_flow_out(const LatView &g, int q, cudaStream_t st)
{
    k_flow_out_m<<<blocks_for(g.N, 256), 256, 0, st>>>(g, q);
}

void mixed_u_out(const LatView &g, int q, double *aos, cudaStream_t st)
{
    k_u_out_m<<<blocks_for(g.N, 256), 256, 0, st>>>(g, q, aos);
}

int mixed_stage(const StructuredLaunch &S, int jst, double dt, double *Lout, cudaEvent_t *ev, int prep_from,
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
    if (prep_from == kPrepFromFlow) {
        k_init_m<<<nb256, 256, 0, st>>>(g, jst);
        name("prep");
        mark();
    } else if (prep_from >= 0) {
        k_prep_m<<<nb256, 256, 0, st>>>(g, prep_from, jst);
        name("prep");
        mark();
    }
    const bool loc = g.loc8 != nullptr;   // lattice with ghost layers and loc codes
    // The viscous pass and the face passes are independent (the update reads
    // both): without event timing the viscous pass runs on the side stream,
    // concurrently with the faces.
    const bool side = S.side && !ev;
    cudaStream_t sv = side ? S.side : st;
    if (side) {
        cudaEventRecord(S.fork, st);
        cudaStreamWaitEvent(sv, S.fork, 0);
    }
    if (S.P.viscous) {
        if (loc)
            k_visc_m<true><<<nb256, 256, 0, sv>>>(g, jst);
        else
            k_visc_m<false><<<nb256, 256, 0, sv>>>(g, jst);
        name("viscous");
    } else {
        k_mu_m<<<nb256, 256, 0, sv>>>(g, jst);
        name("mu_only");
    }
    if (side) cudaEventRecord(S.join, sv);
    mark();
    // the three face passes write separate fluxes: the j and k passes run on
    // their own streams, so that no pass waits for the last wave of another
    const bool fside = side && S.face_side[0] && S.face_side[1];
    cudaStream_t sj = fside ? S.face_side[0] : st, sk = fside ? S.face_side[1] : st;
    if (fside) {
        cudaStreamWaitEvent(sj, S.fork, 0);
        cudaStreamWaitEvent(sk, S.fork, 0);
    }
    launch_face_tile<0>(g, st, S.tile_i);
    name("face_i");
    mark();
    launch_face_tile<1>(g, sj, S.tile_jk);
    name("face_j");
    mark();
    launch_face_tile<2>(g, sk, S.tile_jk);
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
        k_update_m<true><<<nb256, 256, 0, st>>>(g, jst);
    else
        k_update_m<false><<<nb256, 256, 0, st>>>(g, jst);
    name("update+prep");
    mark();
    return k;
}

void mixed_face_pass(const StructuredLaunch &S, int d, int tile, cudaStream_t st)
{
    const LatView g = make_view(S, 0.0, nullptr);
    if (d == 0) launch_face_tile<0>(g, st, tile);
    else if (d == 1) launch_face_tile<1>(g, st, tile);
    else launch_face_tile<2>(g, st, tile);
}

namespace {

// rho = 1, zero velocity, p = 1: the FP32 face inputs of a uniform state
__global__ void k_uniform_inputs(float *Q32, float *R32, float *FEG32, long long N)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const float q[5] = {1.0f, 0.0f, 0.0f, 0.0f, 2.5f}, r[5] = {0.0f, 0.0f, 0.0f, 1.0f, 3.5f};
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        Q32[c * N + n] = q[c];
        R32[c * N + n] = r[c];
    }
#pragma unroll
    for (int c = 0; c < 15; ++c) FEG32[c * N + n] = 0.0f;
}

}  // namespace

void reduced_uniform_inputs(const StructuredLaunch &S, cudaStream_t st)
{
    const long long N = (long long)S.ni * S.nj * S.nk;
    k_uniform_inputs<<<blocks_for(N, 256), 256, 0, st>>>(S.Q32, S.R32, S.FEG32, N);
}

}  // namespace cfd

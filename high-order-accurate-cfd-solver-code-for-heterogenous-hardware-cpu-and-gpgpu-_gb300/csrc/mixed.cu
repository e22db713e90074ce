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
// Kernels per stage: k_visc_m (radius-2 star), k_face_m<d> x3 (one thread
// per face), k_update_m (RK stage + the next stage's U_Q); k_init_m /
// k_prep_m supply U_Q when no update produced it.  The per-node operations
// are in lattice_mixed.cuh.  This file is compiled with FMA contraction on
// and approximate FP32 division/square root (the mixed form's error budget
// is 1e-6 relative L2 against the FP64 form).
#include "boundary.h"
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

template <bool LOC>
__global__ void __launch_bounds__(256) k_visc_m(LatView g, int q)
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

template <int D>
__global__ void __launch_bounds__(128, CFD_MFACE_MIN_BLOCKS) k_face_m(LatView g)
{
    const int n = node_id();
    if (n < g.N) mx::face_node<D>(g, n);
}

template <bool LOC>
__global__ void __launch_bounds__(256) k_update_m(LatView g, int jst)
{
    const int n = node_id();
    if (n < g.N) mx::update_node<LOC>(g, n, jst);
}

__global__ void k_bc_m(LatView g, const BcEntry *__restrict__ E, int n, int type, int q, double mach, int sequential)
{
    if (sequential) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            for (int e = 0; e < n; ++e) mx::bc_entry(g, type, E[e], q, mach);
        return;
    }
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) mx::bc_entry(g, type, E[e], q, mach);
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
    for (int t = 0; t < BC_NTYPES; ++t) {
        if (bc.n[t] == 0) continue;
        const unsigned blocks = bc.seq[t] ? 1u : blocks_for(bc.n[t], 128);
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
    const unsigned nb256 = blocks_for(g.N, 256), nb128 = blocks_for(g.N, 128);
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
    if (S.P.viscous) {
        if (loc)
            k_visc_m<true><<<nb256, 256, 0, st>>>(g, jst);
        else
            k_visc_m<false><<<nb256, 256, 0, st>>>(g, jst);
        name("viscous");
    } else {
        k_mu_m<<<nb256, 256, 0, st>>>(g, jst);
        name("mu_only");
    }
    mark();
    k_face_m<0><<<nb128, 128, 0, st>>>(g);
    name("face_i");
    mark();
    k_face_m<1><<<nb128, 128, 0, st>>>(g);
    name("face_j");
    mark();
    k_face_m<2><<<nb128, 128, 0, st>>>(g);
    name("face_k");
    mark();
    if (loc)
        k_update_m<true><<<nb256, 256, 0, st>>>(g, jst);
    else
        k_update_m<false><<<nb256, 256, 0, st>>>(g, jst);
    name("update+prep");
    mark();
    return k;
}

}  // namespace cfd

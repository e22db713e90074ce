// mixed.cu -- the mixed-precision form of the structured (lattice) stage.
//
// What runs in FP32: the characteristic projection, WENO5 weights and
// reconstruction, the LLF split and face fluxes, the viscous and SGS fluxes,
// the node fluxes used by the sixth-order correction.  What stays FP64: the
// conserved state U0/U1/U2 and FLOW, the RK3 stage accumulation and the
// right-hand side sum, the derivatives of U that feed the viscous terms, and
// the metric/Jacobian inputs (rounded to FP32 only where a face flux uses
// them).  Stage intermediates are stored in FP32 (half the bytes).
//
// Kernels per stage: k_prep_m (pointwise), k_visc_m (radius-2 star),
// k_face_m<d> x3 (one thread per face), k_update_m (FP64 RK stage); the
// per-node operations are in lattice_mixed.cuh.  This file is compiled with
// FMA contraction on and approximate FP32 division/square root (the mixed
// form's error budget is 1e-6 relative L2 against the FP64 form).
#include "internal.h"
#include "lattice_mixed.cuh"
#include "structured.h"

namespace cfd {

namespace {

__device__ __forceinline__ int node_id() { return blockIdx.x * blockDim.x + threadIdx.x; }

__global__ void __launch_bounds__(256) k_prep_m(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) mx::prep_node(g, n, q);
}

__global__ void __launch_bounds__(256) k_visc_m(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) mx::visc_node(g, n, q);
}

__global__ void __launch_bounds__(256) k_mu_m(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) mx::mu_node(g, n, q);
}

template <int D>
__global__ void __launch_bounds__(128) k_face_m(LatView g)
{
    const int n = node_id();
    if (n < g.N) mx::face_node<D>(g, n);
}

__global__ void __launch_bounds__(256) k_update_m(LatView g, int jst)
{
    const int n = node_id();
    if (n < g.N) mx::update_node(g, n, jst, false);
}

__global__ void __launch_bounds__(256) k_update_prep_m(LatView g, int jst)
{
    const int n = node_id();
    if (n < g.N) mx::update_node(g, n, jst, true);
}

__global__ void k_recip(const double *__restrict__ a, double *__restrict__ b, long long n)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = 1.0 / a[t];
}

__global__ void k_to_float(const double *__restrict__ a, float *__restrict__ b, long long n)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = (float)a[t];
}

}  // namespace

void mixed_geometry(const StructuredLaunch &S)
{
    const long long N = (long long)S.ni * S.nj * S.nk;
    k_to_float<<<blocks_for(9 * N, 256), 256, 0, S.stream>>>(S.fm, S.fm32, 9 * N);
    k_to_float<<<blocks_for(3 * N, 256), 256, 0, S.stream>>>(S.fdet, S.fdet32, 3 * N);
    k_to_float<<<blocks_for(9 * N, 256), 256, 0, S.stream>>>(S.m9, S.m932, 9 * N);
    k_recip<<<blocks_for(N, 256), 256, 0, S.stream>>>(S.det, S.idet, N);
}

int mixed_stage(const StructuredLaunch &S, int jst, double dt, double *Lout, cudaEvent_t *ev, bool prep, bool fuse,
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
    if (prep) {
        k_prep_m<<<nb256, 256, 0, st>>>(g, jst);
        name("prep");
        mark();
    }
    if (S.P.viscous) {
        k_visc_m<<<nb256, 256, 0, st>>>(g, jst);
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
    if (fuse) {
        k_update_prep_m<<<nb256, 256, 0, st>>>(g, jst);
        name("update+prep");
    } else {
        k_update_m<<<nb256, 256, 0, st>>>(g, jst);
        name("update");
    }
    mark();
    return k;
}

}  // namespace cfd

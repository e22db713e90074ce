// structured.cu -- face-based RHS kernels for an (i,j,k) lattice, FP64 form.
//
// When the reference's neighbour table is a lattice -- periodic, or padded by
// ghost layers in non-periodic directions (detected by the solver at create
// time, lattice_host.h) -- the same arithmetic runs on a structure-of-arrays
// layout with index arithmetic instead of neighbour chains, and every face is
// computed once.  The reference computes each face twice: as i+1/2 of node i
// and as i-1/2 of node i+1, from identical inputs (the face metric and face
// det of Main.cpp:2369-2440 are single-valued, the Roe average is symmetric
// in its two nodes), so one evaluation per face gives the same fluxes.
//
// Per RK stage j:
//   k_prep    pointwise: Q, U_j = det*Q (U_Q.cl), contravariant node fluxes
//             F,E,G (Viscous.cl:560-631), sqrt(rho) and H for the Roe average
//   k_visc    radius-2 star: viscous + MTS SGS fluxes Fv,Ev,Gv and mu
//   k_face<d, mb> one thread per face i+1/2 along d (face_fp64.cuh, at the
//     register budget the solver's tuner picked): Roe eigenvectors, WENO5,
//             LLF, 6th-order correction -> corrected face flux
//   k_update  pointwise + radius-2: L = -(flux differences + viscous
//             divergence), SSP-RK3 stage j, primitive recovery
// Layout: every field is [component][N] with n = i + ni*(j + nj*k).
//
// The per-node operations live in lattice_fp64.cuh (exact evaluation order)
// and this file is compiled with --fmad=false: the face flux of face i+1/2 is
// bit-identical to what the reference computes for it (twice).  The mixed
// form lives in mixed.cu.
#include "internal.h"
#include "lattice_fp64.cuh"
#include "structured.h"

namespace cfd {

namespace {

__device__ __forceinline__ int node_id() { return blockIdx.x * blockDim.x + threadIdx.x; }

__global__ void __launch_bounds__(128) k_prep(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) ex::prep_node(g, n, q);
}

__global__ void __launch_bounds__(128) k_visc(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) ex::visc_node(g, n, q);
}

__global__ void __launch_bounds__(128) k_mu_only(LatView g, int q)
{
    const int n = node_id();
    if (n < g.N) ex::mu_node(g, n, q);
}


__global__ void __launch_bounds__(128) k_update(LatView g, int jst)
{
    const int n = node_id();
    if (n < g.N) ex::update_node(g, n, jst, false);
}

// AoS reference rows (row stride `stride` doubles) <-> SoA [comp][N].
__global__ void k_aos_to_soa(const double *__restrict__ aos, int stride, int ncomp, long long N,
                             double *__restrict__ soa, const int *__restrict__ row_of)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * ncomp) return;
    const long long n = t / ncomp;
    const int c = (int)(t % ncomp);
    const long long r = row_of ? (long long)row_of[n] : n + 1;
    soa[c * N + n] = aos[r * stride + c];
}

__global__ void k_soa_to_aos(const double *__restrict__ soa, int stride, int ncomp, long long N,
                             double *__restrict__ aos, const int *__restrict__ row_of)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * ncomp) return;
    const long long n = t / ncomp;
    const int c = (int)(t % ncomp);
    const long long r = row_of ? (long long)row_of[n] : n + 1;
    aos[r * stride + c] = soa[c * N + n];
}

}  // namespace

int structured_stage(const StructuredLaunch &S, int jst, double dt, double *Lout, cudaEvent_t *ev,
                     const char **names, int prep_from)
{
    if (S.mixed == 2) return split_stage(S, jst, dt, Lout, ev, prep_from, names);
    if (S.mixed) return mixed_stage(S, jst, dt, Lout, ev, prep_from, names);
    const LatView g = make_view(S, dt, Lout);
    const unsigned nb = blocks_for(g.N, 128);
    cudaStream_t st = S.stream;
    int e = 0;
    auto mark = [&]() {
        if (ev) cudaEventRecord(ev[e++], st);
    };
    static const char *fp64_names[6] = {"prep", "viscous", "face_i", "face_j", "face_k", "update"};
    if (names)
        for (int i = 0; i < 6; ++i) names[i] = fp64_names[i];
    if (names && !S.P.viscous) names[1] = "mu_only";
    mark();
    k_prep<<<nb, 128, 0, st>>>(g, jst);
    mark();
    if (S.P.viscous)
        k_visc<<<nb, 128, 0, st>>>(g, jst);
    else
        k_mu_only<<<nb, 128, 0, st>>>(g, jst);
    mark();
    fp64_face_pass(g, 0, S.face_mb[0], st);
    mark();
    fp64_face_pass(g, 1, S.face_mb[1], st);
    mark();
    fp64_face_pass(g, 2, S.face_mb[2], st);
    mark();
    k_update<<<nb, 128, 0, st>>>(g, jst);
    mark();
    return 6;
}

void fp64_face_pass(const LatView &g, int d, int mb, cudaStream_t st)
{
    if (mb == 2)
        fp64_face_pass_mb2(g, d, st);
    else if (mb == 4)
        fp64_face_pass_mb4(g, d, st);
    else
        fp64_face_pass_mb3(g, d, st);
}

void fp64_face_pass(const StructuredLaunch &S, int d, int mb, cudaStream_t st)
{
    fp64_face_pass(make_view(S, 0.0, nullptr), d, mb, st);
}

void fp64_prep_pass(const StructuredLaunch &S, int jst)
{
    const LatView g = make_view(S, 0.0, nullptr);
    k_prep<<<blocks_for(g.N, 128), 128, 0, S.stream>>>(g, jst);
}

void aos_to_soa(cudaStream_t st, const double *aos, int stride, int ncomp, long long N, double *soa, const int *row_of)
{
    const long long t = N * ncomp;
    k_aos_to_soa<<<blocks_for(t, 256), 256, 0, st>>>(aos, stride, ncomp, N, soa, row_of);
}

void soa_to_aos(cudaStream_t st, const double *soa, int stride, int ncomp, long long N, double *aos, const int *row_of)
{
    const long long t = N * ncomp;
    k_soa_to_aos<<<blocks_for(t, 256), 256, 0, st>>>(soa, stride, ncomp, N, aos, row_of);
}

}  // namespace cfd

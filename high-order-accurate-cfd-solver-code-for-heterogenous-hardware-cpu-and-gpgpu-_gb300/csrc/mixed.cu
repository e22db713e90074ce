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
// k_face_m<d> x3 (one thread per face), k_update_m (FP64 RK stage).
// This file is compiled with FMA contraction on and approximate FP32
// division/square root (the mixed form's error budget is 1e-6 relative L2
// against the FP64 form).
#include "internal.h"
#include "structured.h"

namespace cfd {

namespace {

__device__ __forceinline__ int wrapm(int x, int n)
{
    x %= n;
    return x < 0 ? x + n : x;
}

struct LatM {
    int ni, nj, nk;
    long long N;
    __device__ __forceinline__ void ijk(long long n, int &i, int &j, int &k) const
    {
        i = (int)(n % ni);
        const long long r = n / ni;
        j = (int)(r % nj);
        k = (int)(r / nj);
    }
    __device__ __forceinline__ long long step(int i, int j, int k, int d, int o) const
    {
        const int ii = d == 0 ? wrapm(i + o, ni) : i;
        const int jj = d == 1 ? wrapm(j + o, nj) : j;
        const int kk = d == 2 ? wrapm(k + o, nk) : k;
        return (long long)ii + (long long)ni * ((long long)jj + (long long)nj * kk);
    }
};

enum { FU = 0, FV = 1, FW = 2, FP = 3, FT = 4, FRHO = 5, FMU = 6, FA = 7, FE = 8 };

// Pointwise: U_j = det*Q (FP64, as U_Q.cl), and the FP32 stage inputs of
// the face kernels: Q, Roe inputs (u, v, w, sqrt(rho), H), node fluxes.
__global__ void __launch_bounds__(256) k_prep_m(LatM g, const double *__restrict__ m9, const double *__restrict__ det,
                                                const double *__restrict__ prim9, double *__restrict__ Uj,
                                                float *__restrict__ Q32, float *__restrict__ R32,
                                                float *__restrict__ FEG32)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    const double rho = prim9[FRHO * N + n], u = prim9[FU * N + n], v = prim9[FV * N + n], w = prim9[FW * N + n],
                 p = prim9[FP * N + n];
    const double D = det[n];
    const double ke = 0.5 * rho * (u * u + v * v + w * w);
    const double E = (p / 0.4) + ke;
    Uj[0 * N + n] = D * rho;
    Uj[1 * N + n] = D * rho * u;
    Uj[2 * N + n] = D * rho * v;
    Uj[3 * N + n] = D * rho * w;
    Uj[4 * N + n] = D * E;
    Q32[0 * N + n] = (float)rho;
    Q32[1 * N + n] = (float)(rho * u);
    Q32[2 * N + n] = (float)(rho * v);
    Q32[3 * N + n] = (float)(rho * w);
    Q32[4 * N + n] = (float)E;
    R32[0 * N + n] = (float)u;
    R32[1 * N + n] = (float)v;
    R32[2 * N + n] = (float)w;
    R32[3 * N + n] = (float)sqrt(rho);
    R32[4 * N + n] = (float)((E + p) / rho);
    float m[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) m[k] = (float)m9[k * N + n];
    const float prim[5] = {(float)rho, (float)u, (float)v, (float)w, (float)p};
    float F[5], Ec[5], G[5];
    node_inviscid_flux<float>(prim, m, (float)D, F, Ec, G);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        FEG32[(0 * 5 + c) * N + n] = F[c];
        FEG32[(1 * 5 + c) * N + n] = Ec[c];
        FEG32[(2 * 5 + c) * N + n] = G[c];
    }
}

// Viscous + MTS SGS fluxes: derivatives of U in FP64 (differences of nearly
// equal values), everything after them in FP32.
__global__ void __launch_bounds__(256) k_visc_m(LatM g, Phys P, const double *__restrict__ m9,
                                                const double *__restrict__ det, const double *__restrict__ Uj,
                                                double *__restrict__ prim9, float *__restrict__ V32)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    int i, j, k;
    g.ijk(n, i, j, k);
    float dU[3][5], KS[3], Ui[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) Ui[c] = (float)Uj[c * N + n];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long m2 = g.step(i, j, k, d, -2), m1 = g.step(i, j, k, d, -1), p1 = g.step(i, j, k, d, 1),
                        p2 = g.step(i, j, k, d, 2);
#pragma unroll
        for (int c = 0; c < 5; ++c)
            dU[d][c] = (float)((1.0 / 12.0) * (8.0 * (Uj[c * N + p1] - Uj[c * N + m1]) - (Uj[c * N + p2] - Uj[c * N + m2])));
        const int c = d + 1;
        const float um = (float)Uj[c * N + m1], up = (float)Uj[c * N + p1];
        const float rm = (float)Uj[m1], rp = (float)Uj[p1];
        const float dlt = (Ui[c] / Ui[0]) - ((0.25f * um + 0.5f * Ui[c] + 0.25f * up) / (0.25f * rm + 0.5f * Ui[0] + 0.25f * rp));
        KS[d] = dlt * dlt;
    }
    float m[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) m[q] = (float)m9[q * N + n];
    const float prim[5] = {(float)prim9[FRHO * N + n], (float)prim9[FU * N + n], (float)prim9[FV * N + n],
                           (float)prim9[FW * N + n], (float)prim9[FP * N + n]};
    float Fv[5], Ev[5], Gv[5], mu;
    viscous_node_flux<float>(dU, Ui, m, (float)det[n], prim, KS, P, Fv, Ev, Gv, mu);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        V32[(0 * 5 + c) * N + n] = Fv[c];
        V32[(1 * 5 + c) * N + n] = Ev[c];
        V32[(2 * 5 + c) * N + n] = Gv[c];
    }
    prim9[FMU * N + n] = (double)mu;
}

// Sutherland viscosity only (inviscid runs still report mu).
__global__ void __launch_bounds__(256) k_mu_m(LatM g, Phys P, const double *__restrict__ Uj, double *__restrict__ prim9)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    const float U0 = (float)Uj[n], iU0 = 1.0f / U0;
    const float uu = (float)Uj[N + n] * iU0, vv = (float)Uj[2 * N + n] * iU0, ww = (float)Uj[3 * N + n] * iU0;
    const float d_temp = 1.4f * (float)P.mach * (float)P.mach * 0.4f * ((float)Uj[4 * N + n] * iU0 - 0.5f * (uu * uu + vv * vv + ww * ww));
    const float sd = sqrtf(d_temp);
    const float S = 110.4f / (float)P.t_inf;
    prim9[FMU * N + n] = (double)((sd * sd * sd) * ((1.0f + S) / (d_temp + S)));
}

// One thread per face n+1/2 along D, all FP32.
template <int D>
__global__ void __launch_bounds__(128) k_face_m(LatM g, float eps, const float *__restrict__ Q32,
                                                const float *__restrict__ R32, const float *__restrict__ fm32,
                                                const float *__restrict__ fdet32, const float *__restrict__ FEG32,
                                                float *__restrict__ Fh32)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    int i, j, k;
    g.ijk(n, i, j, k);
    long long s[6];
#pragma unroll
    for (int o = 0; o < 6; ++o) s[o] = g.step(i, j, k, D, o - 2);
    float pts[6][5];
#pragma unroll
    for (int o = 0; o < 6; ++o)
#pragma unroll
        for (int c = 0; c < 5; ++c) pts[o][c] = Q32[c * N + s[o]];
    float roe[5];
    {
        const long long l = s[2], r = s[3];
        roe_average<float>(R32[3 * N + r], R32[r], R32[N + r], R32[2 * N + r], R32[4 * N + r], R32[3 * N + l],
                           R32[l], R32[N + l], R32[2 * N + l], R32[4 * N + l], roe);
    }
    float Fhat[5];
    llf_face_flux<float>(pts, fm32[(D * 3 + 0) * N + n], fm32[(D * 3 + 1) * N + n], fm32[(D * 3 + 2) * N + n],
                         fdet32[D * N + n], roe, eps, Fhat);
    const float *NF = FEG32 + (size_t)D * 5 * N;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        float f[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) f[o] = NF[c * N + s[o]];
        Fh32[(D * 5 + c) * N + n] = Fhat[c] + face_correction<float>(f);
    }
}

// RHS sum and SSP-RK3 stage in FP64 from the FP32 face and viscous fluxes.
__global__ void __launch_bounds__(256) k_update_m(LatM g, int viscous, int jst, double mach, double dt,
                                                  const double *__restrict__ det, const float *__restrict__ Fh32,
                                                  const float *__restrict__ V32, double *__restrict__ U0,
                                                  double *__restrict__ U1, double *__restrict__ U2,
                                                  double *__restrict__ prim9, unsigned *flags,
                                                  double *__restrict__ Lout)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    int i, j, k;
    g.ijk(n, i, j, k);
    double L[5] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long m1 = g.step(i, j, k, d, -1);
#pragma unroll
        for (int c = 0; c < 5; ++c) L[c] += (double)Fh32[(d * 5 + c) * N + n] - (double)Fh32[(d * 5 + c) * N + m1];
        if (viscous) {
            const long long m2 = g.step(i, j, k, d, -2), p1 = g.step(i, j, k, d, 1), p2 = g.step(i, j, k, d, 2);
            const float *Vd = V32 + (size_t)d * 5 * N;
#pragma unroll
            for (int c = 0; c < 5; ++c)
                L[c] += (double)((1.0f / 12.0f) * (8.0f * (Vd[c * N + p1] - Vd[c * N + m1]) - (Vd[c * N + p2] - Vd[c * N + m2])));
        }
    }
#pragma unroll
    for (int c = 0; c < 5; ++c) L[c] = -L[c];
    if (Lout) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Lout[c * N + n] = L[c];
    }
    double Un[5];
    if (jst == 0) {
#pragma unroll
        for (int c = 0; c < 5; ++c) { Un[c] = U0[c * N + n] + dt * L[c]; U1[c * N + n] = Un[c]; }
    } else if (jst == 1) {
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            Un[c] = 0.75 * U0[c * N + n] + 0.25 * U1[c * N + n] + 0.25 * dt * L[c];
            U2[c * N + n] = Un[c];
        }
    } else {
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            Un[c] = (1.0 / 3.0) * U0[c * N + n] + (2.0 / 3.0) * U2[c * N + n] + (2.0 / 3.0) * (dt * L[c]);
            U0[c * N + n] = Un[c];
        }
    }
    const double idet = 1.0 / det[n];
    const double rho = idet * Un[0];
    const double ir = 1.0 / rho;
    const double u = (idet * Un[1]) * ir, v = (idet * Un[2]) * ir, w = (idet * Un[3]) * ir;
    const double e = ((idet * Un[4]) * ir) - 0.5 * (u * u + v * v + w * w);
    const double p = e * rho * 0.4;
    prim9[FRHO * N + n] = rho;
    prim9[FU * N + n] = u;
    prim9[FV * N + n] = v;
    prim9[FW * N + n] = w;
    prim9[FE * N + n] = e;
    prim9[FP * N + n] = p;
    prim9[FT * N + n] = (1.4 * mach * mach) * (p * ir);
    prim9[FA * N + n] = sqrt(1.4 * p * ir);
    if (!(isfinite(rho) && isfinite(u) && isfinite(v) && isfinite(w) && isfinite(p))) atomicOr(flags, CFD_FLAG_NONFINITE);
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
}

void mixed_stage(const StructuredLaunch &S, int jst, double dt, double *Lout, cudaEvent_t *ev)
{
    const LatM g{S.ni, S.nj, S.nk, (long long)S.ni * S.nj * S.nk};
    const unsigned nb256 = blocks_for(g.N, 256), nb128 = blocks_for(g.N, 128);
    cudaStream_t st = S.stream;
    double *Uj = S.U[jst];
    int e = 0;
    auto mark = [&]() {
        if (ev) cudaEventRecord(ev[e++], st);
    };
    mark();
    k_prep_m<<<nb256, 256, 0, st>>>(g, S.m9, S.det, S.prim9, Uj, S.Q32, S.R32, S.FEG32);
    mark();
    if (S.P.viscous)
        k_visc_m<<<nb256, 256, 0, st>>>(g, S.P, S.m9, S.det, Uj, S.prim9, S.V32);
    else
        k_mu_m<<<nb256, 256, 0, st>>>(g, S.P, Uj, S.prim9);
    mark();
    const float eps = (float)S.P.eps;
    k_face_m<0><<<nb128, 128, 0, st>>>(g, eps, S.Q32, S.R32, S.fm32, S.fdet32, S.FEG32, S.Fh32);
    mark();
    k_face_m<1><<<nb128, 128, 0, st>>>(g, eps, S.Q32, S.R32, S.fm32, S.fdet32, S.FEG32, S.Fh32);
    mark();
    k_face_m<2><<<nb128, 128, 0, st>>>(g, eps, S.Q32, S.R32, S.fm32, S.fdet32, S.FEG32, S.Fh32);
    mark();
    k_update_m<<<nb256, 256, 0, st>>>(g, S.P.viscous, jst, S.P.mach, dt, S.det, S.Fh32, S.V32, S.U[0], S.U[1],
                                      S.U[2], S.prim9, S.flags, Lout);
    mark();
}

}  // namespace cfd

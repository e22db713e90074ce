// lattice_mixed.cuh -- per-node operations of the mixed-precision lattice
// stage.  FP32: characteristic projection, WENO5, LLF, face and node fluxes,
// viscous/SGS fluxes.  FP64: the state U0/U1/U2 and FLOW, the RHS sum and RK
// accumulation, the derivatives of U feeding the viscous terms, and the
// geometry inputs.  Include only from translation units compiled with FMA
// contraction and approximate FP32 division/square root.
#pragma once

#include "lattice.cuh"

namespace cfd {
namespace mx {

// U_Q for one node from primitives in registers: U_q = det*Q (FP64) and the
// FP32 inputs of the face stage: Q, Roe inputs (u, v, w, sqrt(rho), H), node
// fluxes.
__device__ __forceinline__ void prep_values(const LatView &g, int n, int q, double rho, double u, double v, double w,
                                            double p)
{
    const int N = g.N;
    const double D = g.det[n];
    const double ke = 0.5 * rho * (u * u + v * v + w * w);
    const double E = p * 2.5 + ke;
    double *Uq = lat_U(g, q);
    Uq[0 * N + n] = D * rho;
    Uq[1 * N + n] = D * rho * u;
    Uq[2 * N + n] = D * rho * v;
    Uq[3 * N + n] = D * rho * w;
    Uq[4 * N + n] = D * E;
    g.Q32[0 * N + n] = (float)rho;
    g.Q32[1 * N + n] = (float)(rho * u);
    g.Q32[2 * N + n] = (float)(rho * v);
    g.Q32[3 * N + n] = (float)(rho * w);
    g.Q32[4 * N + n] = (float)E;
    const float rf = (float)rho;
    g.R32[0 * N + n] = (float)u;
    g.R32[1 * N + n] = (float)v;
    g.R32[2 * N + n] = (float)w;
    g.R32[3 * N + n] = sqrtf(rf);
    g.R32[4 * N + n] = (float)(E + p) / rf;
    float m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = g.m9_32[c * N + n];
    const float prim[5] = {rf, (float)u, (float)v, (float)w, (float)p};
    float F[5], Ec[5], G[5];
    node_inviscid_flux<float>(prim, m, (float)D, F, Ec, G);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        g.FEG32[(0 * 5 + c) * N + n] = F[c];
        g.FEG32[(1 * 5 + c) * N + n] = Ec[c];
        g.FEG32[(2 * 5 + c) * N + n] = G[c];
    }
}

__device__ __forceinline__ void prep_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    prep_values(g, n, q, g.prim9[LF_RHO * N + n], g.prim9[LF_U * N + n], g.prim9[LF_V * N + n],
                g.prim9[LF_W * N + n], g.prim9[LF_P * N + n]);
}

// Viscous + MTS SGS fluxes: derivatives of U_q in FP64, the rest in FP32.
__device__ __forceinline__ void visc_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    const double *Uj = lat_U(g, q);
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    float dU[3][5], KS[3], Ui[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) Ui[c] = (float)Uj[c * N + n];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int m2 = lat_step(g, i, j, k, d, -2), m1 = lat_step(g, i, j, k, d, -1), p1 = lat_step(g, i, j, k, d, 1),
                  p2 = lat_step(g, i, j, k, d, 2);
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
    for (int c = 0; c < 9; ++c) m[c] = g.m9_32[c * N + n];
    const float prim[5] = {(float)g.prim9[LF_RHO * N + n], (float)g.prim9[LF_U * N + n], (float)g.prim9[LF_V * N + n],
                           (float)g.prim9[LF_W * N + n], (float)g.prim9[LF_P * N + n]};
    float Fv[5], Ev[5], Gv[5], mu;
    viscous_node_flux<float>(dU, Ui, m, (float)g.det[n], prim, KS, g.P, Fv, Ev, Gv, mu);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        g.V32[(0 * 5 + c) * N + n] = Fv[c];
        g.V32[(1 * 5 + c) * N + n] = Ev[c];
        g.V32[(2 * 5 + c) * N + n] = Gv[c];
    }
    g.prim9[LF_MU * N + n] = (double)mu;
}

__device__ __forceinline__ void mu_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    const double *Uj = lat_U(g, q);
    const float U0 = (float)Uj[n], iU0 = 1.0f / U0;
    const float uu = (float)Uj[N + n] * iU0, vv = (float)Uj[2 * N + n] * iU0, ww = (float)Uj[3 * N + n] * iU0;
    const float mach = (float)g.P.mach;
    const float d_temp = 1.4f * mach * mach * 0.4f * ((float)Uj[4 * N + n] * iU0 - 0.5f * (uu * uu + vv * vv + ww * ww));
    const float sd = sqrtf(d_temp);
    const float S = 110.4f / (float)g.P.t_inf;
    g.prim9[LF_MU * N + n] = (double)((sd * sd * sd) * ((1.0f + S) / (d_temp + S)));
}

// Face n+1/2 along D, all FP32.
template <int D>
__device__ __forceinline__ void face_node(const LatView &g, int n)
{
    const int N = g.N;
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    int s[6];
#pragma unroll
    for (int o = 0; o < 6; ++o) s[o] = lat_step(g, i, j, k, D, o - 2);
    float pts[6][5];
#pragma unroll
    for (int o = 0; o < 6; ++o)
#pragma unroll
        for (int c = 0; c < 5; ++c) pts[o][c] = g.Q32[c * N + s[o]];
    float r[5];
    {
        const int l = s[2], rr = s[3];
        const float *R = g.R32;
        roe_average<float>(R[3 * N + rr], R[rr], R[N + rr], R[2 * N + rr], R[4 * N + rr], R[3 * N + l], R[l],
                           R[N + l], R[2 * N + l], R[4 * N + l], r);
    }
    float Fhat[5];
    llf_face_flux<float>(pts, g.fm32[(D * 3 + 0) * N + n], g.fm32[(D * 3 + 1) * N + n], g.fm32[(D * 3 + 2) * N + n],
                         g.fdet32[D * N + n], r, (float)g.P.eps, Fhat);
    const float *NF = g.FEG32 + (size_t)D * 5 * N;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        float f[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) f[o] = NF[c * N + s[o]];
        g.Fh32[(D * 5 + c) * N + n] = Fhat[c] + face_correction<float>(f);
    }
}

// 1/x in FP64 from an FP32 seed and two Newton steps (relative error near
// FP64 rounding; the mixed form does not need the correctly rounded value).
__device__ __forceinline__ double recip_fast(double x)
{
    double r = (double)(1.0f / (float)x);
    r = r * fma(-x, r, 2.0);
    r = r * fma(-x, r, 2.0);
    return r;
}

// RHS and SSP-RK3 stage from the FP32 face and viscous fluxes.  L is summed
// in FP32: neighbouring face fluxes are within a factor of two of each other,
// so their FP32 difference is exact, and L's error is dominated by the FP32
// face fluxes themselves.  The RK accumulation and the state are FP64.  With
// fuse_next, the next stage's prep on the new primitives.
__device__ __forceinline__ void update_node(const LatView &g, int n, int jst, bool fuse_next)
{
    const int N = g.N;
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    float Lf[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int m1 = lat_step(g, i, j, k, d, -1);
#pragma unroll
        for (int c = 0; c < 5; ++c) Lf[c] += g.Fh32[(d * 5 + c) * N + n] - g.Fh32[(d * 5 + c) * N + m1];
        if (g.P.viscous) {
            const int m2 = lat_step(g, i, j, k, d, -2), p1 = lat_step(g, i, j, k, d, 1), p2 = lat_step(g, i, j, k, d, 2);
            const float *Vd = g.V32 + (size_t)d * 5 * N;
#pragma unroll
            for (int c = 0; c < 5; ++c)
                Lf[c] += (1.0f / 12.0f) * (8.0f * (Vd[c * N + p1] - Vd[c * N + m1]) - (Vd[c * N + p2] - Vd[c * N + m2]));
        }
    }
    double L[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) L[c] = -(double)Lf[c];
    if (g.Lout) {
#pragma unroll
        for (int c = 0; c < 5; ++c) g.Lout[c * N + n] = L[c];
    }
    const double dt = g.dt;
    double Un[5];
    if (jst == 0) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Un[c] = g.U0[c * N + n] + dt * L[c];
    } else if (jst == 1) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Un[c] = 0.75 * g.U0[c * N + n] + 0.25 * g.U1[c * N + n] + 0.25 * dt * L[c];
    } else {
#pragma unroll
        for (int c = 0; c < 5; ++c)
            Un[c] = (1.0 / 3.0) * g.U0[c * N + n] + (2.0 / 3.0) * g.U2[c * N + n] + (2.0 / 3.0) * (dt * L[c]);
    }
    double *Uo = jst == 0 ? g.U1 : (jst == 1 ? g.U2 : g.U0);
    if (!fuse_next) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Uo[c * N + n] = Un[c];
    }
    const double idet = g.idet[n];
    const double rho = idet * Un[0];
    const double ir = recip_fast(rho);
    const double s = idet * ir;
    const double u = Un[1] * s, v = Un[2] * s, w = Un[3] * s;
    const double e = Un[4] * s - 0.5 * (u * u + v * v + w * w);
    const double p = e * rho * 0.4;
    const double mach = g.P.mach;
    const double pr = p * ir;
    g.prim9[LF_RHO * N + n] = rho;
    g.prim9[LF_U * N + n] = u;
    g.prim9[LF_V * N + n] = v;
    g.prim9[LF_W * N + n] = w;
    g.prim9[LF_E * N + n] = e;
    g.prim9[LF_P * N + n] = p;
    g.prim9[LF_T * N + n] = (1.4 * mach * mach) * pr;
    g.prim9[LF_A * N + n] = (double)sqrtf(1.4f * (float)pr);
    if (!(isfinite(rho) && isfinite(u) && isfinite(v) && isfinite(w) && isfinite(p))) atomicOr(g.flags, 2u);
    // the next stage's U_Q overwrites U_{jst+1} (mod 3) with det*Q(FLOW)
    if (fuse_next) prep_values(g, n, jst == 2 ? 0 : jst + 1, rho, u, v, w, p);
}

}  // namespace mx
}  // namespace cfd

// lattice_mixed.cuh -- per-node operations of the mixed-precision lattice
// stage, written for a part whose FP64 rate is a small fraction of its FP32
// rate.
//
// State: each conserved value of U0/U1/U2 is carried as hi + lo, two FP32
// numbers (about 48 significant bits; double-float arithmetic after Dekker,
// "A floating-point technique for extending the available precision", 1971,
// with the FMA-based exact product).  The RK3 accumulation runs in that
// arithmetic on the FP32 pipe.
// FP32: characteristic projection, WENO5, LLF, face and node fluxes, the
// viscous/SGS fluxes, the right-hand side sum, and the primitives derived
// from the state each stage (rounded once from hi/lo quotients).  On a
// lattice with ghost layers the same loc-code branches as the FP64 form,
// and the boundary routine on the hi/lo state (bc_target).
// FP64 only at the boundary: FLOW in (kPrepFromFlow) and FLOW/U out.
// Include only from translation units compiled with FMA contraction and
// approximate FP32 division/square root; the hi/lo routines below use
// explicit fmaf and plain additions, which contraction leaves exact.
#pragma once

#include "boundary.h"
#include "face_tile.cuh"
#include "lattice.cuh"
#include "physics_x2.cuh"

namespace cfd {
namespace mx {

struct dfl {
    float h, l;
};

// s + e == a + b exactly (Knuth's two-sum)
__device__ __forceinline__ dfl two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

// s + e == a + b exactly when |a| >= |b| or a == 0 (Dekker's fast two-sum)
__device__ __forceinline__ dfl quick_two_sum(float a, float b)
{
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ dfl df_add(dfl x, dfl y)
{
    const dfl s = two_sum(x.h, y.h);
    const dfl t = two_sum(x.l, y.l);
    dfl v = quick_two_sum(s.h, s.l + t.h);
    return quick_two_sum(v.h, t.l + v.l);
}

// x * c, c given as hi + lo
__device__ __forceinline__ dfl df_mul(dfl x, dfl c)
{
    const float p = x.h * c.h;
    float e = fmaf(x.h, c.h, -p);
    e = fmaf(x.h, c.l, fmaf(x.l, c.h, e));
    return quick_two_sum(p, e);
}

// x * c rounded once to FP32
__device__ __forceinline__ float df_mul_f(dfl x, dfl c)
{
    return fmaf(x.h, c.h, fmaf(x.h, c.l, x.l * c.h));
}

// a / b rounded to FP32 (within about one ulp), r an approximation of 1/b.h
__device__ __forceinline__ float df_div_f(dfl a, dfl b, float r)
{
    const float q = a.h * r;
    const float rem = fmaf(-q, b.h, a.h) + (a.l - q * b.l);
    return fmaf(rem, r, q);
}

// a / b as hi + lo (error near 2^-44 relative)
__device__ __forceinline__ dfl df_div(dfl a, dfl b, float r)
{
    const float q = df_div_f(a, b, r);
    const float p = q * b.h;
    const float pe = fmaf(q, b.h, -p);
    // remainder a - q*b, then one correction step
    const float rem = ((a.h - p) - pe) + (a.l - q * b.l);
    return quick_two_sum(q, rem * r);
}

// 1/3 and 2/3 as hi + lo
constexpr float kThirdH = (float)(1.0 / 3.0);
constexpr float kThirdL = (float)(1.0 / 3.0 - (double)(float)(1.0 / 3.0));
constexpr float kTwoThirdH = (float)(2.0 / 3.0);
constexpr float kTwoThirdL = (float)(2.0 / 3.0 - (double)(float)(2.0 / 3.0));
// gamma - 1 = 0.4 as hi + lo
constexpr float kGm1H = (float)0.4;
constexpr float kGm1L = (float)(0.4 - (double)(float)0.4);

__device__ __forceinline__ void load_state(const LatView &g, int q, int n, dfl Un[5])
{
    const int N = g.N;
    const float *W = lat_W(g, q);
#pragma unroll
    for (int c = 0; c < 5; ++c) Un[c] = {W[c * N + n], W[(5 + c) * N + n]};
}

__device__ __forceinline__ void store_state(const LatView &g, int q, int n, const dfl Un[5])
{
    const int N = g.N;
    float *W = lat_W(g, q);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        W[c * N + n] = Un[c].h;
        W[(5 + c) * N + n] = Un[c].l;
    }
}

// U_Q of the next stage from the state Un (= det * Q): the inputs of the
// face stage -- Q, the Roe inputs (u, v, w, sqrt(rho), H), the contravariant
// node fluxes -- and the pressure (prim32); the viscous pass takes rho from
// Q and u, v, w from the Roe inputs, and FLOW leaves through flow_out_node.
__device__ __forceinline__ void derive(const LatView &g, int n, const dfl Un[5])
{
    const int N = g.N;
    const dfl idet = {g.idet32[n], g.idet32[N + n]};
    const float r0 = 1.0f / Un[0].h;
    const float rho = df_mul_f(Un[0], idet);
    const float u = df_div_f(Un[1], Un[0], r0), v = df_div_f(Un[2], Un[0], r0), w = df_div_f(Un[3], Un[0], r0);
    const float ke = 0.5f * (u * u + v * v + w * w);
    const dfl q4 = df_div(Un[4], Un[0], r0);   // E / rho
    const dfl e2 = df_add(q4, {-ke, 0.0f});      // internal energy e
    const dfl rho2 = df_mul(Un[0], idet);
    const float p = df_mul_f(df_mul(rho2, e2), {kGm1H, kGm1L});
    const float irho = 1.0f / rho;
    const float pr = p * irho;
    g.prim32[LF_P * N + n] = p;
    if (!(isfinite(rho) && isfinite(u) && isfinite(v) && isfinite(w) && isfinite(p))) atomicOr(g.flags, 2u);
    const float E = df_mul_f(Un[4], idet);
    g.Q32[0 * N + n] = rho;
    g.Q32[1 * N + n] = df_mul_f(Un[1], idet);
    g.Q32[2 * N + n] = df_mul_f(Un[2], idet);
    g.Q32[3 * N + n] = df_mul_f(Un[3], idet);
    g.Q32[4 * N + n] = E;
    g.R32[0 * N + n] = u;
    g.R32[1 * N + n] = v;
    g.R32[2 * N + n] = w;
    g.R32[3 * N + n] = sqrtf(rho);
    g.R32[4 * N + n] = q4.h + (q4.l + pr);     // H = E/rho + p/rho
    float m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = g.node32[c * N + n];
    const float prim[5] = {rho, u, v, w, p};
    float Fx[5], Ex[5], Gx[5];
    node_inviscid_flux<float>(prim, m, g.node32[9 * N + n], Fx, Ex, Gx);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        g.FEG32[(0 * 5 + c) * N + n] = Fx[c];
        g.FEG32[(1 * 5 + c) * N + n] = Ex[c];
        g.FEG32[(2 * 5 + c) * N + n] = Gx[c];
    }
}

// U_Q from the FP64 FLOW (after an upload): U = det * Q(FLOW) in FP64, split
// into hi + lo in slot q, then derive.
__device__ __forceinline__ void init_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    const double rho = g.prim9[LF_RHO * N + n], u = g.prim9[LF_U * N + n], v = g.prim9[LF_V * N + n],
                 w = g.prim9[LF_W * N + n], p = g.prim9[LF_P * N + n];
    const double D = g.det[n];
    const double E = p / 0.4 + 0.5 * rho * (u * u + v * v + w * w);
    const double U[5] = {D * rho, D * rho * u, D * rho * v, D * rho * w, D * E};
    dfl Un[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        Un[c].h = (float)U[c];
        Un[c].l = (float)(U[c] - (double)Un[c].h);
    }
    store_state(g, q, n, Un);
    g.prim32[LF_MU * N + n] = (float)g.prim9[LF_MU * N + n];
    derive(g, n, Un);
}

// U_Q from the state in slot src, copied to slot dst (a stage run out of the
// usual order: U_dst = det * Q(FLOW) with FLOW the current state).
__device__ __forceinline__ void prep_node(const LatView &g, int n, int src, int dst)
{
    dfl Un[5];
    load_state(g, src, n, Un);
    if (src != dst) store_state(g, dst, n, Un);
    derive(g, n, Un);
}

// Derivative of branch b (physics.cuh visc_branch) from the six neighbour
// differences dl[m] = f[m+1] - f[m] of the values at offsets -3..3: every
// formula rewritten as a sum of neighbour differences, which the hi/lo
// state gives to FP32 accuracy.
__device__ __forceinline__ float branch_deriv_diff(int b, const float dl[6])
{
    switch (b) {
    case 1: return (1.0f / 6.0f) * (11.0f * dl[2] - 7.0f * dl[1] + 2.0f * dl[0]);
    case 2: return (1.0f / 6.0f) * (11.0f * dl[3] - 7.0f * dl[4] + 2.0f * dl[5]);
    case 3: return (1.0f / 6.0f) * (2.0f * dl[3] + 5.0f * dl[2] - dl[1]);
    case 4: return (1.0f / 6.0f) * (2.0f * dl[2] + 5.0f * dl[3] - dl[4]);
    case 5: return (1.0f / 12.0f) * (8.0f * (dl[2] + dl[3]) - (dl[1] + dl[2] + dl[3] + dl[4]));
    default: return 0.0f;
    }
}

// Viscous + MTS SGS fluxes from slot q.  Derivatives of U from hi/lo
// differences (exact hi differences for neighbours within a factor of two):
// central on a periodic lattice (LOC = false), the reference's loc-code
// branches on a lattice with loc codes (LOC = true; zero at ghosts);
// everything else in FP32.
template <bool LOC>
__device__ __forceinline__ void visc_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    const float *W = lat_W(g, q);
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    float dU[3][5], KS[3], Ui[5];
    const bool ghost = LOC && lat_ghost(g, n);
    const unsigned lflag = (LOC && g.locflag) ? g.locflag[n] : 7u;
#pragma unroll
    for (int c = 0; c < 5; ++c) Ui[c] = W[c * N + n];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int m2 = lat_step(g, i, j, k, d, -2), m1 = lat_step(g, i, j, k, d, -1), p1 = lat_step(g, i, j, k, d, 1),
                  p2 = lat_step(g, i, j, k, d, 2);
        if (ghost) {
#pragma unroll
            for (int c = 0; c < 5; ++c) dU[d][c] = 0.0f;
        } else if (!LOC || !lat_locdir(g, d) || !((lflag >> d) & 1u)) {
#pragma unroll
            for (int c = 0; c < 5; ++c) {
                // the state slot is read-only in this pass: non-coherent loads
                const float *H = W + c * N, *L = W + (5 + c) * N;
                const float d1 = (__ldg(H + p1) - __ldg(H + m1)) + (__ldg(L + p1) - __ldg(L + m1));
                const float d2 = (__ldg(H + p2) - __ldg(H + m2)) + (__ldg(L + p2) - __ldg(L + m2));
                dU[d][c] = (1.0f / 12.0f) * (8.0f * d1 - d2);
            }
        } else {
            int s[7], L7[7];
#pragma unroll
            for (int o = 0; o < 7; ++o) {
                s[o] = lat_step(g, i, j, k, d, o - 3);
                L7[o] = g.loc8[s[o]];
            }
            const int b = visc_branch(L7);
#pragma unroll
            for (int c = 0; c < 5; ++c) {
                const float *H = W + c * N, *L = W + (5 + c) * N;
                float dl[6];
#pragma unroll
                for (int m = 0; m < 6; ++m) dl[m] = (H[s[m + 1]] - H[s[m]]) + (L[s[m + 1]] - L[s[m]]);
                dU[d][c] = branch_deriv_diff(b, dl);
            }
        }
        const int c = d + 1;
        const float um = __ldg(W + c * N + m1), up = __ldg(W + c * N + p1);
        const float rm = __ldg(W + m1), rp = __ldg(W + p1);
        const float dlt = qdiv(Ui[c], Ui[0]) - qdiv(0.25f * um + 0.5f * Ui[c] + 0.25f * up, 0.25f * rm + 0.5f * Ui[0] + 0.25f * rp);
        KS[d] = dlt * dlt;
    }
    float m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = g.node32[c * N + n];
    const float prim[5] = {g.Q32[n], g.R32[n], g.R32[N + n], g.R32[2 * N + n], g.prim32[LF_P * N + n]};
    float Fv[5], Ev[5], Gv[5], mu;
    viscous_node_flux<float>(dU, Ui, m, g.node32[9 * N + n], g.node32[10 * N + n], prim, KS, g.P, Fv, Ev, Gv, mu);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        g.V32[(0 * 5 + c) * N + n] = Fv[c];
        g.V32[(1 * 5 + c) * N + n] = Ev[c];
        g.V32[(2 * 5 + c) * N + n] = Gv[c];
    }
    g.prim32[LF_MU * N + n] = mu;
}

__device__ __forceinline__ void mu_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    const float *W = lat_W(g, q);
    const float U0 = W[n], iU0 = qdiv(1.0f, U0);
    const float uu = W[N + n] * iU0, vv = W[2 * N + n] * iU0, ww = W[3 * N + n] * iU0;
    const float mach = (float)g.P.mach;
    const float d_temp = 1.4f * mach * mach * 0.4f * (W[4 * N + n] * iU0 - 0.5f * (uu * uu + vv * vv + ww * ww));
    const float sd = sqrtf(d_temp);
    const float S = 110.4f / (float)g.P.t_inf;
    g.prim32[LF_MU * N + n] = (sd * sd * sd) * qdiv(1.0f + S, d_temp + S);
}

// Face n+1/2 along D, all FP32, on paired lanes (physics_x2.cuh).
template <int D>
__device__ __forceinline__ void face_node(const LatView &g, int n)
{
    const int N = g.N;
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    if (!lat_face_needed(g, i, j, k, D)) return;
    int s[6];
#pragma unroll
    for (int o = 0; o < 6; ++o) s[o] = lat_step(g, i, j, k, D, o - 2);
    float2 P[3][5];   // (point k, point 5-k)
#pragma unroll
    for (int o = 0; o < 3; ++o)
#pragma unroll
        for (int c = 0; c < 5; ++c) P[o][c] = make_float2(g.Q32[c * N + s[o]], g.Q32[c * N + s[5 - o]]);
    float r[5];
    {
        const int l = s[2], rr = s[3];
        const float *R = g.R32;
        roe_average<float>(R[3 * N + rr], R[rr], R[N + rr], R[2 * N + rr], R[4 * N + rr], R[3 * N + l], R[l],
                           R[N + l], R[2 * N + l], R[4 * N + l], r);
    }
    float Fhat[5];
    x2::llf_face_flux2(P, g.fm32[(D * 3 + 0) * N + n], g.fm32[(D * 3 + 1) * N + n], g.fm32[(D * 3 + 2) * N + n],
                       g.fdet32[D * N + n], r, (float)g.P.eps, Fhat);
    const float *NF = g.FEG32 + (size_t)D * 5 * N;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        float f[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) f[o] = NF[c * N + s[o]];
        g.Fh32[(D * 5 + c) * N + n] = Fhat[c] + x2::face_correction_sym(f);
    }
}

// Faces along D of one staged tile (face_tile.cuh): the block of
// kFaceThreads threads stages the tile's stencil lines into smem
// (tile_smem_floats<T>() floats) and each thread evaluates its face.  Every
// thread of the block must call it (it synchronises the block).  RO as in
// stage_face_lines.
template <class T, int D, bool RO = true>
__device__ __forceinline__ void face_tile(const LatView &g, TileAt at, float *smem)
{
    constexpr int S = T::kStaged;
    float *sQ = smem, *sR = smem + 5 * S, *sF = smem + 10 * S;
    stage_face_lines<T, D, RO>(g, at, sQ, sR, sF);
    int n, t, a;
    if (!tile_face<T, D>(g, at, n, t, a)) return;
    const int N = g.N;
    float2 P[3][5];
    float r[5];
    tile_stencil<T>(sQ, sR, t, a, P, r);
    float Fhat[5];
    x2::llf_face_flux2(P, g.fm32[(D * 3 + 0) * N + n], g.fm32[(D * 3 + 1) * N + n], g.fm32[(D * 3 + 2) * N + n],
                       g.fdet32[D * N + n], r, (float)g.P.eps, Fhat);
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        float f[6];
        tile_node_fluxes<T>(sF, q, t, a, f);
        g.Fh32[(D * 5 + q) * N + n] = Fhat[q] + x2::face_correction_sym(f);
    }
}

// RHS and SSP-RK3 stage jst from the FP32 face and viscous fluxes, then the
// next stage's U_Q.  L is summed in FP32 (neighbouring face fluxes within a
// factor of two subtract exactly); the RK accumulation is hi/lo:
//   jst 0: U1 = U0 + dt L
//   jst 1: U2 = 3/4 U0 + 1/4 U1 + 1/4 dt L
//   jst 2: U0 = 1/3 U0 + 2/3 U2 + 2/3 dt L
// and the new state lands in slot (jst+1) mod 3, which is also the next
// stage's U_Q slot.  LOC as for visc_node.  RO: the face and viscous
// fluxes were written by an earlier launch, so they may be read through the
// non-coherent path (not in the batched kernel, which writes them in the
// same launch).
template <bool LOC, bool RO = true>
__device__ __forceinline__ void update_node(const LatView &g, int n, int jst)
{
    auto ld = [](const float *p) { return RO ? __ldg(p) : *p; };
    const int N = g.N;
    if (LOC && lat_ghost(g, n)) {
        // Ghosts are the boundary routine's, which fills those next to face
        // nodes after this kernel; the others (behind edges and corners) keep
        // their state, which moves on to the next stage's slot.
        if (g.Lout) {
#pragma unroll
            for (int c = 0; c < 5; ++c) g.Lout[c * N + n] = 0.0;
        }
        dfl Us[5];
        load_state(g, jst, n, Us);
        store_state(g, jst == 2 ? 0 : jst + 1, n, Us);
        return;
    }
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    const unsigned lflag = (LOC && g.locflag) ? g.locflag[n] : 7u;
    float Lf[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int m1 = lat_step(g, i, j, k, d, -1);
#pragma unroll
        for (int c = 0; c < 5; ++c) Lf[c] += ld(g.Fh32 + (d * 5 + c) * N + n) - ld(g.Fh32 + (d * 5 + c) * N + m1);
        if (LOC && g.P.viscous && lat_locdir(g, d) && ((lflag >> d) & 1u)) {
            int s[7], L7[7];
#pragma unroll
            for (int o = 0; o < 7; ++o) {
                s[o] = lat_step(g, i, j, k, d, o - 3);
                L7[o] = g.loc8[s[o]];
            }
            const int b = weno_visc_branch(L7);
            const float *Vd = g.V32 + (size_t)d * 5 * N;
#pragma unroll
            for (int c = 0; c < 5; ++c) {
                float f[7];
#pragma unroll
                for (int o = 0; o < 7; ++o) f[o] = ld(Vd + c * N + s[o]);
                Lf[c] += branch_deriv<float>(b, f);
            }
        } else if (g.P.viscous) {
            const int m2 = lat_step(g, i, j, k, d, -2), p1 = lat_step(g, i, j, k, d, 1), p2 = lat_step(g, i, j, k, d, 2);
            const float *Vd = g.V32 + (size_t)d * 5 * N;
#pragma unroll
            for (int c = 0; c < 5; ++c)
                Lf[c] += (1.0f / 12.0f) * (8.0f * (ld(Vd + c * N + p1) - ld(Vd + c * N + m1))
                                           - (ld(Vd + c * N + p2) - ld(Vd + c * N + m2)));
        }
    }
    if (g.Lout) {
#pragma unroll
        for (int c = 0; c < 5; ++c) g.Lout[c * N + n] = -(double)Lf[c];
    }
    const dfl dt = {g.dt_hi, g.dt_lo};
    dfl U0[5], Un[5];
    load_state(g, 0, n, U0);
    if (jst == 0) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Un[c] = df_add(U0[c], df_mul({-Lf[c], 0.0f}, dt));
    } else if (jst == 1) {
        dfl U1[5];
        load_state(g, 1, n, U1);
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            const dfl a = df_mul(U0[c], {0.75f, 0.0f});
            const dfl b = {0.25f * U1[c].h, 0.25f * U1[c].l};
            const dfl t = df_mul({-0.25f * Lf[c], 0.0f}, dt);
            Un[c] = df_add(df_add(a, b), t);
        }
    } else {
        dfl U2[5];
        load_state(g, 2, n, U2);
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            const dfl a = df_mul(U0[c], {kThirdH, kThirdL});
            const dfl b = df_mul(U2[c], {kTwoThirdH, kTwoThirdL});
            const dfl t = df_mul(df_mul({-Lf[c], 0.0f}, dt), {kTwoThirdH, kTwoThirdL});
            Un[c] = df_add(df_add(a, b), t);
        }
    }
    store_state(g, jst == 2 ? 0 : jst + 1, n, Un);
    derive(g, n, Un);
}

// ------------------------------------------------ boundary routine ---

// FP64 primitives of the hi/lo state of node n in slot q.
__device__ __forceinline__ void state_prims(const LatView &g, int q, int n, double mach, double &rho, double &u,
                                            double &v, double &w, double &p, double &t)
{
    const int N = g.N;
    const float *W = lat_W(g, q);
    double fu[5];
    const double id = 1.0 / g.det[n];
#pragma unroll
    for (int c = 0; c < 5; ++c) fu[c] = id * ((double)W[c * N + n] + (double)W[(5 + c) * N + n]);
    rho = fu[0];
    u = fu[1] / fu[0];
    v = fu[2] / fu[0];
    w = fu[3] / fu[0];
    const double e = fu[4] / fu[0] - 0.5 * (u * u + v * v + w * w);
    p = e * rho * 0.4;
    t = (1.4 * mach * mach) * (p / rho);
}

// Node n takes the state of primitives (rho, u, v, w, p) in slot q, and the
// next stage's U_Q outputs.
__device__ __forceinline__ void set_prims(const LatView &g, int q, int n, double rho, double u, double v, double w,
                                          double p)
{
    const double D = g.det[n];
    const double E = p / 0.4 + 0.5 * rho * (u * u + v * v + w * w);
    const double U[5] = {D * rho, D * rho * u, D * rho * v, D * rho * w, D * E};
    dfl Un[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        Un[c].h = (float)U[c];
        Un[c].l = (float)(U[c] - (double)Un[c].h);
    }
    store_state(g, q, n, Un);
    derive(g, n, Un);
}

// Target m of one entry of the reference's boundary routine
// (bc_target_rules) on the hi/lo state in slot q.
struct HiLoState {
    const LatView &g;
    int q;
    double mach;
    __device__ __forceinline__ void prims(int n, double &rho, double &u, double &v, double &w, double &p,
                                          double &t) const
    {
        state_prims(g, q, n, mach, rho, u, v, w, p, t);
    }
    __device__ __forceinline__ void set(int n, double rho, double u, double v, double w, double p) const
    {
        set_prims(g, q, n, rho, u, v, w, p);
    }
};

__device__ __forceinline__ void bc_target(const LatView &g, int type, const BcEntry &e, int m, int q, double mach)
{
    bc_target_rules(HiLoState{g, q, mach}, type, e, m, mach);
}

// FP64 FLOW of the state in slot q (boundary output): the FP64 form's
// primitive formulas on hi + lo; mu from the last viscous pass.
__device__ __forceinline__ void flow_out_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    const float *W = lat_W(g, q);
    double fu[5];
    const double id = 1.0 / g.det[n];
#pragma unroll
    for (int c = 0; c < 5; ++c) fu[c] = id * ((double)W[c * N + n] + (double)W[(5 + c) * N + n]);
    const double rho = fu[0], u = fu[1] / fu[0], v = fu[2] / fu[0], w = fu[3] / fu[0];
    const double e = (fu[4] / fu[0]) - 0.5 * (u * u + v * v + w * w);
    const double p = e * rho * 0.4;
    const double mach = g.P.mach;
    double *F = g.prim9;
    F[LF_RHO * N + n] = rho;
    F[LF_U * N + n] = u;
    F[LF_V * N + n] = v;
    F[LF_W * N + n] = w;
    F[LF_E * N + n] = e;
    F[LF_P * N + n] = p;
    F[LF_T * N + n] = (1.4 * mach * mach) * (p / rho);
    F[LF_A * N + n] = sqrt(1.4 * p / rho);
    F[LF_MU * N + n] = (double)g.prim32[LF_MU * N + n];
}

}  // namespace mx
}  // namespace cfd

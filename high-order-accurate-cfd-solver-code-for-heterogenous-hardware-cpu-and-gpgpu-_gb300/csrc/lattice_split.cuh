// lattice_split.cuh -- per-node operations of the split-precision lattice
// stage: FP64 for what carries the conserved state and the geometry, FP32
// for the flux physics.
//
// FP64: the state U0/U1/U2 ([5][N] doubles, the FP64 form's layout), the
// SSP-RK3 accumulation (Weno.cl:3084-3126), Q = U / det through the FP64
// reciprocal of det (U_Q.cl:112-122), the contravariant face flux
// DET_f (m_f . F) of the reconstructed face states with its LLF central
// average (Weno.cl:2585-2728, 2913-2947; physics_x2.cuh
// llf_face_flux2_split), and the flux difference L (Weno.cl:3060-3082).
// FP32: the Roe average, eigenvectors, characteristic projection, WENO5 (on
// the stencil's deviation from the face's left node), back-projection, the
// face states' velocities and pressures, lambda_5 and the LLF dissipation
// alpha (q+ - q-), the viscous and SGS fluxes and their divergence
// (Viscous.cl:439-631, the mixed form's code on a hi + lo FP32 read copy of
// the FP64 state), and the node fluxes with the sixth-order correction
// -d2/24 + 7 d4/5760 they feed (a high-order correction added to the FP64
// face flux).
// Include only from translation units compiled with FMA contraction and
// approximate FP32 division/square root.
#pragma once

#include "boundary.h"
#include "lattice.cuh"
#include "lattice_mixed.cuh"
#include "physics_x2.cuh"

namespace cfd {
namespace sp {

__device__ __forceinline__ void load_state(const LatView &g, int q, int n, double Un[5])
{
    const int N = g.N;
    const double *U = lat_U(g, q);
#pragma unroll
    for (int c = 0; c < 5; ++c) Un[c] = U[c * N + n];
}

__device__ __forceinline__ void store_state(const LatView &g, int q, int n, const double Un[5])
{
    const int N = g.N;
    double *U = lat_U(g, q);
#pragma unroll
    for (int c = 0; c < 5; ++c) U[c * N + n] = Un[c];
}

// U_Q of the next stage from the state Un (= det * Q): Q in FP64, rounded
// once to FP32 for the face stage; the Roe inputs (u, v, w, sqrt(rho), H),
// the pressure and the contravariant node fluxes in FP32; and the state as
// hi + lo FP32 pairs in g.Whl ([10][N]), a read copy from which the viscous
// pass takes its neighbour differences on the FP32 pipe (the differences of
// hi parts are exact between neighbours within a factor of two).
__device__ __forceinline__ void derive(const LatView &g, int n, const double Un[5])
{
    const int N = g.N;
    // FP32 <-> FP64 conversions, the hi/lo split and the products by 1/det
    // on the integer pipe (emu64.cuh; the same bits as the FP64 pipe's)
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        float h, l;
        emu::hi_lo(Un[c], h, l);
        g.Whl[c * N + n] = h;
        g.Whl[(5 + c) * N + n] = l;
    }
    const double id = g.idet64[n];
    float q[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) q[c] = emu::d2f(emu::mul(Un[c], id));
    const float rho = q[0];
    const float ir = 1.0f / rho;
    const float u = q[1] * ir, v = q[2] * ir, w = q[3] * ir;
    const float p = 0.4f * (q[4] - 0.5f * (q[1] * u + q[2] * v + q[3] * w));
    g.prim32[LF_P * N + n] = p;
    if (!(isfinite(rho) && isfinite(u) && isfinite(v) && isfinite(w) && isfinite(p))) atomicOr(g.flags, 2u);
#pragma unroll
    for (int c = 0; c < 5; ++c) g.Q32[c * N + n] = q[c];
    g.R32[0 * N + n] = u;
    g.R32[1 * N + n] = v;
    g.R32[2 * N + n] = w;
    g.R32[3 * N + n] = sqrtf(rho);
    g.R32[4 * N + n] = (q[4] + p) * ir;   // H = (E + p) / rho
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

// U = det * Q(FLOW) in FP64 (U_Q.cl:112-116) into slot q, then derive.
__device__ __forceinline__ void set_prims(const LatView &g, int q, int n, double rho, double u, double v, double w,
                                          double p)
{
    const double D = g.det[n];
    const double E = p / 0.4 + 0.5 * rho * (u * u + v * v + w * w);
    const double Un[5] = {D * rho, D * rho * u, D * rho * v, D * rho * w, D * E};
    store_state(g, q, n, Un);
    derive(g, n, Un);
}

// U_Q from the FP64 FLOW (after an upload).
__device__ __forceinline__ void init_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    g.prim32[LF_MU * N + n] = (float)g.prim9[LF_MU * N + n];
    set_prims(g, q, n, g.prim9[LF_RHO * N + n], g.prim9[LF_U * N + n], g.prim9[LF_V * N + n], g.prim9[LF_W * N + n],
              g.prim9[LF_P * N + n]);
}

// U_Q from the state in slot src, copied to slot dst.
__device__ __forceinline__ void prep_node(const LatView &g, int n, int src, int dst)
{
    double Un[5];
    load_state(g, src, n, Un);
    if (src != dst) store_state(g, dst, n, Un);
    derive(g, n, Un);
}

// The view the mixed form's viscous pass (mx::visc_node, mx::mu_node) reads
// as its hi/lo state: every U slot aliases the read copy g.Whl of the
// current stage's state, which derive wrote.
__host__ __device__ __forceinline__ LatView hilo_view(const LatView &g)
{
    LatView v = g;
    v.U0 = v.U1 = v.U2 = reinterpret_cast<double *>(g.Whl);
    return v;
}

// The FP64 face flux of face n+1/2 along D from its stencil (P, pairs of
// points k and 5-k) and Roe state r, plus corr, the FP32 sixth-order
// correction of each component.
template <int D>
__device__ __forceinline__ void face_flux(const LatView &g, int n, const float2 P[3][5], const float r[5],
                                          const float corr[5], double out[5])
{
    const int N = g.N;
    const double dm[3] = {g.fm[(D * 3 + 0) * N + n], g.fm[(D * 3 + 1) * N + n], g.fm[(D * 3 + 2) * N + n]};
    x2::llf_face_flux2_split(P, g.fm32[(D * 3 + 0) * N + n], g.fm32[(D * 3 + 1) * N + n],
                             g.fm32[(D * 3 + 2) * N + n], dm, g.fdet[D * N + n], r, emu::d2f(g.P.eps), corr, out);
}

// Face n+1/2 along D with its stencil read from the lattice (the batched
// kernel's face item; the single-lattice pass stages tiles in split.cu).
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
    float2 P[3][5];
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
    const float *NF = g.FEG32 + (size_t)D * 5 * N;
    float corr[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        float f[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) f[o] = NF[c * N + s[o]];
        corr[c] = x2::face_correction_sym(f);
    }
    double Fh[5];
    face_flux<D>(g, n, P, r, corr, Fh);
#pragma unroll
    for (int c = 0; c < 5; ++c) g.Fh[(D * 5 + c) * N + n] = Fh[c];
}

// Faces along D of one staged tile (mx::face_tile with the FP64 face
// flux of face_flux written to Fh).
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
    float corr[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        float f[6];
        tile_node_fluxes<T>(sF, q, t, a, f);
        corr[q] = x2::face_correction_sym(f);
    }
    double Fh[5];
    face_flux<D>(g, n, P, r, corr, Fh);
#pragma unroll
    for (int q = 0; q < 5; ++q) g.Fh[(D * 5 + q) * N + n] = Fh[q];
}

// RHS and SSP-RK3 stage jst: the face-flux difference in FP64, the viscous
// divergence in FP32 (added in FP64), and the RK accumulation in FP64:
//   jst 0: U1 = U0 + dt L
//   jst 1: U2 = 3/4 U0 + 1/4 U1 + 1/4 dt L
//   jst 2: U0 = 1/3 U0 + 2/3 U2 + 2/3 dt L
// The new state lands in slot (jst+1) mod 3, which is also the next stage's
// U_Q slot.  LOC and RO as for the mixed form's update_node.
template <bool LOC, bool RO = true>
__device__ __forceinline__ void update_node(const LatView &g, int n, int jst)
{
    auto ldf = [](const float *p) { return RO ? __ldg(p) : *p; };
    auto ldd = [](const double *p) { return RO ? __ldg(p) : *p; };
    const int N = g.N;
    if (LOC && lat_ghost(g, n)) {   // ghosts: the state moves on (mixed form's update_node)
        if (g.Lout) {
#pragma unroll
            for (int c = 0; c < 5; ++c) g.Lout[c * N + n] = 0.0;
        }
        double Us[5];
        load_state(g, jst, n, Us);
        store_state(g, jst == 2 ? 0 : jst + 1, n, Us);
        return;
    }
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    const unsigned lflag = (LOC && g.locflag) ? g.locflag[n] : 7u;
    double Ld[5];   // sum of flux differences (= -L), started by the i direction's
    float Lv[5] = {0.f, 0.f, 0.f, 0.f, 0.f};     // viscous divergence
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int m1 = lat_step(g, i, j, k, d, -1);
        // FP64 pipe: the integer-pipe add (emu::add) costs more issue than it
        // frees here (TGV 128^3: update 0.23 -> 0.31 ms with one direction)
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            const double df = ldd(g.Fh + (d * 5 + c) * N + n) - ldd(g.Fh + (d * 5 + c) * N + m1);
            Ld[c] = d == 0 ? df : Ld[c] + df;
        }
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
                for (int o = 0; o < 7; ++o) f[o] = ldf(Vd + c * N + s[o]);
                Lv[c] += branch_deriv<float>(b, f);
            }
        } else if (g.P.viscous) {
            const int m2 = lat_step(g, i, j, k, d, -2), p1 = lat_step(g, i, j, k, d, 1), p2 = lat_step(g, i, j, k, d, 2);
            const float *Vd = g.V32 + (size_t)d * 5 * N;
#pragma unroll
            for (int c = 0; c < 5; ++c)
                Lv[c] += (1.0f / 12.0f) * (8.0f * (ldf(Vd + c * N + p1) - ldf(Vd + c * N + m1))
                                           - (ldf(Vd + c * N + p2) - ldf(Vd + c * N + m2)));
        }
    }
#pragma unroll
    for (int c = 0; c < 5; ++c) Ld[c] += emu::f2d(Lv[c]);
    if (g.Lout) {
#pragma unroll
        for (int c = 0; c < 5; ++c) g.Lout[c * N + n] = -Ld[c];
    }
    const double dt = g.dt;
    double U0[5], Un[5];
    load_state(g, 0, n, U0);
    if (jst == 0) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Un[c] = fma(-dt, Ld[c], U0[c]);
    } else if (jst == 1) {
        double U1[5];
        load_state(g, 1, n, U1);
#pragma unroll
        for (int c = 0; c < 5; ++c) Un[c] = fma(0.75, U0[c], fma(0.25, U1[c], (-0.25 * dt) * Ld[c]));
    } else {
        double U2[5];
        load_state(g, 2, n, U2);
#pragma unroll
        for (int c = 0; c < 5; ++c)
            Un[c] = fma(1.0 / 3.0, U0[c], fma(2.0 / 3.0, U2[c], (-2.0 / 3.0 * dt) * Ld[c]));
    }
    store_state(g, jst == 2 ? 0 : jst + 1, n, Un);
    derive(g, n, Un);
}

// ------------------------------------------------ boundary routine ---

// FP64 primitives of the state of node n in slot q.
__device__ __forceinline__ void state_prims(const LatView &g, int q, int n, double mach, double &rho, double &u,
                                            double &v, double &w, double &p, double &t)
{
    const int N = g.N;
    const double *U = lat_U(g, q);
    double fu[5];
    const double id = 1.0 / g.det[n];
#pragma unroll
    for (int c = 0; c < 5; ++c) fu[c] = id * U[c * N + n];
    rho = fu[0];
    u = fu[1] / fu[0];
    v = fu[2] / fu[0];
    w = fu[3] / fu[0];
    const double e = fu[4] / fu[0] - 0.5 * (u * u + v * v + w * w);
    p = e * rho * 0.4;
    t = (1.4 * mach * mach) * (p / rho);
}

struct F64State {
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
    bc_target_rules(F64State{g, q, mach}, type, e, m, mach);
}

// FP64 FLOW of the state in slot q (boundary output); mu from the last
// viscous pass.
__device__ __forceinline__ void flow_out_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    const double mach = g.P.mach;
    double rho, u, v, w, p, t;
    state_prims(g, q, n, mach, rho, u, v, w, p, t);
    double *F = g.prim9;
    F[LF_RHO * N + n] = rho;
    F[LF_U * N + n] = u;
    F[LF_V * N + n] = v;
    F[LF_W * N + n] = w;
    F[LF_E * N + n] = p / (0.4 * rho);
    F[LF_P * N + n] = p;
    F[LF_T * N + n] = t;
    F[LF_A * N + n] = sqrt(1.4 * p / rho);
    F[LF_MU * N + n] = (double)g.prim32[LF_MU * N + n];
}

}  // namespace sp
}  // namespace cfd

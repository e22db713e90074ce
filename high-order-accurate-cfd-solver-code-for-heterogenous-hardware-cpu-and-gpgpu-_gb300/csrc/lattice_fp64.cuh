// lattice_fp64.cuh -- per-node operations of the FP64 lattice stage in the
// reference's evaluation order (physics_exact.cuh).  Include only from
// translation units compiled with --fmad=false.
//
// One RK stage j = prep (U_Q) -> visc (Viscous) -> face x3 + update (Weno).
// The update can also perform the next stage's prep on the values it just
// produced (fused form); the arithmetic is identical to a separate prep pass.
#pragma once

#include "lattice.cuh"
#include "physics_exact.cuh"

namespace cfd {
namespace ex {

// U_Q.cl for one node from primitives in registers: U_q = det*Q, Q, the
// contravariant node fluxes (Viscous.cl:560-631), sqrt(rho) and H.
__device__ __forceinline__ void prep_values(const LatView &g, int n, int q, double rho, double u, double v, double w,
                                            double p)
{
    const int N = g.N;
    const double D = g.det[n];
    const double ke = xdiv::scale2<-1>(rho) * (u * u + v * v + w * w);   // 0.5 rho on the integer pipe, same bits
    const double E = dv(p, 0.4) + ke;
    double *Uq = lat_U(g, q);
    g.Q[0 * N + n] = rho;
    g.Q[1 * N + n] = rho * u;
    g.Q[2 * N + n] = rho * v;
    g.Q[3 * N + n] = rho * w;
    g.Q[4 * N + n] = E;
    Uq[0 * N + n] = D * rho;
    Uq[1 * N + n] = D * rho * u;
    Uq[2 * N + n] = D * rho * v;
    Uq[3 * N + n] = D * rho * w;
    Uq[4 * N + n] = D * E;
    double m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = g.m9[c * N + n];
    const double prim[5] = {rho, u, v, w, p};
    double F[5], Ec[5], G[5];
    node_flux(prim, m, D, F, Ec, G);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        g.FEG[(0 * 5 + c) * N + n] = F[c];
        g.FEG[(1 * 5 + c) * N + n] = Ec[c];
        g.FEG[(2 * 5 + c) * N + n] = G[c];
    }
    g.sh[n] = sqrt(rho);
    g.sh[N + n] = enthalpy(rho, u, v, w, p);
}

__device__ __forceinline__ void prep_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    prep_values(g, n, q, g.prim9[LF_RHO * N + n], g.prim9[LF_U * N + n], g.prim9[LF_V * N + n],
                g.prim9[LF_W * N + n], g.prim9[LF_P * N + n]);
}

// The seven nodes at offsets -3..3 along d and their loc codes.
__device__ __forceinline__ void loc_line(const LatView &g, int i, int j, int k, int d, int s[7], int L[7])
{
#pragma unroll
    for (int o = 0; o < 7; ++o) {
        s[o] = lat_step(g, i, j, k, d, o - 3);
        L[o] = g.loc8[s[o]];
    }
}

// Viscous.cl on a lattice: derivatives of U_q (4th-order central on a
// periodic lattice, where every node has loc 0; the loc-code branches of
// Viscous.cl:285-332 on a lattice with loc codes; zero at ghosts, which no
// branch covers), viscous + MTS SGS fluxes, mu.
__device__ __forceinline__ void visc_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    const double *Uj = lat_U(g, q);
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    double dU[3][5], KS[3], Ui[5];
    const bool ghost = lat_ghost(g, n);
    // nodes outside the loc-code band take the central branch (the same
    // expression as the reference's central branch: the same bits)
    const unsigned lflag = g.locflag ? g.locflag[n] : 7u;
#pragma unroll
    for (int c = 0; c < 5; ++c) Ui[c] = Uj[c * N + n];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int m2 = lat_step(g, i, j, k, d, -2), m1 = lat_step(g, i, j, k, d, -1), p1 = lat_step(g, i, j, k, d, 1),
                  p2 = lat_step(g, i, j, k, d, 2);
        if (ghost) {
#pragma unroll
            for (int c = 0; c < 5; ++c) dU[d][c] = 0.0;
        } else if (!lat_locdir(g, d) || !((lflag >> d) & 1u)) {
#pragma unroll
            for (int c = 0; c < 5; ++c)
                dU[d][c] = central4(Uj[c * N + m2], Uj[c * N + m1], Uj[c * N + p1], Uj[c * N + p2]);
        } else {
            int s[7], L[7];
            loc_line(g, i, j, k, d, s, L);
#pragma unroll
            for (int c = 0; c < 5; ++c) {
                double f[7];
#pragma unroll
                for (int o = 0; o < 7; ++o) f[o] = Uj[c * N + s[o]];
                dU[d][c] = visc_deriv_ref(f, L);
            }
        }
        const int c = d + 1;
        KS[d] = ks(Ui[c], Ui[0], Uj[c * N + m1], Uj[m1], Uj[c * N + p1], Uj[p1]);
    }
    double m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = g.m9[c * N + n];
    const double prim[5] = {g.prim9[LF_RHO * N + n], g.prim9[LF_U * N + n], g.prim9[LF_V * N + n],
                            g.prim9[LF_W * N + n], g.prim9[LF_P * N + n]};
    double Fv[5], Ev[5], Gv[5], mu;
    const Visc Vp{g.P.mach, g.P.reynolds, g.P.prandtl, g.P.t_inf, g.P.les, g.P.cs};
    viscous_node(dU, Ui, m, g.det[n], prim, KS, Vp, Fv, Ev, Gv, mu);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        g.V[(0 * 5 + c) * N + n] = Fv[c];
        g.V[(1 * 5 + c) * N + n] = Ev[c];
        g.V[(2 * 5 + c) * N + n] = Gv[c];
    }
    g.prim9[LF_MU * N + n] = mu;
}

// Sutherland viscosity only (inviscid runs still report mu, Viscous.cl:458).
__device__ __forceinline__ void mu_node(const LatView &g, int n, int q)
{
    const int N = g.N;
    const double *Uj = lat_U(g, q);
    const double Ui[5] = {Uj[n], Uj[N + n], Uj[2 * N + n], Uj[3 * N + n], Uj[4 * N + n]};
    g.prim9[LF_MU * N + n] = mu_of(Ui, g.P.mach, g.P.t_inf);
}

// Face n+1/2 along D: Roe average of the two nodes, LLF face flux and the
// 6th-order correction (Weno.cl:336-3058 for that face, once).  SD: shared
// reciprocals for divisions by one divisor (physics_exact.cuh Over).
template <int D, bool SD = true>
__device__ __forceinline__ void face_node(const LatView &g, int n)
{
    const int N = g.N;
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    if (!lat_face_needed(g, i, j, k, D)) return;
    int s[6];
#pragma unroll
    for (int o = 0; o < 6; ++o) s[o] = lat_step(g, i, j, k, D, o - 2);
    double pts[6][5];
#pragma unroll
    for (int o = 0; o < 6; ++o)
#pragma unroll
        for (int c = 0; c < 5; ++c) pts[o][c] = g.Q[c * N + s[o]];
    double r[5];
    {
        const int l = s[2], rr = s[3];   // node (left) and its +D neighbour
        roe<SD>(g.sh[rr], g.prim9[LF_U * N + rr], g.prim9[LF_V * N + rr], g.prim9[LF_W * N + rr], g.sh[N + rr],
                g.sh[l], g.prim9[LF_U * N + l], g.prim9[LF_V * N + l], g.prim9[LF_W * N + l], g.sh[N + l], r);
    }
    double Fhat[5];
    face_flux<SD>(pts, g.fm[(D * 3 + 0) * N + n], g.fm[(D * 3 + 1) * N + n], g.fm[(D * 3 + 2) * N + n], g.fdet[D * N + n],
              r, g.P.eps, Fhat);
    const double *NF = g.FEG + (size_t)D * 5 * N;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        double f[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) f[o] = NF[c * N + s[o]];
        g.Fh[(D * 5 + c) * N + n] = corrected(Fhat[c], f);
    }
}

// Weno.cl:3060-3135 at one owned node (ghosts are the boundary routine's):
// L from the face fluxes and the viscous divergence (the loc-code branches
// of Weno.cl:2732-2856 on a lattice with loc codes), SSP-RK3 stage jst,
// primitives.  With fuse_next the node then runs the next stage's prep on
// the new primitives.
__device__ __forceinline__ void update_node(const LatView &g, int n, int jst, bool fuse_next)
{
    const int N = g.N;
    if (lat_ghost(g, n)) {
        if (g.Lout) {
#pragma unroll
            for (int c = 0; c < 5; ++c) g.Lout[c * N + n] = 0.0;
        }
        return;
    }
    int i, j, k;
    lat_ijk(g, n, i, j, k);
    double dflux[3][5], dvis[3][5];
    const unsigned lflag = g.locflag ? g.locflag[n] : 7u;   // as in visc_node
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int m1 = lat_step(g, i, j, k, d, -1);
#pragma unroll
        for (int c = 0; c < 5; ++c) dflux[d][c] = g.Fh[(d * 5 + c) * N + n] - g.Fh[(d * 5 + c) * N + m1];
        if (g.P.viscous && lat_locdir(g, d) && ((lflag >> d) & 1u)) {
            int s[7], L[7];
            loc_line(g, i, j, k, d, s, L);
            const double *Vd = g.V + (size_t)d * 5 * N;
#pragma unroll
            for (int c = 0; c < 5; ++c) {
                double f[7];
#pragma unroll
                for (int o = 0; o < 7; ++o) f[o] = Vd[c * N + s[o]];
                dvis[d][c] = weno_visc_deriv_ref(f, L);
            }
        } else if (g.P.viscous) {
            const int m2 = lat_step(g, i, j, k, d, -2), p1 = lat_step(g, i, j, k, d, 1), p2 = lat_step(g, i, j, k, d, 2);
            const double *Vd = g.V + (size_t)d * 5 * N;
#pragma unroll
            for (int c = 0; c < 5; ++c) dvis[d][c] = central4(Vd[c * N + m2], Vd[c * N + m1], Vd[c * N + p1], Vd[c * N + p2]);
        } else {
#pragma unroll
            for (int c = 0; c < 5; ++c) dvis[d][c] = 0.0;
        }
    }
    double L[5];
#pragma unroll
    for (int c = 0; c < 5; ++c)
        L[c] = (-1.0) * (dflux[0][c] + dflux[1][c] + dflux[2][c] + dvis[0][c] + dvis[1][c] + dvis[2][c]);
    if (g.Lout) {
#pragma unroll
        for (int c = 0; c < 5; ++c) g.Lout[c * N + n] = L[c];
    }
    double u0[5], u1[5], u2[5], Un[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) { u0[c] = g.U0[c * N + n]; u1[c] = g.U1[c * N + n]; u2[c] = g.U2[c * N + n]; }
    double rho, u, v, w, e, p, t, a;
    rk_and_primitives(jst, g.dt, g.P.mach, g.det[n], u0, u1, u2, L, Un, rho, u, v, w, e, p, t, a);
    double *Uo = jst == 0 ? g.U1 : (jst == 1 ? g.U2 : g.U0);
#pragma unroll
    for (int c = 0; c < 5; ++c) Uo[c * N + n] = Un[c];
    g.prim9[LF_RHO * N + n] = rho;
    g.prim9[LF_U * N + n] = u;
    g.prim9[LF_V * N + n] = v;
    g.prim9[LF_W * N + n] = w;
    g.prim9[LF_E * N + n] = e;
    g.prim9[LF_P * N + n] = p;
    g.prim9[LF_T * N + n] = t;
    g.prim9[LF_A * N + n] = a;
    if (!(isfinite(rho) && isfinite(u) && isfinite(v) && isfinite(w) && isfinite(p))) atomicOr(g.flags, 2u);
    if (fuse_next) prep_values(g, n, jst == 2 ? 0 : jst + 1, rho, u, v, w, p);
}

}  // namespace ex
}  // namespace cfd

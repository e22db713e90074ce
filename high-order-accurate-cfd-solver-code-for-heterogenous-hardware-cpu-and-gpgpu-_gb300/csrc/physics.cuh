// physics.cuh -- device arithmetic of the RHS path, shared by the drop-in
// (reference-layout) kernels and the structured face-based kernels.
//
// Every function follows the reference kernels' formulas (cited per
// function) with gamma = 1.4 written as the reference writes it (0.4, 1.4,
// 0.2).  Functions are templated on the compute type T; the mixed-precision
// form instantiates them with float (the FP64 form uses the exact-order
// restatement in physics_exact.cuh).  Repeated divisors are inverted once.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace cfd {

// Quotient and reciprocal square root.  The float forms use the hardware
// approximations (__fdividef: about 2 ulp for |b| < 2^126; rsqrtf); other
// types compute them exactly.
template <class T> __device__ __forceinline__ T qdiv(T a, T b) { return a / b; }
template <> __device__ __forceinline__ float qdiv<float>(float a, float b) { return __fdividef(a, b); }
template <class T> __device__ __forceinline__ T qrsqrt(T x) { return T(1) / sqrt(x); }
template <> __device__ __forceinline__ float qrsqrt<float>(float x) { return rsqrtf(x); }

// Roe-averaged face state from the two adjacent nodes (U_Q.cl:60-109):
// out = {u, v, w, h, rho}.  sb/hb belong to the neighbour, si/hi to the node.
template <class T>
__device__ __forceinline__ void roe_average(T sb, T ub, T vb, T wb, T hb, T si, T ui, T vi, T wi, T hi,
                                            T out[5])
{
    const T iden = qdiv(T(1.0), sb + si);
    out[4] = sb * si;
    out[0] = (sb * ub + si * ui) * iden;
    out[1] = (sb * vb + si * vi) * iden;
    out[2] = (sb * wb + si * wi) * iden;
    out[3] = (sb * hb + si * hi) * iden;
}

// Roe eigen-system of one face (Weno.cl:337-413): k_bar = grad(zeta)/|grad(zeta)|
// from the face metric, sound speed from the Roe state, left (Lm) and right
// (R) eigenvector matrices of the Euler flux Jacobian along k_bar.
template <class T>
struct FaceEigen {
    T kx, ky, kz, a, alpha, beta, theta, phi, ru, rv, rw, rr, irr, ia2;

    __device__ __forceinline__ void init(T mx, T my, T mz, const T roe[5])
    {
        ru = roe[0];
        rv = roe[1];
        rw = roe[2];
        const T rh = roe[3];
        rr = roe[4];
        const T ikk = qrsqrt(mx * mx + my * my + mz * mz);
        a = sqrt(T(0.4) * (rh - T(0.5) * (ru * ru + rv * rv + rw * rw)));
        kx = mx * ikk;
        ky = my * ikk;
        kz = mz * ikk;
        theta = kx * ru + ky * rv + kz * rw;
        phi = T(0.5) * T(0.4) * (ru * ru + rv * rv + rw * rw);
        const T is2 = T(0.70710678118654752);  // 1/sqrt(2.0)
        const T ia = qdiv(T(1.0), a);
        irr = qdiv(T(1.0), rr);
        ia2 = ia * ia;
        alpha = rr * ia * is2;
        beta = irr * ia * is2;
    }

    // Left eigenvectors, rows of l_eigen_Q (Weno.cl:384-412).
    __device__ __forceinline__ void left(T Lm[5][5]) const
    {
        const T ph = phi * ia2;
        const T g2 = T(0.4) * ia2;
        Lm[0][0] = kx * (T(1.0) - ph) - ((kz * rv - ky * rw) * irr);
        Lm[0][1] = kx * g2 * ru;
        Lm[0][2] = (kx * g2 * rv) + (kz * irr);
        Lm[0][3] = (kx * g2 * rw) - (ky * irr);
        Lm[0][4] = -kx * g2;
        Lm[1][0] = ky * (T(1.0) - ph) - ((kx * rw - kz * ru) * irr);
        Lm[1][1] = (ky * g2 * ru) - kz * irr;
        Lm[1][2] = ky * g2 * rv;
        Lm[1][3] = (ky * g2 * rw) + (kx * irr);
        Lm[1][4] = -ky * g2;
        Lm[2][0] = kz * (T(1.0) - ph) - ((ky * ru - kx * rv) * irr);
        Lm[2][1] = kz * g2 * ru + (ky * irr);
        Lm[2][2] = kz * g2 * rv - (kx * irr);
        Lm[2][3] = kz * g2 * rw;
        Lm[2][4] = -kz * g2;
        Lm[3][0] = beta * (phi - theta * a);
        Lm[3][1] = -beta * (T(0.4) * ru - kx * a);
        Lm[3][2] = -beta * (T(0.4) * rv - ky * a);
        Lm[3][3] = -beta * (T(0.4) * rw - kz * a);
        Lm[3][4] = beta * T(0.4);
        Lm[4][0] = beta * (phi + theta * a);
        Lm[4][1] = -beta * (T(0.4) * ru + kx * a);
        Lm[4][2] = -beta * (T(0.4) * rv + ky * a);
        Lm[4][3] = -beta * (T(0.4) * rw + kz * a);
        Lm[4][4] = beta * T(0.4);
    }

};

// Branch selection of the location-code-driven first derivative of the
// Viscous kernel (Viscous.cl:285-332; the same set for eta and xi) from the
// loc codes L[0..6] of offsets -3..3.  The reference tests its branches in
// sequence and the last match wins: 1 one-sided backward, 2 one-sided
// forward, 3/4 biased next to a boundary node, 5 central; 0 = no branch
// (the derivative is 0).
__host__ __device__ __forceinline__ int visc_branch(const int L[7])
{
    const int L0 = L[3];
    int b = 0;
    if (L0 > 0 && L0 <= 52 && L[4] == 100) b = 1;
    if (L0 > 0 && L0 <= 52 && L[2] == 100) b = 2;
    if (L0 == 0 && L[4] > 0 && L[4] <= 52 && L[5] == 100) b = 3;
    if (L0 == 0 && L[2] > 0 && L[1] == 100) b = 4;
    if (L0 == 0 && L[1] != 100 && L[2] != 100 && L[5] != 100 && L[4] != 100) b = 5;
    if (L0 > 0 && L[1] != 100 && L[2] != 100 && L[5] != 100 && L[4] != 100) b = 5;
    return b;
}

// Viscous-flux derivative branches of the Weno kernel (Weno.cl:2732-2856):
// central unless a one-sided or biased branch matches.  The reference has
// no branch for a boundary node away from ghosts in a direction (its value
// is uninitialised there); the central form is used.
__host__ __device__ __forceinline__ int weno_visc_branch(const int L[7])
{
    const int L0 = L[3];
    int b = 5;
    if (L0 > 0 && L0 <= 52 && L[4] == 100) b = 1;
    if (L0 > 0 && L0 <= 52 && L[2] == 100) b = 2;
    if (L0 == 0 && L[4] > 0 && L[4] <= 52 && L[5] == 100) b = 3;
    if (L0 == 0 && L[2] > 0 && L[2] <= 52 && L[1] == 100) b = 4;
    return b;
}

// The derivative of branch b from the values f[0..6] at offsets -3..3, as
// the reference writes each formula.
template <class T>
__device__ __forceinline__ T branch_deriv(int b, const T f[7])
{
    switch (b) {
    case 1: return (T(1.0) / T(6.0)) * (T(11.0) * f[3] - T(18.0) * f[2] + T(9.0) * f[1] - T(2.0) * f[0]);
    case 2: return (T(1.0) / T(6.0)) * (T(-11.0) * f[3] + T(18.0) * f[4] - T(9.0) * f[5] + T(2.0) * f[6]);
    case 3: return (T(1.0) / T(6.0)) * (T(2.0) * f[4] + T(3.0) * f[3] - T(6.0) * f[2] + f[1]);
    case 4: return (T(1.0) / T(6.0)) * ((T(-2.0)) * f[2] - T(3.0) * f[3] + T(6.0) * f[4] - f[5]);
    case 5: return (T(1.0) / T(12.0)) * (T(8.0) * (f[4] - f[2]) - (f[5] - f[1]));
    default: return T(0.0);
    }
}

__device__ __forceinline__ double visc_deriv_ref(const double f[7], const int L[7])
{
    return branch_deriv<double>(visc_branch(L), f);
}

__device__ __forceinline__ double weno_visc_deriv_ref(const double f[7], const int L[7])
{
    return branch_deriv<double>(weno_visc_branch(L), f);
}

// Physical constants of one run.
struct Phys {
    double mach, reynolds, prandtl, t_inf, eps;
    int viscous, les;   // les: 0 none, 1 mixed time scale, 2 Smagorinsky
    double cs;          // Smagorinsky C_s
};

// Viscous and SGS fluxes at one node from the derivatives of U along the
// three directions (Viscous.cl:439-631), FMA-friendly rewrite for the
// mixed-precision form (T = float there).  dU[d][c]: derivative of U_c along
// direction d; Ui: U at the node; m: node metrics (9); det: node det;
// DEL: the filter width det^(-1/3); prim: rho,u,v,w,p of FLOW at the node;
// KS: the three MTS test-filter velocity-difference squares.  Writes
// contravariant Fv/Ev/Gv (x det) and mu.
template <class T>
__device__ __forceinline__ void viscous_node_flux(const T dU[3][5], const T Ui[5], const T m[9], T det, T DEL,
                                                  const T prim[5], const T KS[3], const Phys &P, T Fv[5], T Ev[5],
                                                  T Gv[5], T &mu_out)
{
    const T Mach = (T)P.mach, Reyl = (T)P.reynolds, Pr = (T)P.prandtl, Free_t = (T)P.t_inf;
    const T U0 = Ui[0], U1 = Ui[1], U2 = Ui[2], U3 = Ui[3], U4 = Ui[4];
    const T iU0 = qdiv(T(1.0), U0);
    const T iU00 = iU0 * iU0;
    T uc[3], vc[3], wc[3], tc[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        uc[d] = iU0 * dU[d][1] - (U1 * iU00) * dU[d][0];
        vc[d] = iU0 * dU[d][2] - (U2 * iU00) * dU[d][0];
        wc[d] = iU0 * dU[d][3] - (U3 * iU00) * dU[d][0];
    }
    const T uu = U1 * iU0, vv = U2 * iU0, ww = U3 * iU0;
#pragma unroll
    for (int d = 0; d < 3; ++d)
        tc[d] = iU0 * dU[d][4] - (U4 * iU00) * dU[d][0] - uu * uc[d] - vv * vc[d] - ww * wc[d];

    // Sutherland's law with T = gamma M^2 (gamma-1) e (Viscous.cl:451-458)
    const T d_temp = (T(1.4) * Mach * Mach * T(0.4) * ((U4 * iU0) - T(0.5) * (uu * uu + vv * vv + ww * ww)));
    const T sd = sqrt(d_temp);
    const T S = T(110.4) / Free_t;
    const T mu = (sd * sd * sd) * qdiv(T(1.0) + S, d_temp + S);
    mu_out = mu;

    const T zx = m[0], zy = m[1], zz = m[2], ex = m[3], ey = m[4], ez = m[5], xx = m[6], xy = m[7], xz = m[8];
    const T dudx = uc[0] * zx + uc[1] * ex + uc[2] * xx, dudy = uc[0] * zy + uc[1] * ey + uc[2] * xy,
            dudz = uc[0] * zz + uc[1] * ez + uc[2] * xz;
    const T dvdx = vc[0] * zx + vc[1] * ex + vc[2] * xx, dvdy = vc[0] * zy + vc[1] * ey + vc[2] * xy,
            dvdz = vc[0] * zz + vc[1] * ez + vc[2] * xz;
    const T dwdx = wc[0] * zx + wc[1] * ex + wc[2] * xx, dwdy = wc[0] * zy + wc[1] * ey + wc[2] * xy,
            dwdz = wc[0] * zz + wc[1] * ez + wc[2] * xz;
    const T dtdx = tc[0] * zx + tc[1] * ex + tc[2] * xx, dtdy = tc[0] * zy + tc[1] * ey + tc[2] * xy,
            dtdz = tc[0] * zz + tc[1] * ez + tc[2] * xz;

    const T kq = -(mu * T(1.4) * qdiv(T(1.0), Pr * Reyl));
    const T qx_ = kq * dtdx, qy_ = kq * dtdy, qz_ = kq * dtdz;   // Viscous.cl:461-463
    const T mr = mu * qdiv(T(1.0), Reyl);                                       // Viscous.cl:466-476
    const T txx = mr * (T(4.0 / 3.0) * dudx - T(2.0 / 3.0) * dvdy - T(2.0 / 3.0) * dwdz);
    const T tyy = mr * (T(4.0 / 3.0) * dvdy - T(2.0 / 3.0) * dudx - T(2.0 / 3.0) * dwdz);
    const T tzz = mr * (T(4.0 / 3.0) * dwdz - T(2.0 / 3.0) * dudx - T(2.0 / 3.0) * dvdy);
    const T sxy = dudy + dvdx, sxz = dudz + dwdx, syz = dvdz + dwdy;
    const T txy = mr * sxy, txz = mr * sxz, tyz = mr * syz;

    T TXY = 0, TYZ = 0, TXZ = 0, TXX = 0, TYY = 0, TZZ = 0, HX = 0, HY = 0, HZ = 0, DX = 0, DY = 0, DZ = 0;
    if (P.les) {  // SGS model: mixed time scale (Viscous.cl:490-558) or Smagorinsky
        const T C_MTS = T(0.03), C_T = T(10.0);
        const T s_xy = T(0.5) * sxy, s_yz = T(0.5) * syz, s_xz = T(0.5) * sxz;
        T ed[3];
        if (P.les == 2) {   // (C_s Delta)^2 |S|, |S| = sqrt(2 S_ij S_ij), Delta = det^(1/3) = 1/DEL
            const T S = sqrt(T(2.0) * (dudx * dudx + dvdy * dvdy + dwdz * dwdz)
                             + T(4.0) * (s_xy * s_xy + s_yz * s_yz + s_xz * s_xz));
            const T ls = qdiv(T(P.cs), DEL);
            ed[0] = ed[1] = ed[2] = (ls * ls) * S;
        } else {
            const T mod = sqrt(T(2.0) * ((s_xy * s_xy + s_yz * s_yz + s_xz * s_xz)
                                         + T(2.0 / 3.0) * (dudx * dudx + dvdy * dvdy + dwdz * dwdz)));
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const T sk = sqrt(KS[d]);
                if (mod != T(0.0)) {
                    const T R = qdiv(DEL * mod, sk);
                    ed[d] = qdiv(C_MTS, T(1.0) + R * (T(1.0) / C_T)) * DEL * sk;
                } else {
                    ed[d] = C_MTS * DEL * sk;
                }
            }
        }
        const T r2 = T(-2.0) * U0;
        TXY = r2 * ed[0] * s_xy;
        TYZ = r2 * ed[1] * s_yz;
        TXZ = r2 * ed[2] * s_xz;
        TXX = r2 * ed[0] * dudx;
        TYY = r2 * ed[1] * dvdy;
        TZZ = r2 * ed[2] * dwdz;
        const T kQ = -qdiv(T(1.0), T(1.4) * T(0.4) * Mach * Mach);
        const T Qx = kQ * ed[0] * dtdx, Qy = kQ * ed[1] * dtdy, Qz = kQ * ed[2] * dtdz;
        HX = Qx + (TXX + TXY + TXZ) * prim[1];
        HY = Qy + (TXY + TYY + TYZ) * prim[2];
        HZ = Qz + (TXZ + TYZ + TZZ) * prim[3];
        DX = T(0.4) * Qx;
        DY = T(0.4) * Qy;
        DZ = T(0.4) * Qz;
    }
    const T u = prim[1], v = prim[2], w = prim[3];
    // Cartesian viscous fluxes, Viscous.cl:580-596
    const T tFv[5] = {T(0), -txx + TXX, -txy + TXY, -txz + TXZ, ((-u * txx - v * txy - w * txz) + qx_ + HX + DX)};
    const T tEv[5] = {T(0), -txy + TXY, -tyy + TYY, -tyz + TYZ, ((-u * txy - v * tyy - w * tyz) + qy_ + HY + DY)};
    const T tGv[5] = {T(0), -txz + TXZ, -tyz + TYZ, -tzz + TZZ, ((-u * txz - v * tyz - w * tzz) + qz_ + HZ + DZ)};
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        Fv[c] = det * (zx * tFv[c] + zy * tEv[c] + zz * tGv[c]);
        Ev[c] = det * (ex * tFv[c] + ey * tEv[c] + ez * tGv[c]);
        Gv[c] = det * (xx * tFv[c] + xy * tEv[c] + xz * tGv[c]);
    }
}

// Contravariant node inviscid fluxes F, E, G (x det) from the primitives,
// Viscous.cl:560-578 and 615-631 (FMA-friendly, mixed form).
template <class T>
__device__ __forceinline__ void node_inviscid_flux(const T prim[5], const T m[9], T det, T F[5], T E[5], T G[5])
{
    const T rho = prim[0], u = prim[1], v = prim[2], w = prim[3], p = prim[4];
    const T Et = (p * T(2.5) + T(0.5) * rho * (u * u + v * v + w * w)) + p;
    const T tF[5] = {rho * u, rho * u * u + p, rho * v * u, rho * u * w, Et * u};
    const T tE[5] = {rho * v, rho * v * u, rho * v * v + p, rho * v * w, Et * v};
    const T tG[5] = {rho * w, rho * u * w, rho * v * w, rho * w * w + p, Et * w};
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        F[c] = det * (m[0] * tF[c] + m[1] * tE[c] + m[2] * tG[c]);
        E[c] = det * (m[3] * tF[c] + m[4] * tE[c] + m[5] * tG[c]);
        G[c] = det * (m[6] * tF[c] + m[7] * tE[c] + m[8] * tG[c]);
    }
}

}  // namespace cfd

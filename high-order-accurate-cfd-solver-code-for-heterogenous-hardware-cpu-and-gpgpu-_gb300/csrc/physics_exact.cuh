// physics_exact.cuh -- FP64 device arithmetic in the reference's own
// evaluation order.
//
// The reference's right-hand side at low Mach number is a small difference
// of large pressure fluxes: re-associating one sum or contracting a*b+c into
// an FMA moves L by 1e-12 .. 1e-11 (relative L2) on the Taylor-Green case.
// The FP64 path therefore evaluates every expression exactly as the
// reference kernels write it (same operand order, same divisions, no
// algebraic rewriting) and the translation units that include this header
// are compiled with --fmad=false.  With IEEE-correct division and square
// root on the GPU this reproduces the reference's results to the last bit
// except where libm functions differ (cbrt).  Divisions that share a divisor
// use one reciprocal and an exactly checked correction (exact_div.cuh,
// `Over`), and the reciprocals, the corrections and the single divisions
// decide their rounding from exact integer remainders: the same bits as the
// division, with most of the work moved from the FP64 pipe (two operations
// per clock per SM on GB300) to the integer pipes.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "exact_div.cuh"

namespace cfd {
namespace ex {

__device__ __forceinline__ double sq(double x) { return x * x; }

// Division of several numerators by one divisor b: Over<true>(b)(x) == x / b,
// bit for bit, with the reciprocal computed once (exact_div.cuh);
// Over<false> divides each numerator (the same bits; faster where the
// kernel's occupancy hides the division latency, e.g. the batched form).
template <bool SHARED>
struct Over;

template <>
struct Over<true> {
    double b, y;
    __device__ __forceinline__ explicit Over(double divisor) : b(divisor), y(xdiv::rcp(divisor)) {}
    __device__ __forceinline__ double operator()(double x) const { return xdiv::div(x, b, y); }
};

template <>
struct Over<false> {
    double b;
    __device__ __forceinline__ explicit Over(double divisor) : b(divisor) {}
    __device__ __forceinline__ double operator()(double x) const { return x / b; }
};

// a / b with the same bits: xdiv::divide (reciprocal and quotient rounding
// on the integer pipe) when CFD_EXACT_DIVIDE is set (the default), else the
// division.
#ifndef CFD_EXACT_DIVIDE
#define CFD_EXACT_DIVIDE 1
#endif
__device__ __forceinline__ double dv(double a, double b) { return CFD_EXACT_DIVIDE ? xdiv::divide(a, b) : a / b; }

// U_Q.cl:64-65
__device__ __forceinline__ double enthalpy(double rho, double u, double v, double w, double p)
{
    return dv((dv(p, 0.4) + xdiv::scale2<-1>(rho) * (u * u + v * v + w * w) + p), rho);
}

// U_Q.cl:60-109 for one face: {u, v, w, h, rho}; (sb,...) the neighbour.
template <bool SD = true>
__device__ __forceinline__ void roe(double sb, double ub, double vb, double wb, double hb, double si, double ui,
                                    double vi, double wi, double hi, double r[5])
{
    r[4] = sb * si;
    const Over<SD> d(sb + si);
    r[0] = d(sb * ub + si * ui);
    r[1] = d(sb * vb + si * vi);
    r[2] = d(sb * wb + si * wi);
    r[3] = d(sb * hb + si * hi);
}

// WENO5 pair, Weno.cl:1056-1280; c[0..5] = left-2 .. right+2.
template <bool SD = true>
__device__ __forceinline__ void weno_pair(const double cc[6], double eps, double &pos, double &neg)
{
    const double *c = cc + 2;   // c[0] = left node of the face
    // products by 2, 4, 1/4 and 1/8 on the integer pipe (xdiv::scale2,
    // the same bits as the multiplies)
    using xdiv::scale2;
    const double p0 = (15.0 / 8.0) * c[1] - (5.0 / 4.0) * c[2] + (3.0 / 8.0) * c[3];
    const double p1 = (3.0 / 8.0) * c[0] + (3.0 / 4.0) * c[1] - scale2<-3>(c[2]);
    const double p2 = -scale2<-3>(c[-1]) + (3.0 / 4.0) * c[0] + (3.0 / 8.0) * c[1];
    const double m0 = p1;
    const double m1 = p2;
    const double m2 = (3.0 / 8.0) * c[-2] - (5.0 / 4.0) * c[-1] + (15.0 / 8.0) * c[0];
    const double ISm2 = (13.0 / 12.0) * (sq(c[-2] - scale2<1>(c[-1]) + c[0])) + scale2<-2>(sq(c[-2] - scale2<2>(c[-1]) + 3.0 * c[0]));
    const double ISm1 = (13.0 / 12.0) * (sq(c[-1] - scale2<1>(c[0]) + c[1])) + scale2<-2>(sq(c[-1] - c[1]));
    const double ISm0 = (13.0 / 12.0) * (sq(c[0] - scale2<1>(c[1]) + c[2])) + scale2<-2>(sq(3.0 * c[0] - scale2<2>(c[1]) + c[2]));
    const double ISp2 = (13.0 / 12.0) * (sq(c[-1] - scale2<1>(c[0]) + c[1])) + scale2<-2>(sq(c[-1] - scale2<2>(c[0]) + 3.0 * c[1]));
    const double ISp1 = (13.0 / 12.0) * (sq(c[0] - scale2<1>(c[1]) + c[2])) + scale2<-2>(sq(c[0] - c[2]));
    const double ISp0 = (13.0 / 12.0) * (sq(c[1] - scale2<1>(c[2]) + c[3])) + scale2<-2>(sq(3.0 * c[1] - scale2<2>(c[2]) + c[3]));
    const double wp0 = xdiv::pow2_over<-4>(sq(eps + (ISp0)));   // (1/16) / ...
    const double wp1 = dv(5.0 / 8.0, sq(eps + (ISp1)));
    const double wp2 = dv(5.0 / 16.0, sq(eps + (ISp2)));
    const double wm0 = dv(5.0 / 16.0, sq(eps + (ISm0)));
    const double wm1 = dv(5.0 / 8.0, sq(eps + (ISm1)));
    const double wm2 = xdiv::pow2_over<-4>(sq(eps + (ISm2)));   // (1/16) / ...
    const Over<SD> sp(wp0 + wp1 + wp2), sm(wm0 + wm1 + wm2);
    const double Wp0 = sp(wp0), Wp1 = sp(wp1), Wp2 = sp(wp2);
    const double Wm0 = sm(wm0), Wm1 = sm(wm1), Wm2 = sm(wm2);
    pos = Wp0 * p0 + Wp1 * p1 + Wp2 * p2;
    neg = Wm0 * m0 + Wm1 * m1 + Wm2 * m2;
}

// The quotients by rho of a face state q (conservative) that its Cartesian
// fluxes and lambda_5 divide by q[0]: q1^2/q0, q2^2/q0, q3^2/q0,
// q1 q2/q0, q1 q3/q0, q2 q3/q0, q1/q0, q2/q0, q3/q0, q4/q0.
struct StateQuot {
    double k1, k2, k3, e12, e13, e23, v1, v2, v3, v4;
};

template <bool SD = true>
__device__ __forceinline__ StateQuot state_quot(const double q[5])
{
    const Over<SD> d(q[0]);
    StateQuot t;
    t.k1 = d(q[1] * q[1]);
    t.k2 = d(q[2] * q[2]);
    t.k3 = d(q[3] * q[3]);
    t.e12 = d(q[1] * q[2]);
    t.e13 = d(q[1] * q[3]);
    t.e23 = d(q[2] * q[3]);
    t.v1 = d(q[1]);
    t.v2 = d(q[2]);
    t.v3 = d(q[3]);
    t.v4 = d(q[4]);
    return t;
}

// Cartesian Euler fluxes of a face state, Weno.cl:2291-2507.
__device__ __forceinline__ void cart_flux(const double q[5], const StateQuot &t, double F[5], double E[5], double G[5])
{
    const double k1 = t.k1, k2 = t.k2, k3 = t.k3;
    const double pr = 0.4 * (q[4] - xdiv::scale2<-1>(k1 + k2 + k3));
    const double hq = (1.4 * q[4] - 0.2 * (k1 + k2 + k3));
    F[0] = q[1];
    F[1] = k1 + pr;
    F[2] = t.e12;
    F[3] = t.e13;
    F[4] = hq * t.v1;
    E[0] = q[2];
    E[1] = t.e12;
    E[2] = k2 + pr;
    E[3] = t.e23;
    E[4] = hq * t.v2;
    G[0] = q[3];
    G[1] = t.e13;
    G[2] = t.e23;
    G[3] = k3 + pr;
    G[4] = hq * t.v3;
}

// lambda_5 of a face state, Weno.cl:2511-2583 element [4].
__device__ __forceinline__ double lambda5(const double q[5], const StateQuot &t, double mx, double my, double mz)
{
    return (mx * t.v1 + my * t.v2 + mz * t.v3)
           + sqrt(1.4 * 0.4 * (t.v4 - dv(q[1] * q[1] + q[2] * q[2] + q[3] * q[3], xdiv::scale2<1>(q[0] * q[0])))
                  * (mx * mx + my * my + mz * mz));
}

// LLF face flux of one face (Weno.cl:336-2947): Roe eigenvectors from the
// face metric and Roe state r = {u,v,w,h,rho}, projection of the six stencil
// points pts (left-2 .. right+2), WENO5, back-projection, contravariant
// fluxes x face det, lambda_5 LLF.
template <bool SD = true>
__device__ __forceinline__ void face_flux(const double pts[6][5], double mx, double my, double mz, double DET_F,
                                          const double r[5], double eps, double Fhat[5])
{
    const double ru = r[0], rv = r[1], rw = r[2], rh = r[3], rrho = r[4];
    const double kk = sqrt(mx * mx + my * my + mz * mz);
    const double a = sqrt(0.4 * (rh - xdiv::scale2<-1>(ru * ru + rv * rv + rw * rw)));
    const Over<SD> dk(kk);
    const double kx = dk(mx), ky = dk(my), kz = dk(mz);
    const double theta = kx * ru + ky * rv + kz * rw;
    const double phi_sq = 0.5 * 0.4 * (ru * ru + rv * rv + rw * rw);
    const double alpha = dv(rrho, sqrt(2.0) * a);
    const double beta = dv(1.0, sqrt(2.0) * rrho * a);
    double cpos[5], cneg[5];
    {
        const Over<SD> da(a * a), dr(rrho);
        const double f = da(phi_sq);
        const double Lm[5][5] = {
            {kx * (1.0 - f) - dr(kz * rv - ky * rw), da(kx * 0.4 * ru), da(kx * 0.4 * rv) + dr(kz),
             da(kx * 0.4 * rw) - dr(ky), da(-kx * 0.4)},
            {ky * (1.0 - f) - dr(kx * rw - kz * ru), da(ky * 0.4 * ru) - dr(kz), da(ky * 0.4 * rv),
             da(ky * 0.4 * rw) + dr(kx), da(-ky * 0.4)},
            {kz * (1.0 - f) - dr(ky * ru - kx * rv), da(kz * 0.4 * ru) + dr(ky), da(kz * 0.4 * rv) - dr(kx),
             da(kz * 0.4 * rw), da(-kz * 0.4)},
            {beta * (phi_sq - theta * a), -beta * (0.4 * ru - kx * a), -beta * (0.4 * rv - ky * a),
             -beta * (0.4 * rw - kz * a), beta * 0.4},
            {beta * (phi_sq + theta * a), -beta * (0.4 * ru + kx * a), -beta * (0.4 * rv + ky * a),
             -beta * (0.4 * rw + kz * a), beta * 0.4}};
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            double cv[6];
#pragma unroll
            for (int o = 0; o < 6; ++o)
                cv[o] = Lm[q][0] * pts[o][0] + Lm[q][1] * pts[o][1] + Lm[q][2] * pts[o][2] + Lm[q][3] * pts[o][3]
                        + Lm[q][4] * pts[o][4];
            weno_pair<SD>(cv, eps, cpos[q], cneg[q]);
        }
    }
    double qp[5], qn[5];
    {
        const Over<SD> d4(0.4);
        const double R[5][5] = {
            {kx, ky, kz, alpha, alpha},
            {kx * ru, ky * ru - kz * rrho, kz * ru + ky * rrho, alpha * (ru + kx * a), alpha * (ru - kx * a)},
            {kx * rv + kz * rrho, ky * rv, kz * rv - kx * rrho, alpha * (rv + ky * a), alpha * (rv - ky * a)},
            {kx * rw - ky * rrho, ky * rw + kx * rrho, kz * rw, alpha * (rw + kz * a), alpha * (rw - kz * a)},
            {d4(kx * phi_sq) + rrho * (kz * rv - ky * rw), d4(ky * phi_sq) + rrho * (kx * rw - kz * ru),
             d4(kz * phi_sq) + rrho * (ky * ru - kx * rv), alpha * (d4(phi_sq + a * a) + theta * a),
             alpha * (d4(phi_sq + a * a) - theta * a)}};
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            qp[q] = R[q][0] * (cpos[0]) + R[q][1] * (cpos[1]) + R[q][2] * (cpos[2]) + R[q][3] * (cpos[3])
                    + R[q][4] * (cpos[4]);
            qn[q] = R[q][0] * (cneg[0]) + R[q][1] * (cneg[1]) + R[q][2] * (cneg[2]) + R[q][3] * (cneg[3])
                    + R[q][4] * (cneg[4]);
        }
    }
    const StateQuot tp = state_quot<SD>(qp), tn = state_quot<SD>(qn);
    const double lp = lambda5(qp, tp, mx, my, mz);
    const double ln = lambda5(qn, tn, mx, my, mz);
    double al = __longlong_as_double(0x7ff8000000000000ULL);   // NaN when neither branch holds (NaN input)
    if (fabs(lp) >= fabs(ln)) al = fabs(lp);
    else if (fabs(ln) >= fabs(lp)) al = fabs(ln);
    double Fp[5], Ep[5], Gp[5];
    cart_flux(qp, tp, Fp, Ep, Gp);
    double Fn[5], En[5], Gn[5];
    cart_flux(qn, tn, Fn, En, Gn);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        const double fcp = DET_F * (mx * Fp[c] + my * Ep[c] + mz * Gp[c]);
        const double fcn = DET_F * (mx * Fn[c] + my * En[c] + mz * Gn[c]);
        const double qpd = DET_F * qp[c], qnd = DET_F * qn[c];
        Fhat[c] = xdiv::scale2<-1>(fcp + fcn - al * (qpd - qnd));
    }
}

// Corrected face flux Fhat - d2/24 + 7 d4/5760, Weno.cl:2950-3058, for the
// face between f[2] and f[3] (f[0..5] = left-2 .. right+2).
__device__ __forceinline__ double corrected(double Fhat, const double f[6])
{
    const double d2 = (1.0 / 48.0) * (-5.0 * f[0] + 39.0 * f[1] - 34.0 * f[2] - 34.0 * f[3] + 39.0 * f[4] - 5.0 * f[5]);
    const double d4 = xdiv::scale2<-1>(f[0] - 3.0 * f[1] + xdiv::scale2<1>(f[2]) + xdiv::scale2<1>(f[3]) - 3.0 * f[4] + f[5]);
    return Fhat - (1.0 / 24.0) * d2 + (7.0 / 5760.0) * d4;
}

// Fourth-order central first derivative (Viscous.cl:325-332 and the loc==0
// branch of Weno.cl:2771-2778); f[0..4] = offsets -2..2.
__device__ __forceinline__ double central4(double fm2, double fm1, double fp1, double fp2)
{
    return (1.0 / 12.0) * (xdiv::scale2<3>(fp1 - fm1) - (fp2 - fm2));   // 8 (...) on the integer pipe, same bits
}

struct Visc {
    double mach, reynolds, prandtl, t_inf;
    int les;       // 0 none, 1 mixed time scale, 2 Smagorinsky
    double cs;     // Smagorinsky C_s
};

// Viscous.cl:439-631 at one node, in the reference's order.  dU[d][c],
// Ui[5], node metrics m[9], det, FLOW primitives (rho,u,v,w,p), the three
// MTS KS values.  Writes the contravariant viscous fluxes Fv,Ev,Gv and mu
// (the inviscid node fluxes come from node_inviscid_flux).
__device__ __forceinline__ void viscous_node(const double dU[3][5], const double Ui[5], const double m[9], double DET_I,
                                             const double prim[5], const double KSv[3], const Visc &P, double Fv[5],
                                             double Ev[5], double Gv[5], double &mu_out)
{
    const double Mach = P.mach, Reyl = P.reynolds, Pr = P.prandtl, Free_t = P.t_inf;
    const double zeta_x = m[0], zeta_y = m[1], zeta_z = m[2], eta_x = m[3], eta_y = m[4], eta_z = m[5];
    const double xi_x = m[6], xi_y = m[7], xi_z = m[8];
    const double U0_I = Ui[0], U1_I = Ui[1], U2_I = Ui[2], U3_I = Ui[3], U4_I = Ui[4];
    // the divisions by U0 and by U0^2 share their reciprocals (Over: the
    // same bits as each division)
    const Over<true> o1(U0_I), o2(U0_I * U0_I);
    const double r0 = o1(1.0), a1 = o2(U1_I), a2 = o2(U2_I), a3 = o2(U3_I), a4 = o2(U4_I);
    double uc[3], vc[3], wc[3], tc[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        uc[d] = r0 * (dU[d][1]) - a1 * (dU[d][0]);
        vc[d] = r0 * (dU[d][2]) - a2 * (dU[d][0]);
        wc[d] = r0 * (dU[d][3]) - a3 * (dU[d][0]);
    }
    const double v1 = o1(U1_I), v2 = o1(U2_I), v3 = o1(U3_I);
#pragma unroll
    for (int d = 0; d < 3; ++d)
        tc[d] = r0 * (dU[d][4]) - a4 * (dU[d][0]) - v1 * uc[d] - v2 * vc[d] - v3 * wc[d];
    const double d_temp = (1.4 * Mach * Mach * 0.4
                           * (o1(U4_I) - xdiv::scale2<-1>(o2(U1_I * U1_I) + o2(U2_I * U2_I) + o2(U3_I * U3_I))));
    const double d_temp1 = sqrt(d_temp) * sqrt(d_temp) * sqrt(d_temp);
    const double st = dv(110.4, Free_t);
    const double mu = (d_temp1) * dv(1.0 + st, d_temp + st);
    mu_out = mu;
#define GX(a) ((a)[0] * zeta_x + (a)[1] * eta_x + (a)[2] * xi_x)
#define GY(a) ((a)[0] * zeta_y + (a)[1] * eta_y + (a)[2] * xi_y)
#define GZ(a) ((a)[0] * zeta_z + (a)[1] * eta_z + (a)[2] * xi_z)
    const double kq = dv(mu * 1.4, Pr * Reyl), mr = dv(mu, Reyl);
    const double qz = (-1.0) * kq * GX(tc);
    const double qe = (-1.0) * kq * GY(tc);
    const double qx = (-1.0) * kq * GZ(tc);
    const double tauzz = mr * ((4.0 / 3.0) * GX(uc) - (2.0 / 3.0) * GY(vc) - (2.0 / 3.0) * GZ(wc));
    const double tauee = mr * ((4.0 / 3.0) * GY(vc) - (2.0 / 3.0) * GX(uc) - (2.0 / 3.0) * GZ(wc));
    const double tauxx = mr * ((4.0 / 3.0) * GZ(wc) - (2.0 / 3.0) * GX(uc) - (2.0 / 3.0) * GY(vc));
    const double s_xy = uc[0] * zeta_y + uc[1] * eta_y + uc[2] * xi_y + vc[0] * zeta_x + vc[1] * eta_x + vc[2] * xi_x;
    const double s_xz = uc[0] * zeta_z + uc[1] * eta_z + uc[2] * xi_z + wc[0] * zeta_x + wc[1] * eta_x + wc[2] * xi_x;
    const double s_yz = vc[0] * zeta_z + vc[1] * eta_z + vc[2] * xi_z + wc[0] * zeta_y + wc[1] * eta_y + wc[2] * xi_y;
    const double tauze = mr * s_xy;
    const double tauzx = mr * s_xz;
    const double tauex = mr * s_yz;
    double TAU_XY = 0, TAU_YZ = 0, TAU_XZ = 0, TAU_XX = 0, TAU_YY = 0, TAU_ZZ = 0;
    double H_X = 0, H_Y = 0, H_Z = 0, D_X = 0, D_Y = 0, D_Z = 0;
    const double u = prim[1], v = prim[2], w = prim[3];
    if (P.les) {
        const double C_MTS = 0.03, C_T = 10.0;
        using xdiv::scale2;   // products by powers of two on the integer pipe, same bits
        const double stress_yz = (scale2<-1>(vc[0] * zeta_z + vc[1] * eta_z + vc[2] * xi_z + wc[0] * zeta_y + wc[1] * eta_y + wc[2] * xi_y));
        const double stress_xz = (scale2<-1>(wc[0] * zeta_x + wc[1] * eta_x + wc[2] * xi_x + uc[0] * zeta_z + uc[1] * eta_z + uc[2] * xi_z));
        const double stress_xy = (scale2<-1>(s_xy));
        const double stress_xx = GX(uc), stress_yy = GY(vc), stress_zz = GZ(wc);
        const double mod_stress = sqrt(scale2<1>((stress_xy * stress_xy + stress_yz * stress_yz + stress_xz * stress_xz)
                                              + (2.0 / 3.0) * (stress_xx * stress_xx + stress_yy * stress_yy + stress_zz * stress_zz)));
        const double DEL = dv(1.0, cbrt(DET_I));
        double EDDY_x, EDDY_y, EDDY_z;
        if (P.les == 2) {
            // Smagorinsky (no counterpart in the reference): (C_s Delta)^2 |S|,
            // |S| = sqrt(2 S_ij S_ij), Delta = det^(1/3) (the cell size; det is
            // the cell volume), in the reference's SGS terms below
            const double S = sqrt(scale2<1>(stress_xx * stress_xx + stress_yy * stress_yy + stress_zz * stress_zz)
                                  + scale2<2>(stress_xy * stress_xy + stress_yz * stress_yz + stress_xz * stress_xz));
            const double ls = P.cs * cbrt(DET_I);
            EDDY_x = EDDY_y = EDDY_z = (ls * ls) * S;
        } else if (mod_stress != 0.0) {
            const double Rx = dv(DEL * (mod_stress), sqrt(KSv[0]));
            const double Ry = dv(DEL * (mod_stress), sqrt(KSv[1]));
            const double Rz = dv(DEL * (mod_stress), sqrt(KSv[2]));
            const Over<true> oct(C_T);
            EDDY_x = dv(C_MTS, 1.0 + oct(1.0 * Rx)) * DEL * sqrt(KSv[0]);
            EDDY_y = dv(C_MTS, 1.0 + oct(1.0 * Ry)) * DEL * sqrt(KSv[1]);
            EDDY_z = dv(C_MTS, 1.0 + oct(1.0 * Rz)) * DEL * sqrt(KSv[2]);
        } else {
            EDDY_x = (C_MTS) * DEL * sqrt(KSv[0]);
            EDDY_y = (C_MTS) * DEL * sqrt(KSv[1]);
            EDDY_z = (C_MTS) * DEL * sqrt(KSv[2]);
        }
        const double m2U0 = -scale2<1>(U0_I);   // -2.0 * U0_I
        TAU_XY = m2U0 * EDDY_x * (stress_xy);
        TAU_YZ = m2U0 * EDDY_y * (stress_yz);
        TAU_XZ = m2U0 * EDDY_z * (stress_xz);
        TAU_XX = m2U0 * EDDY_x * stress_xx;
        TAU_YY = m2U0 * EDDY_y * stress_yy;
        TAU_ZZ = m2U0 * EDDY_z * stress_zz;
        const double ck = dv(1.0, 1.4 * 0.4 * Mach * Mach);
        const double Q_x = ck * (-1.0) * (EDDY_x) * GX(tc);
        const double Q_y = ck * (-1.0) * (EDDY_y) * GY(tc);
        const double Q_z = ck * (-1.0) * (EDDY_z) * GZ(tc);
        H_X = Q_x + (TAU_XX * u + TAU_XY * u + TAU_XZ * u);
        H_Y = Q_y + (TAU_XY * v + TAU_YY * v + TAU_YZ * v);
        H_Z = Q_z + (TAU_XZ * w + TAU_YZ * w + TAU_ZZ * w);
        D_X = 0.4 * Q_x;
        D_Y = 0.4 * Q_y;
        D_Z = 0.4 * Q_z;
    }
#undef GX
#undef GY
#undef GZ
    const double tFv[5] = {0.0, (-1.0) * tauzz + TAU_XX, (-1.0) * tauze + TAU_XY, (-1.0) * tauzx + TAU_XZ,
                           (((-1.0) * u * tauzz - v * tauze - w * tauzx) + qz + H_X + D_X)};
    const double tEv[5] = {0.0, (-1.0) * tauze + TAU_XY, (-1.0) * tauee + TAU_YY, (-1.0) * tauex + TAU_YZ,
                           (((-1.0) * u * tauze - v * tauee - w * tauex) + qe + H_Y + D_Y)};
    const double tGv[5] = {0.0, (-1.0) * tauzx + TAU_XZ, (-1.0) * tauex + TAU_YZ, (-1.0) * tauxx + TAU_ZZ,
                           (((-1.0) * u * tauzx - v * tauex - w * tauxx) + qx + H_Z + D_Z)};
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        Fv[c] = DET_I * (zeta_x * tFv[c] + zeta_y * tEv[c] + zeta_z * tGv[c]);
        Ev[c] = DET_I * (eta_x * tFv[c] + eta_y * tEv[c] + eta_z * tGv[c]);
        Gv[c] = DET_I * (xi_x * tFv[c] + xi_y * tEv[c] + xi_z * tGv[c]);
    }
}

// Contravariant inviscid node fluxes F, E, G (x det) from the primitives
// (rho,u,v,w,p), Viscous.cl:560-578 and 615-631.
__device__ __forceinline__ void node_flux(const double prim[5], const double m[9], double DET_I, double F[5],
                                          double E[5], double G[5])
{
    const double rho = prim[0], u = prim[1], v = prim[2], w = prim[3], p = prim[4];
    const double Et = ((dv(p, 0.4) + xdiv::scale2<-1>(rho) * (u * u + v * v + w * w)) + p);
    const double tF[5] = {rho * u, rho * u * u + p, rho * v * u, rho * u * w, Et * u};
    const double tE[5] = {rho * v, rho * v * u, rho * v * v + p, rho * v * w, Et * v};
    const double tG[5] = {rho * w, rho * u * w, rho * v * w, rho * w * w + p, Et * w};
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        F[c] = DET_I * (m[0] * tF[c] + m[1] * tE[c] + m[2] * tG[c]);
        E[c] = DET_I * (m[3] * tF[c] + m[4] * tE[c] + m[5] * tG[c]);
        G[c] = DET_I * (m[6] * tF[c] + m[7] * tE[c] + m[8] * tG[c]);
    }
}

// MTS test-filter velocity difference squared (Viscous.cl:493-495) for the
// velocity component c along its own direction.
__device__ __forceinline__ double ks(double Uc_i, double U0_i, double Uc_m, double U0_m, double Uc_p, double U0_p)
{
    using xdiv::scale2;   // 0.25 * x and 0.5 * x on the integer pipe, same bits
    return sq((dv(Uc_i, U0_i) - dv(scale2<-2>(Uc_m) + scale2<-1>(Uc_i) + scale2<-2>(Uc_p),
                                   scale2<-2>(U0_m) + scale2<-1>(U0_i) + scale2<-2>(U0_p))));
}

// Sutherland viscosity from U only (Viscous.cl:451-458).
__device__ __forceinline__ double mu_of(const double Ui[5], double Mach, double Free_t)
{
    const double U0_I = Ui[0], U1_I = Ui[1], U2_I = Ui[2], U3_I = Ui[3], U4_I = Ui[4];
    const Over<true> o2(U0_I * U0_I);
    const double d_temp = (1.4 * Mach * Mach * 0.4
                           * (dv(U4_I, U0_I) - xdiv::scale2<-1>(o2(U1_I * U1_I) + o2(U2_I * U2_I) + o2(U3_I * U3_I))));
    const double d_temp1 = sqrt(d_temp) * sqrt(d_temp) * sqrt(d_temp);
    const double st = dv(110.4, Free_t);
    return (d_temp1) * dv(1.0 + st, d_temp + st);
}

// SSP-RK3 stage j and primitive recovery (Weno.cl:3084-3135).  Returns the
// new U in Un and writes FLOW fields rho,u,v,w,e,p,t,a into fo[9]
// (u,v,w,p,t,rho,mu,a,e order; mu untouched).
__device__ __forceinline__ void rk_and_primitives(int j, double del_t, double mach, double det, const double U0[5],
                                                  const double U1[5], const double U2[5], const double L[5],
                                                  double Un[5], double &rho, double &u, double &v, double &w,
                                                  double &e, double &p, double &t, double &a_)
{
    if (j == 0) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Un[c] = U0[c] + del_t * L[c];
    } else if (j == 1) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Un[c] = (3.0 / 4.0) * U0[c] + (1.0 / 4.0) * U1[c] + 0.25 * del_t * L[c];
    } else {
        const Over<true> d3(3.0);
#pragma unroll
        for (int c = 0; c < 5; ++c) Un[c] = d3(U0[c]) + ((2.0 / 3.0) * U2[c]) + (2.0 / 3.0) * (del_t * L[c]);
    }
    double fu[5];
    const double idet = dv(1.0, det);
#pragma unroll
    for (int c = 0; c < 5; ++c) fu[c] = idet * Un[c];
    rho = fu[0];
    const Over<true> d0(fu[0]);   // u, v, w, e share the divisor rho
    u = d0(fu[1]);
    v = d0(fu[2]);
    w = d0(fu[3]);
    e = d0(fu[4]) - xdiv::scale2<-1>(u * u + v * v + w * w);
    p = e * rho * 0.4;
    const Over<true> dr(rho);
    t = (1.4 * mach * mach) * dr(p);
    a_ = sqrt(dr(1.4 * p));
}

}  // namespace ex
}  // namespace cfd

// physics_x2.cuh -- the mixed form's LLF face flux on paired FP32 lanes.
//
// Blackwell issues two FP32 operations per packed instruction (__ffma2_rn,
// __fmul2_rn, __fadd2_rn).  The face flux pairs naturally:
//   * the characteristic projection of stencil point k is paired with that
//     of point 5-k;
//   * WENO5's left-biased ("neg") value is its right-biased ("pos") formula
//     applied to the reversed stencil, so lane x (stencil) and lane y
//     (reversed stencil) of one evaluation give pos and neg;
//   * the back-projection, the contravariant fluxes and the LLF split run on
//     the (pos, neg) pair.
// The formulas follow the reference's Weno kernel (Weno.cl:337-413 eigen
// system, 1056-1280 WENO5, 2188-2583 back-projection and fluxes, 2859-3058
// LLF and the sixth-order correction); only the lane packing is new.
#pragma once

#include "emu64.cuh"
#include "physics.cuh"

namespace cfd {
namespace x2 {

__device__ __forceinline__ float2 b2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, b2(-1.0f), a); }
__device__ __forceinline__ float2 swap2(float2 a) { return make_float2(a.y, a.x); }
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(__fdividef(1.0f, a.x), __fdividef(1.0f, a.y)); }

// Jiang-Shu smoothness indicator of a three-point stencil from its two
// differences t (second) and u (first-derivative form): 13/12 t^2 + 1/4 u^2
__device__ __forceinline__ float2 smooth2(float2 t, float2 u)
{
    return fma2(mul2(b2(13.0f / 12.0f), t), t, mul2(mul2(b2(0.25f), u), u));
}

// Right-biased WENO5 value at the face between c[2] and c[3] of the six
// points c[0..5] (candidates 15/8,-5/4,3/8 | 3/8,3/4,-1/8 | -1/8,3/4,3/8,
// linear weights 1/16, 5/8, 5/16, w_k = d_k/(eps+IS_k)^2), on both lanes.
__device__ __forceinline__ float2 weno5_pos2(const float2 c[6], float eps)
{
    const float2 cm1 = c[1], c0 = c[2], c1 = c[3], c2 = c[4], c3 = c[5];
    const float2 p0 = fma2(b2(15.0f / 8.0f), c1, fma2(b2(-5.0f / 4.0f), c2, mul2(b2(3.0f / 8.0f), c3)));
    const float2 p1 = fma2(b2(3.0f / 8.0f), c0, fma2(b2(3.0f / 4.0f), c1, mul2(b2(-1.0f / 8.0f), c2)));
    const float2 p2 = fma2(b2(-1.0f / 8.0f), cm1, fma2(b2(3.0f / 4.0f), c0, mul2(b2(3.0f / 8.0f), c1)));
    const float2 IS0 = smooth2(fma2(b2(-2.0f), c2, add2(c1, c3)), fma2(b2(3.0f), c1, fma2(b2(-4.0f), c2, c3)));
    const float2 IS1 = smooth2(fma2(b2(-2.0f), c1, add2(c0, c2)), sub2(c0, c2));
    const float2 IS2 = smooth2(fma2(b2(-2.0f), c0, add2(cm1, c1)), fma2(b2(3.0f), c1, fma2(b2(-4.0f), c0, cm1)));
    const float2 e0 = add2(b2(eps), IS0), e1 = add2(b2(eps), IS1), e2 = add2(b2(eps), IS2);
    const float2 w0 = mul2(b2(1.0f / 16.0f), rcp2(mul2(e0, e0)));
    const float2 w1 = mul2(b2(5.0f / 8.0f), rcp2(mul2(e1, e1)));
    const float2 w2 = mul2(b2(5.0f / 16.0f), rcp2(mul2(e2, e2)));
    const float2 num = fma2(w0, p0, fma2(w1, p1, mul2(w2, p2)));
    return mul2(num, rcp2(add2(add2(w0, w1), w2)));
}

// q = R c on both lanes (R: right eigenvectors of the face, Weno.cl:349-380)
__device__ __forceinline__ void right_times2(const FaceEigen<float> &eg, const float2 c[5], float2 q[5])
{
    const float kx = eg.kx, ky = eg.ky, kz = eg.kz, al = eg.alpha, a = eg.a, ru = eg.ru, rv = eg.rv, rw = eg.rw,
                rr = eg.rr, th = eg.theta;
    const float e0 = (eg.phi + a * a) * 2.5f, ph5 = eg.phi * 2.5f;
    const float2 s34 = add2(c[3], c[4]), d34 = sub2(c[3], c[4]);
    q[0] = fma2(b2(kx), c[0], fma2(b2(ky), c[1], fma2(b2(kz), c[2], mul2(b2(al), s34))));
    // alpha (ru + kx a) c3 + alpha (ru - kx a) c4 = alpha ru (c3 + c4) + alpha kx a (c3 - c4)
    q[1] = fma2(b2(kx * ru), c[0], fma2(b2(ky * ru - kz * rr), c[1], fma2(b2(kz * ru + ky * rr), c[2],
                fma2(b2(al * ru), s34, mul2(b2(al * kx * a), d34)))));
    q[2] = fma2(b2(kx * rv + kz * rr), c[0], fma2(b2(ky * rv), c[1], fma2(b2(kz * rv - kx * rr), c[2],
                fma2(b2(al * rv), s34, mul2(b2(al * ky * a), d34)))));
    q[3] = fma2(b2(kx * rw - ky * rr), c[0], fma2(b2(ky * rw + kx * rr), c[1], fma2(b2(kz * rw), c[2],
                fma2(b2(al * rw), s34, mul2(b2(al * kz * a), d34)))));
    q[4] = fma2(b2(kx * ph5 + rr * (kz * rv - ky * rw)), c[0],
                fma2(b2(ky * ph5 + rr * (kx * rw - kz * ru)), c[1],
                     fma2(b2(kz * ph5 + rr * (ky * ru - kx * rv)), c[2],
                          fma2(b2(al * e0), s34, mul2(b2(al * th * a), d34)))));
}

// Contravariant Euler flux of the face states on both lanes through the face
// metric (mx,my,mz) and lambda_5 = U.m + c|m| (Weno.cl:2291-2583).
__device__ __forceinline__ float2 contravariant_flux2(const float2 q[5], float mx, float my, float mz, float2 f[5])
{
    const float2 ir = rcp2(q[0]);
    const float2 u = mul2(q[1], ir), v = mul2(q[2], ir), w = mul2(q[3], ir);
    const float2 ke2 = fma2(q[1], u, fma2(q[2], v, mul2(q[3], w)));        // |m|^2 / rho
    const float2 pr = mul2(b2(0.4f), fma2(b2(-0.5f), ke2, q[4]));
    const float2 hq = fma2(b2(1.4f), q[4], mul2(b2(-0.2f), ke2));
    const float2 un = fma2(b2(mx), u, fma2(b2(my), v, mul2(b2(mz), w)));
    f[0] = mul2(q[0], un);
    f[1] = fma2(q[1], un, mul2(b2(mx), pr));
    f[2] = fma2(q[2], un, mul2(b2(my), pr));
    f[3] = fma2(q[3], un, mul2(b2(mz), pr));
    f[4] = mul2(hq, un);
    const float2 e = fma2(q[4], ir, mul2(b2(-0.5f), fma2(u, u, fma2(v, v, mul2(w, w)))));
    const float2 c2k = mul2(b2(1.4f * 0.4f * (mx * mx + my * my + mz * mz)), e);
    return add2(un, make_float2(sqrtf(c2k.x), sqrtf(c2k.y)));
}

// Reconstructed face states of one face on the two lanes, (pos, neg):
// the Roe eigen-system of the face, the characteristic projection of the
// stencil, WENO5 on both sides and the back-projection (Weno.cl:337-413,
// 1056-2289).  P[k][c] = (Q_c of stencil point k, Q_c of point 5-k), k =
// 0..2, points left-2 .. right+2; roe = Roe state of the face.
// DEV: the stencil enters as its deviation from ref (the face's left node)
// and ref is added back to the face states.  The projection is linear and
// WENO5 is unchanged by a constant shift (candidate weights sum to one, the
// smoothness indicators see differences only), so this is the same
// reconstruction; in FP32 its rounding scales with the variation across the
// stencil instead of with Q, and a uniform stencil returns ref exactly.
template <bool DEV = false>
__device__ __forceinline__ void reconstruct_face2(const float2 P[3][5], float mx, float my, float mz,
                                                  const float roe[5], float eps, const float *ref, float2 q[5])
{
    FaceEigen<float> eg;
    eg.init(mx, my, mz, roe);
    float2 C[5];   // (pos, neg) of each characteristic variable
    {
        float Lm[5][5];
        eg.left(Lm);
        float2 Pd[3][5];
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int c = 0; c < 5; ++c) Pd[k][c] = DEV ? sub2(P[k][c], b2(ref[c])) : P[k][c];
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            float2 cv[3];
#pragma unroll
            for (int k = 0; k < 3; ++k)
                cv[k] = fma2(b2(Lm[r][0]), Pd[k][0], fma2(b2(Lm[r][1]), Pd[k][1], fma2(b2(Lm[r][2]), Pd[k][2],
                             fma2(b2(Lm[r][3]), Pd[k][3], mul2(b2(Lm[r][4]), Pd[k][4])))));
            const float2 st[6] = {cv[0], cv[1], cv[2], swap2(cv[2]), swap2(cv[1]), swap2(cv[0])};
            C[r] = weno5_pos2(st, eps);
        }
    }
    right_times2(eg, C, q);
    if (DEV) {
#pragma unroll
        for (int c = 0; c < 5; ++c) q[c] = add2(q[c], b2(ref[c]));
    }
}

// LLF face flux (Weno.cl:2859-2947): Fhat = 0.5 det (Fp + Fn - alpha (qp - qn)),
// alpha = max |lambda_5|, all FP32.
__device__ __forceinline__ void llf_face_flux2(const float2 P[3][5], float mx, float my, float mz, float det_f,
                                               const float roe[5], float eps, float Fhat[5])
{
    float2 q[5], f[5];
    reconstruct_face2<false>(P, mx, my, mz, roe, eps, nullptr, q);
    const float2 lam = contravariant_flux2(q, mx, my, mz, f);
    const float alpha = fmaxf(fabsf(lam.x), fabsf(lam.y));
    const float2 sa = make_float2(-alpha, alpha);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        const float2 t = fma2(sa, q[c], f[c]);
        Fhat[c] = (0.5f * det_f) * (t.x + t.y);
    }
}

// The same LLF face flux with the metric and Jacobian products in FP64 (the
// split form): the face states (q+, q-) reconstructed as deviations from
// the face's left node (reconstruct_face2<true>), their velocities and
// pressures, lambda_5 and the dissipation alpha (q+ - q-) in FP32; the
// contravariant fluxes' metric products and their product by det_f / 2 in
// FP64 (Weno.cl:2585-2728, 2913-2947).  The central sum of the two states'
// fluxes q U_n + m p (and (E + p) U_n) is taken as
//   q+ U+ + q- U- = (q+ + q-) (U+ + U-) / 2 + (q+ - q-) (U+ - U-) / 2:
// the first term, which carries the metric, in FP64 with U+ + U- = m.(u+ +
// u-) from the FP64 face metric dm; the second, a product of two
// differences across the face, in FP32 with the dissipation.  A uniform
// stencil (q+ = q-) gives exactly the FP64 flux of that state.  m (FP32) is
// the face metric rounded, for the eigenvectors and lambda_5.  extra[c]
// (FP32) is added to component c with the other FP32 terms.
__device__ __forceinline__ void llf_face_flux2_split(const float2 P[3][5], float mx, float my, float mz,
                                                     const double dm[3], double det_f, const float roe[5], float eps,
                                                     const float extra[5], double Fhat[5])
{
    float2 q[5];
    const float ref[5] = {P[2][0].x, P[2][1].x, P[2][2].x, P[2][3].x, P[2][4].x};   // the left node
    reconstruct_face2<true>(P, mx, my, mz, roe, eps, ref, q);
    const float2 ir = rcp2(q[0]);
    const float2 u = mul2(q[1], ir), v = mul2(q[2], ir), w = mul2(q[3], ir);
    const float2 ke2 = fma2(q[1], u, fma2(q[2], v, mul2(q[3], w)));        // |m|^2 / rho
    const float2 pr = mul2(b2(0.4f), fma2(b2(-0.5f), ke2, q[4]));
    // lambda_5 = U.m + c |m| in FP32 (the LLF speed)
    const float2 un32 = fma2(b2(mx), u, fma2(b2(my), v, mul2(b2(mz), w)));
    const float2 e = fma2(q[4], ir, mul2(b2(-0.5f), fma2(u, u, fma2(v, v, mul2(w, w)))));
    const float2 c2k = mul2(b2(1.4f * 0.4f * (mx * mx + my * my + mz * mz)), e);
    const float2 lam = add2(un32, make_float2(sqrtf(c2k.x), sqrtf(c2k.y)));
    const float alpha = fmaxf(fabsf(lam.x), fabsf(lam.y));
    const double hd = 0.5 * det_f;
    const float hd32 = emu::d2f(hd);
    // FP32 terms: extra, less the dissipation, plus the difference term
    // (q+ - q-) (U+ - U-) / 2, all times det_f / 2 where they belong
    const float dun = un32.x - un32.y;
    float qs[5], x[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        const float qp = c == 4 ? q[4].x + pr.x : q[c].x, qn = c == 4 ? q[4].y + pr.y : q[c].y;
        qs[c] = qp + qn;
        x[c] = fmaf(hd32, fmaf(0.5f * (qp - qn), dun, -alpha * (q[c].x - q[c].y)), extra[c]);
    }
    // FP64: the metric products of the sum term and of the pressure (the
    // FP32 -> FP64 conversions on the integer pipe, emu::f2d: exact)
    using emu::f2d;
    const double hsun = hd * (0.5 * fma(dm[0], f2d(u.x + u.y), fma(dm[1], f2d(v.x + v.y), dm[2] * f2d(w.x + w.y))));
    const double hps = hd * f2d(pr.x + pr.y);
    Fhat[0] = fma(f2d(qs[0]), hsun, f2d(x[0]));
#pragma unroll
    for (int c = 1; c < 4; ++c) Fhat[c] = fma(dm[c - 1], hps, fma(f2d(qs[c]), hsun, f2d(x[c])));
    Fhat[4] = fma(f2d(qs[4]), hsun, f2d(x[4]));
}

// Sixth-order correction of a face flux from the node fluxes f[0..5]
// (Weno.cl:2950-3058): -d2/24 + 7 d4/5760, d2 = (-5,39,-34,-34,39,-5)/48,
// d4 = (1,-3,2,2,-3,1)/2 -- symmetric, so summed over mirrored pairs first.
__device__ __forceinline__ float face_correction_sym(const float f[6])
{
    const float s0 = f[0] + f[5], s1 = f[1] + f[4], s2 = f[2] + f[3];
    constexpr float a0 = (float)(5.0 / (48.0 * 24.0) + 7.0 / (5760.0 * 2.0));
    constexpr float a1 = (float)(-39.0 / (48.0 * 24.0) - 21.0 / (5760.0 * 2.0));
    constexpr float a2 = (float)(34.0 / (48.0 * 24.0) + 14.0 / (5760.0 * 2.0));
    return fmaf(a0, s0, fmaf(a1, s1, a2 * s2));
}

}  // namespace x2
}  // namespace cfd

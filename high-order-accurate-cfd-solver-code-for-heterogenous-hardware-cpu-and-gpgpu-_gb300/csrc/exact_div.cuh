// exact_div.cuh -- IEEE-exact FP64 arithmetic with fewer FP64 instructions:
// x / b with a reciprocal shared between several numerators (div), x * 2^K
// on the integer pipe (scale2), and 2^K / x from a reciprocal (pow2_over).
// All return the same bits as the IEEE operation (round to nearest even).
//
// Given y = 1/b (one IEEE division, reused for every numerator over b):
//   q0 = RN(x*y),  r0 = RN(b*(-q0) + x),  q1 = RN(r0*y + q0)
// is Markstein's correction step (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34,
// 1990); q1 is within a tiny fraction of an ulp of x/b.  Whether it is the
// correctly rounded quotient is then decided exactly: the remainder
// r1 = x - q1*b is exact in one FMA (q1 is a faithful quotient), and since a
// quotient of two binary64 numbers is never exactly halfway between two
// binary64 numbers, q1 = RN(x/b) if and only if |r1| < ulp(q1)/2 * |b|.
// Both sides are compared as bit patterns (non-negative doubles order like
// integers); the right side is |b| with its exponent moved, exact.
// Anything outside the plain case -- a zero, subnormal or non-finite value
// anywhere, q1 a power of two (whose lower neighbour is half an ulp away),
// exponents near the range ends, or a failed test -- takes div_rare: IEEE
// 754's exact results for zero and infinite operands, else the IEEE
// division x / b itself.  The results are therefore identical to x / b for
// all inputs; the gain is 4 FP64 instructions per shared division instead of a
// full division sequence.  quotient_int goes further on a part whose FP64
// rate is a small fraction of its integer rate: only q0 on the FP64 pipe,
// its rounding decided from the exact integer remainder of the significands
// (the default of div()).
#pragma once

#include <cstdint>
#include <cmath>
#if defined(__CUDACC__)
#include <cuda_runtime.h>
#define CFD_XDIV_HD __host__ __device__ __forceinline__
#else
#define CFD_XDIV_HD inline
#endif

// Where quotient_int's first quotient q0 comes from: 1 (the default) the
// top 53 bits of the integer product of the significands of x and y (no
// FP64 instruction; the faster choice in kernels with warps to hide its
// integer latency, 3 or more blocks of 128 per SM), 0 the FP64 product
// RN(x*y) (kernels at 2 blocks per SM: the drop-in's face kernel, the
// batched stage, the FP64 face passes at that budget).  A translation unit
// sets it before its first include; the two variants live in different
// inline namespaces, so the host functions of units built with different
// choices do not collide at link time.  Both give the same bits.
#ifndef CFD_XDIV_QPROD
#define CFD_XDIV_QPROD 1
#endif
#if CFD_XDIV_QPROD
#define CFD_XDIV_VARIANT qprod_int
#else
#define CFD_XDIV_VARIANT qprod_fp64
#endif

namespace cfd {
namespace xdiv {
inline namespace CFD_XDIV_VARIANT {

CFD_XDIV_HD uint64_t bits(double v)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t u;
    __builtin_memcpy(&u, &v, 8);
    return u;
#endif
}

CFD_XDIV_HD double fma_rn(double a, double b, double c)
{
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

CFD_XDIV_HD double from_bits(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double v;
    __builtin_memcpy(&v, &u, 8);
    return v;
#endif
}

CFD_XDIV_HD double mul_rn(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    volatile double r = a * b;
    return r;
#endif
}

// The plain-case quotient, or 0 with ok = false.
CFD_XDIV_HD double quotient(double x, double b, double y, bool &ok)
{
    const double q0 = mul_rn(x, y);
    const double r0 = fma_rn(-q0, b, x);
    const double q1 = fma_rn(r0, y, q0);
    const double r1 = fma_rn(-q1, b, x);
    const uint64_t uq = bits(q1), ub = bits(b) & 0x7fffffffffffffffULL, ur = bits(r1) & 0x7fffffffffffffffULL;
    const int eq = (int)((uq >> 52) & 0x7ff), eb = (int)(ub >> 52);
    // |b| * ulp(q1) / 2 = |b| * 2^(eq - 1023 - 53): biased exponent et
    const int et = eb + eq - 1076;
    ok = eq > 0 && eq < 0x7ff && (uq & 0x000fffffffffffffULL) != 0 && eb > 0 && eb < 0x7ff && et > 0 && et < 0x7ff
         && ur < (((uint64_t)et << 52) | (ub & 0x000fffffffffffffULL));
    return q1;
}

// The IEEE division, out of line so that the plain case carries none of
// its instructions.
#if defined(__CUDACC__)
static __host__ __device__ __noinline__ double ieee_div(double x, double b) { return x / b; }
#else
static double ieee_div(double x, double b) { return x / b; }
#endif

// The high 64 bits of the 128-bit product a*b.
CFD_XDIV_HD uint64_t mul_hi64(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// x / b given y = 1 / b (IEEE), with the rounding decided on the integer
// pipe.  q0 lies within two ulps of x/b: either RN(x*y), or x*y truncated
// to 53 bits, from the high word of the product of the significands
// shifted to the top of their words (X*Y in [2^104, 2^106), so
// H = floor(X*Y / 2^42) lies in [2^62, 2^64) and its top 53 bits are
// floor(X*Y / 2^(52 + t)), t = 1 when X*Y >= 2^105) -- y = RN(1/b) is within
// half an ulp of 1/b and the truncation drops less than one.  With
// significands X, B, Q (53-bit integers, hidden bit set) and
// s = ex - eb - eq + 1075 (52 or 53 in the plain case), X*2^s and Q*B are
// the dividend and q0 times the divisor on a common scale, so
// R = X*2^s - Q*B is the exact remainder (|R| < 2^56: the low 64 bits of
// both products give it).  x/b is (Q + R/B) ulps, never exactly halfway
// between two doubles, so the correctly rounded quotient is q0 moved by the
// nearest integer to R/B, found by comparing 2R with +-B and +-3B.  The
// plain case: x, y, q0 and 1/b normal (b below 2^1022), the significand of
// q0 in [2^52 + 3, 2^53 - 2] (a step of up to two ulps then rounds within
// the binade, or lands exactly on its upper end) and |R/B| < 5/2;
// everything else takes div_rare.  No FP64 instruction (QP = 1; one FP64
// multiply with QP = 0) instead of the four of quotient().
template <int QP>
CFD_XDIV_HD double quotient_int_v(double x, double b, double y, bool &ok)
{
    constexpr uint64_t kFrac = 0x000fffffffffffffULL, kHidden = 0x0010000000000000ULL;
    const uint64_t ux = bits(x), ub = bits(b);
    const int ex = (int)((ux >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
    const uint64_t X = (ux & kFrac) | kHidden;
    const uint64_t B = (ub & kFrac) | kHidden;
    uint64_t uq;
    int eq;
    bool y_ok = true;
    if (QP) {
        const uint64_t uy = bits(y);
        const int ey = (int)((uy >> 52) & 0x7ff);
        const uint64_t H = mul_hi64(X << 11, ((uy & kFrac) | kHidden) << 11);
        const int t = (int)(H >> 63);
        eq = ex + ey - 1023 + t;
        uq = ((ux ^ uy) & 0x8000000000000000ULL) | ((uint64_t)(eq & 0x7ff) << 52) | ((H >> (10 + t)) & kFrac);
        y_ok = (unsigned)(ey - 1) < 2046u;
    } else {
        uq = bits(mul_rn(x, y));
        eq = (int)((uq >> 52) & 0x7ff);
    }
    const uint64_t F = uq & kFrac;
    const int s = ex - eb - eq + 1075;
    const int64_t R = (int64_t)((X << (s & 63)) - (F | kHidden) * B);
    const int64_t R2 = R * 2, Bs = (int64_t)B, B3 = 3 * (int64_t)B;
    const int d = (int)(R2 > Bs) + (int)(R2 > B3) - (int)(R2 < -Bs) - (int)(R2 < -B3);
    ok = y_ok && (unsigned)(ex - 1) < 2046u && (unsigned)(eb - 1) < 2044u && (unsigned)(eq - 1) < 2045u
         && (unsigned)(s - 52) < 2u && F - 3u < 0x000ffffffffffffcULL && R2 < 5 * Bs && R2 > -5 * Bs;
    return from_bits(uq + (uint64_t)(int64_t)d);
}

// quotient_int_v with this translation unit's CFD_XDIV_QPROD.
CFD_XDIV_HD double quotient_int(double x, double b, double y, bool &ok)
{
    return quotient_int_v<CFD_XDIV_QPROD>(x, b, y, ok);
}

// x / b given y = 1 / b, outside quotient_int's plain case.
//  * q0 = RN(x*y) within three ulps of either end of its binade (the plain
//    case's margin): x / b is (Q + R/B) ulps as there, and when that lies in
//    q0's binade -- F*B + R >= 0 at the lower end (x / b at least 2^e), R <
//    (2^52 - F)*B at the upper end (below 2^(e+1)) -- rounding at q0's ulp
//    is correct, and a step onto 2^(e+1) carries into the exponent field.
//    Exact powers of two and their neighbours are common quotients: a WENO
//    weight over three equal smoothness indicators (a uniform region), a
//    unit normal's component on an extruded lattice.
//  * Zero and infinite operands have exact results (IEEE 754 6.1, 6.3, 7.3):
//    0 / nonzero and finite / Inf are zeros, nonzero / 0 and Inf / finite
//    are infinities, each with the exclusive or of the operands' signs.
//    Flows that stay two-dimensional in a three-dimensional lattice divide
//    exact zeros (a velocity component, a metric term, a derivative across
//    the extrusion) at every node and face, and the MTS model divides by a
//    test-filter value of exactly 0 across the extrusion and then by the
//    infinite quotient.
// All on the integer pipe; everything else (0 / 0, Inf / Inf, NaN,
// subnormal operands, quotients near the ends of the range or leaving q0's
// binade) is the IEEE division.  Out of line, as the division was: the
// plain case carries none of it and the kernels' code stays the size it was.
#if defined(__CUDACC__)
static __host__ __device__ __noinline__ double div_rare(double x, double b, double y)
#else
static double div_rare(double x, double b, double y)
#endif
{
    constexpr uint64_t kSign = 0x8000000000000000ULL, kInf = 0x7ff0000000000000ULL;
    constexpr uint64_t kFrac = 0x000fffffffffffffULL, kHidden = 0x0010000000000000ULL;
    const uint64_t ux = bits(x), ub = bits(b);
    {
        const double q0 = mul_rn(x, y);
        const uint64_t uq = bits(q0);
        const int ex = (int)((ux >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff), eq = (int)((uq >> 52) & 0x7ff);
        const uint64_t X = (ux & kFrac) | kHidden, B = (ub & kFrac) | kHidden, F = uq & kFrac;
        const int s = ex - eb - eq + 1075;
        const int64_t R = (int64_t)((X << (s & 63)) - (F | kHidden) * B);
        const int64_t R2 = R * 2, Bs = (int64_t)B, B3 = 3 * (int64_t)B;
        const int d = (int)(R2 > Bs) + (int)(R2 > B3) - (int)(R2 < -Bs) - (int)(R2 < -B3);
        if ((unsigned)(ex - 1) < 2046u && (unsigned)(eb - 1) < 2044u && (unsigned)(eq - 1) < 2045u
            && (unsigned)(s - 52) < 2u && R2 < 5 * Bs && R2 > -5 * Bs
            && ((F < 3u && R + (int64_t)F * Bs >= 0) || (F > kFrac - 3u && R < (int64_t)(kHidden - F) * Bs)))
            return from_bits(uq + (uint64_t)(int64_t)d);
    }
    const uint64_t ax = ux & ~kSign, ab = ub & ~kSign, sign = (ux ^ ub) & kSign;
    if (ax <= kInf && ab <= kInf && !(ax == ab && (ax == 0 || ax == kInf))) {
        if (ax == 0 || ab == kInf) return from_bits(sign);
        if (ab == 0 || ax == kInf) return from_bits(sign | kInf);
    }
    return ieee_div(x, b);
}

#if defined(__CUDACC__)
// 1 / b rounded to nearest even, for b whose reciprocal is a normal number
// (biased exponent eb in [1, 2044]) and whose significand B is not a power
// of two (rcp returns that exact reciprocal in its rare branch): a float
// reciprocal of B's top 24 bits seeds one Newton step on the FP64 pipe,
//   e = RN(1 - |b| y0),  y1 = RN(y0 e + y0)   (relative error ~2^-47),
// and the rounding is then decided on the integer pipe: with Y the
// significand of y1, R = 2^105 - Y*B is the exact remainder (|R| < 2^61:
// the seed is within 1.5 2^-23 and the step squares that, so the low 64
// bits of the product give it), R/B is estimated from the top
// bits of R and Y (Y ~ 2^105 / B), the estimate's remainder R1 is exact, and
// Y moves by the nearest integer to R/B (2^105 / B is never halfway between
// two integers).  ok = false (and the caller divides) outside that case.
__device__ __forceinline__ double rcp_int(double b, bool &ok)
{
    const uint64_t ub = bits(b);
    const int eb = (int)((ub >> 52) & 0x7ff);
    const uint64_t F = ub & 0x000fffffffffffffULL, B = F | 0x0010000000000000ULL;
    const uint64_t sign = ub & 0x8000000000000000ULL;
    const float rf = __frcp_rn(__uint_as_float(0x3f800000u | (uint32_t)(F >> 29)));   // ~ 2^52 / B, in (0.5, 1]
    const uint32_t rb = __float_as_uint(rf);
    const int ey0 = (int)(rb >> 23) - 127 + 2046 - eb;   // biased exponent of rf * 2^(1023 - eb)
    const double y0 = from_bits(((uint64_t)(unsigned)ey0 << 52) | ((uint64_t)(rb & 0x7fffffu) << 29));
    const double e = fma_rn(-from_bits(ub & 0x7fffffffffffffffULL), y0, 1.0);
    const double y1 = fma_rn(y0, e, y0);
    const uint64_t u1 = bits(y1);
    const uint64_t Y = (u1 & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    const int64_t R = (int64_t)(0ULL - Y * B);
    const int64_t d0 = ((R >> 29) * (int64_t)(Y >> 23)) >> 53;   // < 2^62 before the shift
    const int64_t R1 = R - d0 * (int64_t)B;
    const int64_t R2 = 2 * R1, Bs = (int64_t)B;
    const int64_t d = d0 + (int64_t)(R2 > Bs) + (int64_t)(R2 > 3 * Bs) - (int64_t)(R2 < -Bs);
    const uint64_t Yn = Y + (uint64_t)d;
    ok = (unsigned)(eb - 1) < 2044u && F != 0 && (int)((u1 >> 52) & 0x7ff) == 2045 - eb && R2 < 5 * Bs
         && R2 > -5 * Bs && (Yn >> 52) == 1u;
    return from_bits(sign | ((uint64_t)(2045 - eb) << 52) | (Yn & 0x000fffffffffffffULL));
}

#endif

// float <-> bits and the float reciprocal RN(1/x) (the host's IEEE division
// stands in for __frcp_rn); the high 64 bits of a signed 128-bit product.
CFD_XDIV_HD uint32_t bits32(float v)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(v);
#else
    uint32_t u;
    __builtin_memcpy(&u, &v, 4);
    return u;
#endif
}

CFD_XDIV_HD float from_bits32(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float v;
    __builtin_memcpy(&v, &u, 4);
    return v;
#endif
}

CFD_XDIV_HD float frcp_rn(float x)
{
#if defined(__CUDA_ARCH__)
    return __frcp_rn(x);
#else
    volatile float one = 1.0f;
    return one / x;
#endif
}

CFD_XDIV_HD int64_t mul_hi64s(int64_t a, int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    return (int64_t)(((__int128)a * b) >> 64);
#endif
}

// rcp_int's case (b's reciprocal normal, B not a power of two) with the
// Newton step on the integer pipe too, no FP64 instruction at all.  With S0
// the significand of the float seed y0 = RN(1/m), m = B's top 24 bits as a
// float in [1, 2) (y0 = S0 2^-24), eps = 1 - (B / 2^52) y0 is exactly
// E / 2^76 with E = 2^76 - S0*B, and |eps| < 2^-22.4 (the seed is within
// 2^-24, the 29 dropped bits within 2^-23), so |E| < 2^54 and the low 64
// bits of S0*B give it.  2^105 / B = S0 2^29 / (1 - eps), so
//   Y = S0 2^29 + S0 (E + E^2 / 2^76) / 2^47
// (two terms of the series; the next is below 2^-13, the two floors below 2)
// is within 2 of 2^105 / B, and the exact remainder R = 2^105 - Y*B
// (|R| < 2^55) decides the rounding: Y moves by the nearest integer to R/B,
// found by comparing 2R with +-B and +-3B.  ok = false outside the plain
// case (a step out of [2^52, 2^53) included).
CFD_XDIV_HD double rcp_int_i(double b, bool &ok)
{
    constexpr uint64_t kFrac = 0x000fffffffffffffULL, kHidden = 0x0010000000000000ULL;
    const uint64_t ub = bits(b);
    const int eb = (int)((ub >> 52) & 0x7ff);
    const uint64_t F = ub & kFrac, B = F | kHidden;
    const uint32_t rb = bits32(frcp_rn(from_bits32(0x3f800000u | (uint32_t)(F >> 29))));   // y0 in (0.5, 1]
    const uint64_t S0 = (uint64_t)((rb & 0x7fffffu) | 0x800000u) << ((rb >> 23) - 126u);   // 2^23 .. 2^24
    const int64_t E = (int64_t)(0ULL - S0 * B);
    const int64_t E2 = mul_hi64s(E, E) >> 12;                          // E^2 / 2^76
    const uint64_t Y = (S0 << 29) + (uint64_t)mul_hi64s((int64_t)(S0 << 17), E + E2);
    const int64_t R = (int64_t)(0ULL - Y * B);
    const int64_t R2 = 2 * R, Bs = (int64_t)B, B3 = 3 * (int64_t)B;
    const int64_t d = (int64_t)(R2 > Bs) + (int64_t)(R2 > B3) - (int64_t)(R2 < -Bs) - (int64_t)(R2 < -B3);
    const uint64_t Yn = Y + (uint64_t)d;
    ok = (unsigned)(eb - 1) < 2044u && F != 0 && R2 < 5 * Bs && R2 > -5 * Bs && (Yn >> 52) == 1u;
    return from_bits((ub & 0x8000000000000000ULL) | ((uint64_t)(2045 - eb) << 52) | (Yn & kFrac));
}

#if defined(__CUDACC__)
// 1 / b outside rcp_int's plain case: 1 / +-0 = +-Inf and 1 / +-Inf = +-0
// (IEEE 754 7.3, 6.1); a power of two b = 2^(eb - 1023) has the exact
// reciprocal 2^(1023 - eb), biased exponent 2046 - eb, normal for eb in
// [1, 2045] (a density or a metric of exactly 1 is common); anything else
// is the IEEE division.  Out of line.
static __device__ __noinline__ double rcp_rare(double b)
{
    constexpr uint64_t kSign = 0x8000000000000000ULL, kInf = 0x7ff0000000000000ULL;
    const uint64_t ub = bits(b), ab = ub & ~kSign;
    if (ab == 0) return from_bits((ub & kSign) | kInf);
    if (ab == kInf) return from_bits(ub & kSign);
    const unsigned eb = (unsigned)(ub >> 52) & 0x7ffu;
    if ((ub & 0x000fffffffffffffULL) == 0 && eb - 1u < 2045u)
        return from_bits((ub & kSign) | ((uint64_t)(2046u - eb) << 52));
    return 1.0 / b;
}
#endif

// 1 / b, the same bits as the IEEE division (rcp_int's plain case on the
// device when CFD_XDIV_RCP is set -- the default; GB300 TGV 128^3: FP64
// face pass 6.62 -> 6.42 ms -- else the division).
#ifndef CFD_XDIV_RCP
#define CFD_XDIV_RCP 1
#endif
// Which Newton step rcp uses: 1 rcp_int_i (integer pipe; by default where
// the first quotient is the integer product too), 0 rcp_int (two FP64 FMAs).
#ifndef CFD_XDIV_RCPI
#define CFD_XDIV_RCPI CFD_XDIV_QPROD
#endif
CFD_XDIV_HD double rcp(double b)
{
#if defined(__CUDA_ARCH__)
    if (CFD_XDIV_RCP) {
        bool ok;
        const double y = CFD_XDIV_RCPI ? rcp_int_i(b, ok) : rcp_int(b, ok);
        if (__builtin_expect(ok, 1)) return y;
        return rcp_rare(b);
    }
#endif
    return 1.0 / b;
}

// Which plain-case quotient div() uses: the integer-pipe rounding
// (quotient_int, 1 FP64 operation; GB300 TGV 128^3: face pass 7.72 ->
// 6.80 ms) or the FP64 Markstein step (quotient, 4).
#ifndef CFD_XDIV_INT
#define CFD_XDIV_INT 1
#endif

// x / b given y = 1 / b (IEEE): the same bits as x / b.
CFD_XDIV_HD double div(double x, double b, double y)
{
    bool ok;
    const double q = CFD_XDIV_INT ? quotient_int(x, b, y, ok) : quotient(x, b, y, ok);
    if (__builtin_expect(ok, 1)) return q;
    return div_rare(x, b, y);
}

// x / b for a divisor used once: its reciprocal (rcp) and the quotient's
// rounding (div); the same bits as x / b.
CFD_XDIV_HD double divide(double x, double b) { return div(x, b, rcp(b)); }

// The IEEE product, out of line (scale2's rare case).
#if defined(__CUDACC__)
static __host__ __device__ __noinline__ double ieee_mul(double x, double c) { return x * c; }
#else
static double ieee_mul(double x, double c)
{
    volatile double r = x * c;
    return r;
}
#endif

// x * 2^K for a constant K, 1 <= |K| <= 8: the same bits as the IEEE product
// x * 2^K.  When x and the product are normal numbers (biased exponents e and
// e + K both in [1, 2046]) the product differs from x only in its exponent
// field, so it is one integer add on the high word; +-0 stays +-0; every
// other operand (subnormal, a product that would overflow or become
// subnormal, Inf, NaN) takes the FP64 multiply out of line.  On a part whose
// FP64 rate is a small fraction of its integer rate this takes a multiply
// by 2, 4, 1/2, 1/4, ... off the FP64 pipe.
template <int K>
CFD_XDIV_HD double scale2(double x)
{
    static_assert(K != 0 && K >= -8 && K <= 8, "scale2: 1 <= |K| <= 8");
    constexpr unsigned lo = K < 0 ? 1u + (unsigned)(-K) : 1u;       // smallest e with a normal product
    constexpr unsigned hi = K > 0 ? 2046u - (unsigned)K : 2046u;     // largest
    constexpr double c = K > 0 ? (double)(1u << (K > 0 ? K : 0)) : 1.0 / (double)(1u << (K < 0 ? -K : 0));
    const uint64_t u = bits(x);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    if (__builtin_expect(e - lo <= hi - lo, 1)) return from_bits(u + ((uint64_t)(int64_t)K << 52));
    if ((u << 1) == 0) return x;
    return ieee_mul(x, c);
}

// 2^K / x for a constant K, 1 <= |K| <= 8: the same bits as the IEEE
// division 2^K / x.  Rounding commutes with scaling by a power of two while
// every value stays a normal number, so with r = 1 / x (IEEE reciprocal,
// cheaper than a division) the quotient is r with its exponent moved by K;
// r zero, subnormal or non-finite, or a result within one binade of the
// normal range's ends, takes the division itself.
template <int K>
CFD_XDIV_HD double pow2_over(double x)
{
    static_assert(K != 0 && K >= -8 && K <= 8, "pow2_over: 1 <= |K| <= 8");
    constexpr unsigned lo = K < 0 ? 2u + (unsigned)(-K) : 2u;
    constexpr unsigned hi = K > 0 ? 2045u - (unsigned)K : 2045u;
    constexpr double c = K > 0 ? (double)(1u << (K > 0 ? K : 0)) : 1.0 / (double)(1u << (K < 0 ? -K : 0));
    const double r = rcp(x);
    const uint64_t u = bits(r);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    if (__builtin_expect(e - lo <= hi - lo, 1)) return from_bits(u + ((uint64_t)(int64_t)K << 52));
    return ieee_div(c, x);
}

}  // namespace CFD_XDIV_VARIANT
}  // namespace xdiv
}  // namespace cfd

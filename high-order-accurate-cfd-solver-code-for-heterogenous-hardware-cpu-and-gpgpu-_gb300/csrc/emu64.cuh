// emu64.cuh -- binary64 operations on the integer pipe with the same bits
// as the hardware instructions: the conversions between binary32 and
// binary64 (f2d exact, d2f rounded to nearest even), and addition and
// multiplication (round to nearest even).
//
// GB300 executes FP64 arithmetic and the F32<->F64 conversions on one FP64
// pipe that issues about two operations per clock per SM, against 128
// 32-bit integer or FP32 lanes.  A precision form that keeps some values in
// FP64 and the rest in FP32 spends a large part of its FP64-pipe time in
// conversions; done here they leave that pipe to the FP64 arithmetic.  The
// routines build each result from the operands' bit patterns -- the
// textbook construction of a correctly rounded binary operation from its
// definition in IEEE 754-2008 (sections 4.3, 5.4.2; e.g. J.-M. Muller et
// al., Handbook of Floating-Point Arithmetic, 2nd ed., 2018, ch. 8,
// "software implementation of the basic operations"): exact significand
// arithmetic, a guard field and a sticky bit, normalisation, rounding to
// nearest with ties to even.
//
// The integer path covers normal numbers (and zeros where that is cheap);
// anything else -- subnormal, infinite or NaN operands, or a result that
// would be subnormal -- takes the hardware instruction out of line, so
// every input gives the IEEE result.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace cfd {
namespace emu {

__device__ __forceinline__ uint64_t u64(double v) { return (uint64_t)__double_as_longlong(v); }
__device__ __forceinline__ double f64(uint64_t u) { return __longlong_as_double((long long)u); }

constexpr uint64_t kSign = 0x8000000000000000ULL;
constexpr uint64_t kAbs = 0x7fffffffffffffffULL;
constexpr uint64_t kFrac = 0x000fffffffffffffULL;
constexpr uint64_t kHidden = 0x0010000000000000ULL;

// the FP64-pipe instructions, out of line so the integer path carries none
// of their code
static __device__ __noinline__ double fp64_add(double a, double b) { return __dadd_rn(a, b); }
static __device__ __noinline__ double fp64_mul(double a, double b) { return __dmul_rn(a, b); }
static __device__ __noinline__ double fp64_of(float f) { return (double)f; }
static __device__ __noinline__ float fp32_of(double x) { return __double2float_rn(x); }

// (double)f, exact.  A normal float's exponent field is rebased by
// 1023 - 127 = 896 and its 23-bit significand moved to the top of the
// double's 52; zeros keep their sign.
__device__ __forceinline__ double f2d(float f)
{
    const uint32_t b = __float_as_uint(f);
    const uint32_t m = b & 0x7fffffffu;
    if (__builtin_expect(m - 0x00800000u >= 0x7f000000u, 0)) {   // zero, subnormal, Inf or NaN
        if (m == 0u) return f64((uint64_t)b << 32);
        return fp64_of(f);
    }
    const uint32_t hi = (b & 0x80000000u) | ((m >> 3) + (896u << 20));
    return f64(((uint64_t)hi << 32) | (uint64_t)(b << 29));
}

// (float)x rounded to nearest even.  For a biased exponent e in
// [897, 1150] (a normal float) the 52-bit significand keeps its top 23 bits;
// the 29 below decide the rounding (above half, or exactly half with an odd
// result, rounds up), and a carry out of the significand moves into the
// exponent (to infinity past the largest float, as IEEE rounding does).
// Zeros keep their sign; smaller, larger and non-finite x take the
// conversion instruction.
__device__ __forceinline__ float d2f(double x)
{
    const uint64_t u = u64(x);
    const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
    const uint32_t e = (hi >> 20) & 0x7ffu;
    if (__builtin_expect(e - 897u >= 254u, 0)) {
        if ((u << 1) == 0) return __uint_as_float(hi);   // +-0
        return fp32_of(x);
    }
    const uint32_t m23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t r = lo & 0x1fffffffu;
    const uint32_t up = (uint32_t)(r > 0x10000000u) | ((uint32_t)(r == 0x10000000u) & m23 & 1u);
    return __uint_as_float((hi & 0x80000000u) | (((e - 896u) << 23) + m23 + up));
}

// The double-float pair of x: hi = (float)x (round to nearest even) and
// lo = (float)(x - hi) -- the same bits as those two conversions with the
// FP64 subtraction between them, which is exact.  For a biased exponent e in
// [950, 1099] the 29 significand bits below hi's 23 give the difference
// directly: D = those bits, less 2^29 when hi rounded up, is an integer of
// at most 29 bits with x - hi = sign(x) D 2^(e - 1075); its float (one
// rounding, the only one) scaled by that power of two is lo.  Other
// exponents take the conversions.
__device__ __forceinline__ void hi_lo(double x, float &hi, float &lo)
{
    const uint64_t u = u64(x);
    const uint32_t hw = (uint32_t)(u >> 32), lw = (uint32_t)u;
    const uint32_t e = (hw >> 20) & 0x7ffu;
    if (__builtin_expect(e - 950u >= 150u, 0)) {
        hi = d2f(x);
        lo = d2f(x - f2d(hi));
        return;
    }
    const uint32_t m23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
    const uint32_t r = lw & 0x1fffffffu;
    const uint32_t up = (uint32_t)(r > 0x10000000u) | ((uint32_t)(r == 0x10000000u) & m23 & 1u);
    hi = __uint_as_float((hw & 0x80000000u) | (((e - 896u) << 23) + m23 + up));
    const int D = (int)r - (int)(up << 29);
    const float f = __int2float_rn(D);   // |D| <= 2^28: a normal float, rounded once
    lo = D == 0 ? 0.0f
                : __uint_as_float((__float_as_uint(f) + ((e - 1075u) << 23)) ^ (hw & 0x80000000u));
}

// a + b.  With |X| >= |Y| (exponents ex >= ey, d = ex - ey) the
// significands, shifted left by 10 (leading bit at 62, ten guard bits), are
// aligned by d with the bits shifted out of Y collected in bit 0 (sticky).
// Whenever bits are lost the aligned Y is odd, so the exact sum lies
// strictly between two integers around the computed S and never on a
// rounding boundary (a multiple of 2^9): rounding S rounds the exact sum.
// S is renormalised so its leading bit is again at 62 (right by one with
// the sticky bit kept, or left with zeros entering; the usual positions are
// tested before a leading-zero count), then rounded at bit 10.  The
// exponent field is added to the rounded significand with its hidden bit,
// so a rounding carry moves into the exponent (and to infinity past the
// largest finite value, as IEEE rounding to nearest does).  An exact
// cancellation gives +0.  For d >= 55 the sum rounds to X (|Y| < ulp(X)/4);
// 32 <= d <= 54 takes the FP64 add.
__device__ __forceinline__ double add(double a, double b)
{
    const uint64_t ua = u64(a), ub = u64(b);
    const bool swp = (ua & kAbs) < (ub & kAbs);
    const uint64_t ux = swp ? ub : ua, uy = swp ? ua : ub;
    const unsigned ex = (unsigned)(ux >> 52) & 0x7ffu, ey = (unsigned)(uy >> 52) & 0x7ffu;
    const unsigned d = ex - ey;
    if (__builtin_expect(ey == 0u || ex == 0x7ffu || d > 31u, 0)) {
        if (d >= 55u && ex != 0x7ffu && ex != 0u) return f64(ux);
        return fp64_add(a, b);
    }
    const uint64_t X = ((ux & kFrac) | kHidden) << 10;
    const uint64_t Y0 = ((uy & kFrac) | kHidden) << 10;
    const uint32_t lost = (uint32_t)Y0 & ((1u << d) - 1u);
    const uint64_t Y = (Y0 >> d) | (uint64_t)(lost != 0u);
    const uint64_t m = (uint64_t)0 - ((ux ^ uy) >> 63);   // all ones when the signs differ
    const uint64_t S = X + (Y ^ m) + (m & 1u);            // X + Y or X - Y
    uint64_t N;
    int er;
    if ((int64_t)S < 0) {   // carry out of bit 62
        N = (S >> 1) | (S & 1u);
        er = (int)ex + 1;
    } else if (S >> 62) {
        N = S;
        er = (int)ex;
    } else if (S >> 61) {   // one bit cancelled
        N = S << 1;
        er = (int)ex - 1;
    } else {
        if (S == 0) return 0.0;
        const int lz = __clzll((long long)S);
        er = (int)ex + 1 - lz;
        N = S << (lz - 1);
    }
    if (__builtin_expect((unsigned)(er - 1) >= 2046u, 0)) return fp64_add(a, b);
    const uint64_t M = N >> 10;
    const unsigned low = (unsigned)N & 0x3ffu;
    const uint64_t up = (low > 0x200u) | ((low == 0x200u) & (unsigned)M & 1u);
    return f64((ux & kSign) | ((((uint64_t)(er - 1)) << 52) + M + up));
}

__device__ __forceinline__ double sub(double a, double b) { return add(a, f64(u64(b) ^ kSign)); }

// a * b.  The 53-bit significands multiply exactly into 106 bits from four
// 32 x 32 -> 64 products; with the leading bit at 105 (top = 1) or 104 the
// result is the product shifted right by 52 + top, the next bit down is the
// round bit and everything below it the sticky flag; then rounding to
// nearest even as in add.  An operand that is zero, subnormal, infinite or
// NaN, or an exponent ea + eb - 1023 (+ top) outside [1, 2046] -- a
// subnormal result or an overflow before rounding -- takes the FP64
// multiply.
__device__ __forceinline__ double mul(double a, double b)
{
    const uint64_t ua = u64(a), ub = u64(b);
    const uint32_t ha = (uint32_t)(ua >> 32), hb = (uint32_t)(ub >> 32);
    const uint32_t la = (uint32_t)ua, lb = (uint32_t)ub;
    const unsigned ea = (ha >> 20) & 0x7ffu, eb = (hb >> 20) & 0x7ffu;
    const int e = (int)ea + (int)eb - 1023;
    if (__builtin_expect(ea - 1u >= 0x7feu || eb - 1u >= 0x7feu || (unsigned)e > 2045u, 0)) return fp64_mul(a, b);
    const uint32_t ah = (ha & 0xfffffu) | 0x100000u, bh = (hb & 0xfffffu) | 0x100000u;
    const uint64_t p0 = (uint64_t)la * lb;
    const uint64_t mid = (uint64_t)ah * lb + (uint64_t)la * bh;
    const uint64_t lo = p0 + (mid << 32);
    const uint64_t hi = (uint64_t)ah * bh + (mid >> 32) + (lo < p0);   // product = hi * 2^64 + lo
    const unsigned top = (unsigned)(hi >> 41);
    const uint64_t M0 = (hi << 12) | (lo >> 52);   // product >> 52
    const uint64_t G = lo << 12;                   // product bits 51..0 at the top
    const uint64_t M = M0 >> top;
    const unsigned rnd = top ? (unsigned)M0 & 1u : (unsigned)(G >> 63);
    const unsigned stk = top ? (G != 0) : ((G << 1) != 0);
    const uint64_t up = rnd & (stk | ((unsigned)M & 1u));
    const int er = e + (int)top;
    if (__builtin_expect(er < 1, 0)) return fp64_mul(a, b);
    return f64(((ua ^ ub) & kSign) | ((((uint64_t)(er - 1)) << 52) + M + up));
}

// A binary64 value whose +, - and * run on the integer pipe (the routines
// above; the same bits as the FP64 instructions).  An expression over Dbl
// reads and evaluates exactly like the same expression over double: the
// same operations in the same order, double constants converted exactly.
struct Dbl {
    double v;
    Dbl() = default;
    __host__ __device__ __forceinline__ constexpr Dbl(double x) : v(x) {}
};
__device__ __forceinline__ Dbl operator+(Dbl a, Dbl b) { return Dbl(add(a.v, b.v)); }
__device__ __forceinline__ Dbl operator-(Dbl a, Dbl b) { return Dbl(sub(a.v, b.v)); }
__device__ __forceinline__ Dbl operator*(Dbl a, Dbl b) { return Dbl(mul(a.v, b.v)); }
__device__ __forceinline__ Dbl operator-(Dbl a) { return Dbl(f64(u64(a.v) ^ kSign)); }

// Products on the integer pipe, sums on the FP64 pipe.
struct DblM {
    double v;
    DblM() = default;
    __host__ __device__ __forceinline__ constexpr DblM(double x) : v(x) {}
};
__device__ __forceinline__ DblM operator+(DblM a, DblM b) { return DblM(__dadd_rn(a.v, b.v)); }
__device__ __forceinline__ DblM operator-(DblM a, DblM b) { return DblM(__dsub_rn(a.v, b.v)); }
__device__ __forceinline__ DblM operator*(DblM a, DblM b) { return DblM(mul(a.v, b.v)); }
__device__ __forceinline__ DblM operator-(DblM a) { return DblM(f64(u64(a.v) ^ kSign)); }

// The double held by a value of any of the three types.
__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(Dbl x) { return x.v; }
__device__ __forceinline__ double val(DblM x) { return x.v; }

}  // namespace emu
}  // namespace cfd

// softfp64.cuh -- IEEE 754 binary64 addition and multiplication, round to
// nearest even, computed on the integer pipes.
//
// GB300 issues FP64 arithmetic at about 1/70 of its instruction rate, so the
// reference's FP64 face flux keeps the FP64 pipe busy while the integer
// pipes idle.  These routines produce the same bits as the hardware's
// add.rn.f64 / mul.rn.f64 (the textbook algorithms: align, add or multiply
// the significands exactly, normalise, round with guard and sticky bits --
// Goldberg, "What every computer scientist should know about floating-point
// arithmetic", 1991; Muller et al., "Handbook of Floating-Point Arithmetic",
// 2nd ed., ch. 7), so moving part of an expression onto them leaves every
// result bit unchanged.  Operands or results outside the normal range (zero
// results of multiplication, subnormals, infinities, NaN, overflow) take the
// hardware instruction instead.
//
// SoftDouble wraps a double whose + and * go through these routines; the
// exact-order FP64 kernels instantiate their arithmetic with it where the
// integer pipes have room.
#pragma once

#include <cstdint>
#if defined(__CUDACC__)
#include <cuda_runtime.h>
#endif

namespace cfd {
namespace soft {

#if defined(__CUDA_ARCH__)
#define CFD_SOFT_HD __device__ __forceinline__
#else
#define CFD_SOFT_HD inline
#endif

constexpr uint64_t kSign = 0x8000000000000000ULL;
constexpr uint64_t kAbs = 0x7fffffffffffffffULL;
constexpr uint64_t kFrac = 0x000fffffffffffffULL;
constexpr uint64_t kHidden = 0x0010000000000000ULL;

CFD_SOFT_HD uint64_t bits(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    __builtin_memcpy(&u, &x, 8);
    return u;
#endif
}

CFD_SOFT_HD double from_bits(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    __builtin_memcpy(&x, &u, 8);
    return x;
#endif
}

CFD_SOFT_HD int clz64(uint64_t x)
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// High 64 bits of the 128-bit product.
CFD_SOFT_HD uint64_t mulhi64(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// Hardware operations for the rare operands.
CFD_SOFT_HD double hw_add(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    volatile double r = a + b;
    return r;
#endif
}

CFD_SOFT_HD double hw_mul(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    volatile double r = a * b;
    return r;
#endif
}

// a + b.  Fast path: both operands finite, the larger one normal, the
// smaller one normal or zero, and a normal (or exactly zero) result.
CFD_SOFT_HD double add(double a, double b)
{
    const uint64_t ua = bits(a), ub = bits(b);
    // order by magnitude: |x| >= |y|
    const bool swap = (ub & kAbs) > (ua & kAbs);
    const uint64_t ux = swap ? ub : ua, uy = swap ? ua : ub;
    const uint64_t mx = ux & kAbs, my = uy & kAbs;
    const int ex = (int)(mx >> 52), ey = (int)(my >> 52);
    if (my == 0) {
        // y is +-0: x, with the sign rule of (+-0) + (+-0)
        if (mx != 0) return from_bits(ux);
        return from_bits(ux & uy);
    }
    if (ex == 0x7ff || ey == 0) return hw_add(a, b);   // inf/nan, or a subnormal smaller operand
    // significands with 10 guard bits: leading bit at 62
    const uint64_t fx = ((mx & kFrac) | kHidden) << 10;
    uint64_t fy = ((my & kFrac) | kHidden) << 10;
    const int d = ex - ey;
    if (d >= 64) {
        fy = 1;   // only the sticky bit survives
    } else if (d > 0) {
        const uint64_t lost = fy << (64 - d);
        fy = (fy >> d) | (lost != 0 ? 1ULL : 0ULL);
    }
    uint64_t s;
    int e = ex;
    if (((ux ^ uy) & kSign) == 0) {
        s = fx + fy;                       // < 2^64
        if (s >> 63) {                     // renormalise to bit 62, keeping the sticky bit
            s = (s >> 1) | (s & 1);
            e += 1;
        }
    } else {
        s = fx - fy;                       // >= 0
        if (s == 0) return 0.0;            // exact cancellation: +0 in round-to-nearest
        const int sh = clz64(s) - 1;       // bring the leading bit to 62
        s <<= sh;
        e -= sh;
    }
    // s in [2^62, 2^63): significand bits 62..10, rounding bits 9..0
    uint64_t m = s >> 10;
    const uint64_t rem = s & 0x3ff;
    m += (rem > 0x200 || (rem == 0x200 && (m & 1))) ? 1 : 0;
    if (e <= 0 || e >= 0x7ff) return hw_add(a, b);   // subnormal or overflowing result
    // (e - 1) << 52 plus the significand with its hidden bit; a rounding carry
    // to 2^53 moves into the exponent field by itself.
    const uint64_t r = ((uint64_t)(e - 1) << 52) + m;
    if ((r >> 52) >= 0x7ff) return hw_add(a, b);
    return from_bits((ux & kSign) | r);
}

// a * b.  Fast path: both operands normal (or one zero with the other
// finite) and a normal result.
CFD_SOFT_HD double mul(double a, double b)
{
    const uint64_t ua = bits(a), ub = bits(b);
    const uint64_t sign = (ua ^ ub) & kSign;
    const int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
    if ((ua & kAbs) == 0 || (ub & kAbs) == 0) {
        if (ea == 0x7ff || eb == 0x7ff) return hw_mul(a, b);   // 0 * inf, nan
        return from_bits(sign);
    }
    if (ea == 0 || eb == 0 || ea == 0x7ff || eb == 0x7ff) return hw_mul(a, b);
    const uint64_t fa = ((ua & kFrac) | kHidden) << 11;   // leading bit at 63
    const uint64_t fb = ((ub & kFrac) | kHidden) << 11;
    uint64_t hi = mulhi64(fa, fb);                        // product in [2^126, 2^128) over 2^64
    uint64_t lo = fa * fb;
    int e = ea + eb - 1023;
    if (hi >> 63) {
        e += 1;
    } else {                                              // bring the leading bit to 63
        hi = (hi << 1) | (lo >> 63);
        lo <<= 1;
    }
    // significand = bits 63..11 of hi; rounding bits 10..0, sticky bit jammed into bit 0
    uint64_t m = hi >> 11;
    const uint64_t rem = (hi & 0x7ff) | (lo != 0 ? 1ULL : 0ULL);
    m += (rem > 0x400 || (rem == 0x400 && (m & 1))) ? 1 : 0;
    if (e <= 0) return hw_mul(a, b);                      // subnormal or zero result
    const uint64_t r = ((uint64_t)(e - 1) << 52) + m;
    if ((r >> 52) >= 0x7ff) return hw_mul(a, b);          // overflow
    return from_bits(sign | r);
}

// A double whose + and * run on the routines above (same bits as the
// hardware instructions); /, sqrt and comparisons stay in hardware FP64.
// a - b is a + (-b), which IEEE 754 defines to be the same value.
struct SoftDouble {
    double v;
    SoftDouble() = default;
    CFD_SOFT_HD SoftDouble(double x) : v(x) {}
    CFD_SOFT_HD operator double() const { return v; }
};

CFD_SOFT_HD SoftDouble operator+(SoftDouble a, SoftDouble b) { return add(a.v, b.v); }
CFD_SOFT_HD SoftDouble operator+(SoftDouble a, double b) { return add(a.v, b); }
CFD_SOFT_HD SoftDouble operator+(double a, SoftDouble b) { return add(a, b.v); }
CFD_SOFT_HD SoftDouble operator-(SoftDouble a, SoftDouble b) { return add(a.v, -b.v); }
CFD_SOFT_HD SoftDouble operator-(SoftDouble a, double b) { return add(a.v, -b); }
CFD_SOFT_HD SoftDouble operator-(double a, SoftDouble b) { return add(a, -b.v); }
CFD_SOFT_HD SoftDouble operator-(SoftDouble a) { return SoftDouble(-a.v); }
CFD_SOFT_HD SoftDouble operator*(SoftDouble a, SoftDouble b) { return mul(a.v, b.v); }
CFD_SOFT_HD SoftDouble operator*(SoftDouble a, double b) { return mul(a.v, b); }
CFD_SOFT_HD SoftDouble operator*(double a, SoftDouble b) { return mul(a, b.v); }

}  // namespace soft
}  // namespace cfd

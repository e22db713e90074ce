// div_cases.h -- operand pairs (x, b) for checking x / b: random bit
// patterns of every class, magnitudes of a flow solution, quotients within
// ~2^-53 ulp of a rounding midpoint (for odd 54-bit M and small c,
// B = c/M mod 2^54 gives B*M = K*2^54 + c, and K/B lies c/(2B) ulp from
// the midpoint M*2^-54), exact quotients, quotients at and next to a power
// of two, zero numerators, power-of-two divisors, extreme exponents, and the
// special values.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace divcases {

struct Rng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);   // splitmix64
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
};

inline double from_bits(uint64_t u)
{
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

inline uint64_t to_bits(double x)
{
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
}

inline double ordinary(Rng &r)
{
    return std::ldexp((double)(r.next() >> 11), -53 + (int)(r.next() % 40) - 20) * ((r.next() & 1) ? -1.0 : 1.0);
}

// M^-1 mod 2^64 for odd M (Newton iteration on the 2-adic inverse)
inline uint64_t inv_odd(uint64_t m)
{
    uint64_t x = m;
    for (int i = 0; i < 6; ++i) x *= 2 - m * x;
    return x;
}

inline bool hard_pair(Rng &r, double &x, double &b)
{
    const uint64_t mask54 = (1ULL << 54) - 1;
    const uint64_t M = ((1ULL << 53) | (r.next() & ((1ULL << 53) - 1))) | 1ULL;   // odd, [2^53, 2^54)
    const uint64_t c = r.next() % 64 + 1;
    const bool below = r.next() & 1;
    const uint64_t B = ((below ? c : (0 - c)) * inv_odd(M)) & mask54;   // B*M = +-c mod 2^54
    if (B < (1ULL << 52) || B >= (1ULL << 53)) return false;
    const unsigned __int128 P = (unsigned __int128)B * M;
    const uint64_t K = (uint64_t)((below ? P - c : P + c) >> 54);
    if (K >= (1ULL << 53) || K == 0) return false;
    const int s1 = (int)(r.next() % 200) - 100, s2 = (int)(r.next() % 200) - 100;
    x = std::ldexp((double)K, s1) * ((r.next() & 1) ? -1.0 : 1.0);
    b = std::ldexp((double)B, s2) * ((r.next() & 1) ? -1.0 : 1.0);
    return true;
}

// n rounds of every class
inline void make(long n, uint64_t seed, std::vector<double> &X, std::vector<double> &B)
{
    Rng r{seed};
    auto add = [&](double x, double b) {
        X.push_back(x);
        B.push_back(b);
    };
    for (long i = 0; i < n; ++i) {
        add(from_bits(r.next()), from_bits(r.next()));
        add(ordinary(r), ordinary(r));
        for (int t = 0; t < 4; ++t) {
            double x, b;
            if (hard_pair(r, x, b)) add(x, b);
        }
        {
            const double q = std::ldexp((double)(r.next() >> 40), -(int)(r.next() % 30));
            const double b = std::ldexp((double)(r.next() >> 35), -(int)(r.next() % 30)) + 1.0;
            add(q * b, b);
        }
        add((r.next() & 1) ? 0.0 : -0.0, ordinary(r));   // zero numerators
        {   // quotients at the ends of a binade: exact powers of two and their neighbours
            const double b = ordinary(r);
            const int k = (int)(r.next() % 40) - 20, m = (int)(r.next() % 7) - 3;
            add(std::ldexp(b, k), b);
            add(std::ldexp(std::nextafter(b, m < 0 ? 0.0 : 2.0 * b), k), b);
            add(std::ldexp(b, k) * (1.0 + m * 0x1p-52), b);
            add(std::ldexp(b, k), b * (1.0 + m * 0x1p-52));
        }
        // power-of-two divisors, subnormal to the largest
        add(ordinary(r), std::ldexp((r.next() & 1) ? 1.0 : -1.0, (int)(r.next() % 2098) - 1074));
        {
            const int e1 = (int)(r.next() % 2046) + 1, e2 = (int)(r.next() % 2046) + 1;
            add(from_bits(((uint64_t)e1 << 52) | (r.next() & 0x000fffffffffffffULL)),
                from_bits(((uint64_t)e2 << 52) | (r.next() & 0x000fffffffffffffULL)));
        }
    }
    const double sp[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1.0, -1.0, 4.9e-324, 2.2250738585072014e-308,
                         1.7976931348623157e308, 0.5, 3.0, 0.4, 1e-300, 1e300};
    for (double a : sp)
        for (double c : sp) add(a, c);
}

}  // namespace divcases

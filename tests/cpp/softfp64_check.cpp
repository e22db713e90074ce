// softfp64_check.cpp -- the integer-pipe binary64 add/mul against the host's
// IEEE arithmetic (round to nearest even), bit for bit, on operand classes
// that exercise every path: random bit patterns, close exponents
// (cancellation), far exponents (sticky bits), exact ties, products near the
// overflow and underflow thresholds, zeros, subnormals, inf, NaN.
//
//   softfp64_check <cases per class> <seed>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "softfp64.cuh"

using cfd::soft::bits;
using cfd::soft::from_bits;

namespace {

uint64_t s64;
uint64_t rnd()
{
    // splitmix64
    uint64_t z = (s64 += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double with_exp(int e, uint64_t frac_bits, bool neg)
{
    return from_bits((neg ? cfd::soft::kSign : 0) | ((uint64_t)e << 52) | (frac_bits & cfd::soft::kFrac));
}

bool same(double x, double y)
{
    if (std::isnan(x) && std::isnan(y)) return true;
    return bits(x) == bits(y);
}

long fails = 0;
void check(double a, double b)
{
    volatile double va = a, vb = b;
    const double hs = va + vb, hm = va * vb, hd = va - vb;
    const double ss = cfd::soft::add(a, b), sm = cfd::soft::mul(a, b);
    const double sd = (double)(cfd::soft::SoftDouble(a) - cfd::soft::SoftDouble(b));
    if (!same(hs, ss) || !same(hm, sm) || !same(hd, sd)) {
        if (fails < 10)
            std::printf("MISMATCH a=%016llx b=%016llx add %016llx/%016llx mul %016llx/%016llx sub %016llx/%016llx\n",
                        (unsigned long long)bits(a), (unsigned long long)bits(b), (unsigned long long)bits(hs),
                        (unsigned long long)bits(ss), (unsigned long long)bits(hm), (unsigned long long)bits(sm),
                        (unsigned long long)bits(hd), (unsigned long long)bits(sd));
        ++fails;
    }
}

}  // namespace

int main(int argc, char **argv)
{
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    s64 = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1;
    long total = 0;
    for (long i = 0; i < n; ++i) {
        // 1. random bit patterns (all classes, mostly large exponent gaps)
        check(from_bits(rnd()), from_bits(rnd()));
        // 2. close exponents, both signs: cancellation and carries
        {
            const int e = 1 + (int)(rnd() % 2046);
            const int e2 = e + (int)(rnd() % 5) - 2;
            if (e2 >= 1 && e2 <= 2046) check(with_exp(e, rnd(), rnd() & 1), with_exp(e2, rnd(), rnd() & 1));
        }
        // 3. exponent gaps 0..70 (sticky bits; trailing zeros give exact ties)
        {
            const int e = 900 + (int)(rnd() % 200);
            const int g = (int)(rnd() % 71);
            uint64_t fb = rnd();
            if (rnd() & 1) fb &= ~((1ULL << (rnd() % 52)) - 1);
            check(with_exp(e, rnd(), rnd() & 1), with_exp(e - g, fb, rnd() & 1));
        }
        // 4. nearly equal magnitudes, opposite signs (massive cancellation)
        {
            const double a = with_exp(1 + (int)(rnd() % 2046), rnd(), false);
            const double b = from_bits((bits(a) + (rnd() % 64) - 32) ^ cfd::soft::kSign);
            check(a, b);
        }
        // 5. products near overflow / underflow; short significands (exact products, ties)
        {
            const int ea = 1 + (int)(rnd() % 2046);
            const int target = (rnd() & 1) ? 2046 - (int)(rnd() % 4) : 1 + (int)(rnd() % 4);
            int eb = target - ea + 1023;
            if (eb < 1) eb = 1;
            if (eb > 2046) eb = 2046;
            uint64_t fa = rnd(), fb = rnd();
            if (rnd() & 1) fa &= ~((1ULL << 30) - 1);
            if (rnd() & 1) fb &= ~((1ULL << 26) - 1);
            check(with_exp(ea, fa, rnd() & 1), with_exp(eb, fb, rnd() & 1));
        }
        // 6. sums near overflow and near the subnormal boundary
        {
            const int e = (rnd() & 1) ? 2046 : 1 + (int)(rnd() % 3);
            check(with_exp(e, rnd(), rnd() & 1), with_exp(e - (int)(rnd() % 2), rnd(), rnd() & 1));
        }
        // 7. magnitudes of a flow solution
        {
            const double a = std::ldexp((double)(rnd() >> 11), -53 + (int)(rnd() % 20) - 10) * ((rnd() & 1) ? -1 : 1);
            const double b = std::ldexp((double)(rnd() >> 11), -53 + (int)(rnd() % 20) - 10) * ((rnd() & 1) ? -1 : 1);
            check(a, b);
        }
        total += 7;
    }
    const double sp[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1.0, -1.0, 4.9e-324, -4.9e-324, 2.2250738585072014e-308,
                         -2.2250738585072014e-308, 1.7976931348623157e308, -1.7976931348623157e308, 0.5, 3.0};
    for (double a : sp)
        for (double b : sp) {
            check(a, b);
            ++total;
        }
    std::printf("softfp64_check: %ld cases, %ld mismatches\n", total, fails);
    return fails == 0 ? 0 : 1;
}

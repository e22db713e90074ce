// exact_div_check.cpp -- cfd::xdiv::div(x, b, 1/b) against the host's IEEE
// division x / b, bit for bit, on the pairs of div_cases.h.  Prints the
// share of plain-case quotients (no fallback division).
//
//   exact_div_check <rounds> <seed>
#include <cstdio>
#include <cstdlib>

#include "div_cases.h"
#include "exact_div.cuh"

int main(int argc, char **argv)
{
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    const uint64_t seed = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1;
    std::vector<double> X, B;
    divcases::make(n, seed, X, B);
    long fails = 0, plain = 0;
    for (size_t i = 0; i < X.size(); ++i) {
        volatile double vx = X[i], vb = B[i], one = 1.0;
        const double want = vx / vb, y = one / vb;
        const double got = cfd::xdiv::div(X[i], B[i], y);
        bool ok;
        cfd::xdiv::quotient(X[i], B[i], y, ok);
        plain += ok;
        const bool same = divcases::to_bits(got) == divcases::to_bits(want) || (std::isnan(got) && std::isnan(want));
        if (!same) {
            if (fails < 10)
                std::printf("MISMATCH x=%016llx b=%016llx want %016llx got %016llx\n",
                            (unsigned long long)divcases::to_bits(X[i]), (unsigned long long)divcases::to_bits(B[i]),
                            (unsigned long long)divcases::to_bits(want), (unsigned long long)divcases::to_bits(got));
            ++fails;
        }
    }
    std::printf("exact_div_check: %zu cases, %ld mismatches, plain case %.4f\n", X.size(), fails,
                (double)plain / (double)X.size());
    return fails == 0 ? 0 : 1;
}

// exact_div_check.cpp -- cfd::xdiv::div(x, b, 1/b) against the host's IEEE
// division x / b, bit for bit, on the pairs of div_cases.h, and
// cfd::xdiv::scale2<K>(x) against x * 2^K and the integer-pipe reciprocal
// cfd::xdiv::rcp_int_i(x) against 1 / x on every operand of those pairs.
// Prints the share of plain-case quotients (no fallback division).
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
    long sfails = 0, scases = 0;
    auto check = [&](double x, double got, double c) {
        volatile double vx = x, vc = c;
        const double want = vx * vc;
        ++scases;
        if (!(divcases::to_bits(got) == divcases::to_bits(want) || (std::isnan(got) && std::isnan(want)))) {
            if (sfails < 10)
                std::printf("SCALE2 MISMATCH x=%016llx c=%g want %016llx got %016llx\n",
                            (unsigned long long)divcases::to_bits(x), c, (unsigned long long)divcases::to_bits(want),
                            (unsigned long long)divcases::to_bits(got));
            ++sfails;
        }
    };
    for (const std::vector<double> *V : {&X, &B})
        for (double x : *V) {
            check(x, cfd::xdiv::scale2<1>(x), 2.0);
            check(x, cfd::xdiv::scale2<2>(x), 4.0);
            check(x, cfd::xdiv::scale2<3>(x), 8.0);
            check(x, cfd::xdiv::scale2<-1>(x), 0.5);
            check(x, cfd::xdiv::scale2<-2>(x), 0.25);
            check(x, cfd::xdiv::scale2<-3>(x), 0.125);
        }
    std::printf("scale2: %ld cases, %ld scale2 mismatches\n", scases, sfails);
    long pfails = 0, pcases = 0;
    auto pcheck = [&](double x, double got, double c) {
        volatile double vx = x, vc = c;
        const double want = vc / vx;
        ++pcases;
        if (!(divcases::to_bits(got) == divcases::to_bits(want) || (std::isnan(got) && std::isnan(want)))) {
            if (pfails < 10)
                std::printf("POW2_OVER MISMATCH x=%016llx c=%g want %016llx got %016llx\n",
                            (unsigned long long)divcases::to_bits(x), c, (unsigned long long)divcases::to_bits(want),
                            (unsigned long long)divcases::to_bits(got));
            ++pfails;
        }
    };
    for (const std::vector<double> *V : {&X, &B})
        for (double x : *V) {
            pcheck(x, cfd::xdiv::pow2_over<-4>(x), 0.0625);
            pcheck(x, cfd::xdiv::pow2_over<-1>(x), 0.5);
            pcheck(x, cfd::xdiv::pow2_over<3>(x), 8.0);
        }
    std::printf("pow2_over: %ld cases, %ld pow2_over mismatches\n", pcases, pfails);
    // the integer-pipe reciprocal (rcp_int_i) where it accepts the operand
    long rfails = 0, rcases = 0, rplain = 0;
    for (const std::vector<double> *V : {&X, &B})
        for (double x : *V) {
            volatile double one = 1.0, vx = x;
            const double want = one / vx;
            bool ok;
            const double got = cfd::xdiv::rcp_int_i(x, ok);
            ++rcases;
            if (!ok) continue;
            ++rplain;
            if (divcases::to_bits(got) != divcases::to_bits(want)) {
                if (rfails < 10)
                    std::printf("RCP MISMATCH x=%016llx want %016llx got %016llx\n", (unsigned long long)divcases::to_bits(x),
                                (unsigned long long)divcases::to_bits(want), (unsigned long long)divcases::to_bits(got));
                ++rfails;
            }
        }
    // and densely at both ends of the significand range (the reciprocal's
    // significand next to 2^53 and to 2^52), at five exponents
    for (uint64_t f = 1; f < 100000; ++f)
        for (uint64_t e : {(uint64_t)1, (uint64_t)500, (uint64_t)1023, (uint64_t)1800, (uint64_t)2044})
            for (uint64_t F : {f, (uint64_t)0x0010000000000000ULL - f, f << 20}) {
                const double x = divcases::from_bits((e << 52) | F);
                volatile double one = 1.0, vx = x;
                const double want = one / vx;
                bool ok;
                const double got = cfd::xdiv::rcp_int_i(x, ok);
                ++rcases;
                if (!ok) continue;
                ++rplain;
                if (divcases::to_bits(got) != divcases::to_bits(want)) ++rfails;
            }
    std::printf("rcp_int_i: %ld cases, plain case %.4f, %ld rcp mismatches\n", rcases, (double)rplain / (double)rcases,
                rfails);
    return fails == 0 && sfails == 0 && pfails == 0 && rfails == 0 ? 0 : 1;
}

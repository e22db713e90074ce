// lattice_map_check.cpp -- the host-side lattice detection of the library
// (csrc/lattice_host.h: map_lattice, faces_single_valued,
// lattice_geometry_soa) on a reference table read from raw files, without
// a GPU.  Prints one line:
//   ok <0|1> ni nj nk per locdirs faces <0|1> row_of_sum soa_sum
// where row_of_sum = sum over lattice nodes n of n * row_of[n] (mod 2^61 - 1)
// and soa_sum is the sum of the converted geometry.
//
//   lattice_map_check <dir> <g_node> <sd_node>
// <dir>/grid.bin (cfd_grid_t rows 0..g_node), metric.bin, deter.bin, det.bin.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "lattice_host.h"

template <class T>
static std::vector<T> read_all(const std::string &path)
{
    std::vector<T> v;
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return v;
    T x;
    while (std::fread(&x, sizeof x, 1, f) == 1) v.push_back(x);
    std::fclose(f);
    return v;
}

int main(int argc, char **argv)
{
    if (argc < 4) return 2;
    const std::string dir = argv[1];
    auto grid = read_all<cfd_grid_t>(dir + "/grid.bin");
    auto metric = read_all<cfd_metric_t>(dir + "/metric.bin");
    auto deter = read_all<cfd_determ_t>(dir + "/deter.bin");
    auto det = read_all<double>(dir + "/det.bin");
    const cfd_geometry_t g{std::atoi(argv[2]), std::atoi(argv[3]), grid.data(), det.data(), deter.data(),
                           metric.data()};
    cfd::LatticeMap m;
    const bool ok = cfd::map_lattice(&g, m);
    const bool faces = ok && cfd::faces_single_valued(&g, m);
    const unsigned long long P = (1ULL << 61) - 1;
    unsigned long long rs = 0;
    double soa = 0.0;
    if (ok) {
        for (size_t n = 0; n < m.row_of.size(); ++n) rs = (rs + (unsigned long long)n * (unsigned)m.row_of[n]) % P;
        cfd::HostDoubles a, b, c, d;
        cfd::lattice_geometry_soa(&g, m, a, b, c, d);
        for (auto *v : {&a, &b, &c, &d})
            for (auto &x : *v) soa += x.v;
    }
    std::printf("ok %d %d %d %d %d %d faces %d %llu %.17g\n", ok, m.ni, m.nj, m.nk, m.per, m.locdirs, faces, rs, soa);
    return 0;
}

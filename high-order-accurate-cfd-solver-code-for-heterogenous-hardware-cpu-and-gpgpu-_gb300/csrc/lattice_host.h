// lattice_host.h -- host-side checks that decide whether a reference
// neighbour table can run on the face-based lattice kernels, and the
// conversion of its geometry to the lattice layout.
#pragma once

#include <cmath>
#include <vector>

#include "cfd_rhs.h"

namespace cfd {

inline int nb_of(const cfd_grid_t &g, int slot)
{
    switch (slot) {
    case 0: return g.N0;
    case 1: return g.N1;
    case 2: return g.N2;
    case 3: return g.N3;
    case 4: return g.N4;
    default: return g.N5;
    }
}

// Lattice detection: rows 1..N, row(i,j,k) = 1 + i + ni*(j + nj*k) with
// N1/N3 = +-i, N0/N2 = +-j, N4/N5 = +-k, periodic wrap, loc == 0.
inline bool detect_lattice(const cfd_geometry_t *g, int &ni, int &nj, int &nk)
{
    const int N = g->sd_node;
    if (g->g_node != N || N < 1) return false;
    auto cycle = [&](int slot) {
        int r = 1, len = 0;
        do {
            r = nb_of(g->grid[r], slot);
            ++len;
            if (r < 1 || r > N || len > N) return -1;
        } while (r != 1);
        return len;
    };
    ni = cycle(1);
    if (ni <= 0) return false;
    const int cj = cycle(0), ck = cycle(4);
    if (cj <= 0 || ck <= 0) return false;
    nj = cj;
    nk = ck;
    if ((long long)ni * nj * nk != N) return false;
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                auto row = [&](int a, int b, int c) {
                    a = (a % ni + ni) % ni;
                    b = (b % nj + nj) % nj;
                    c = (c % nk + nk) % nk;
                    return 1 + a + ni * (b + nj * c);
                };
                const cfd_grid_t &r = g->grid[row(i, j, k)];
                if (r.loc != 0) return false;
                if (r.N1 != row(i + 1, j, k) || r.N3 != row(i - 1, j, k) || r.N0 != row(i, j + 1, k)
                    || r.N2 != row(i, j - 1, k) || r.N4 != row(i, j, k + 1) || r.N5 != row(i, j, k - 1))
                    return false;
            }
    return true;
}

// The face-based path evaluates face n+1/2 from node n's +d data; the
// reference evaluates it again from node n+1's -d data.  Both must agree.
inline bool faces_single_valued(const cfd_geometry_t *g)
{
    const int N = g->sd_node;
    const double tol = 1e-13;
    auto close = [&](double a, double b, double scale) { return std::fabs(a - b) <= tol * scale; };
    for (int r = 1; r <= N; ++r) {
        const double *m = (const double *)&g->metric[r];
        const double *dd = (const double *)&g->deter[r];
        const int slots[3] = {1, 0, 4};
        for (int d = 0; d < 3; ++d) {
            const int nbr = nb_of(g->grid[r], slots[d]);
            const double *mn = (const double *)&g->metric[nbr];
            const double *dn = (const double *)&g->deter[nbr];
            double scale = 0;
            for (int c = 0; c < 3; ++c) scale = std::fmax(scale, std::fabs(m[9 * (1 + 2 * d) + 3 * d + c]));
            for (int c = 0; c < 3; ++c)
                if (!close(m[9 * (1 + 2 * d) + 3 * d + c], mn[9 * (2 + 2 * d) + 3 * d + c], scale)) return false;
            if (!close(dd[2 * d], dn[2 * d + 1], std::fabs(dd[2 * d]))) return false;
        }
    }
    return true;
}

// Geometry of a lattice (rows 1..N of the reference arrays) as SoA host
// arrays: m9 [9][N], det [N], fm [3 dir][3 comp][N] (metric of face n+1/2),
// fdet [3][N] (det of face n+1/2).
inline void lattice_geometry_soa(const cfd_geometry_t *g, size_t N, std::vector<double> &m9, std::vector<double> &det,
                                 std::vector<double> &fm, std::vector<double> &fdet)
{
    m9.assign(9 * N, 0.0);
    det.assign(N, 0.0);
    fm.assign(9 * N, 0.0);
    fdet.assign(3 * N, 0.0);
    for (size_t n = 0; n < N; ++n) {
        const double *m = (const double *)&g->metric[n + 1];
        const double *dd = (const double *)&g->deter[n + 1];
        for (int q = 0; q < 9; ++q) m9[q * N + n] = m[q];
        det[n] = g->det[n + 1];
        for (int d = 0; d < 3; ++d) {
            for (int c = 0; c < 3; ++c) fm[(d * 3 + c) * N + n] = m[9 * (1 + 2 * d) + 3 * d + c];
            fdet[d * N + n] = dd[2 * d];
        }
    }
}

}  // namespace cfd

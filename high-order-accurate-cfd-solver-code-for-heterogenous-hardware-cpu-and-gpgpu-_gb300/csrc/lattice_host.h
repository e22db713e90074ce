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

// Largest lattice the face-based kernels address: they index component
// arrays of up to 15 components as c * N + n in 32-bit arithmetic.
constexpr long long kLatticeMaxNodes = 2147483647LL / 15;

// A reference neighbour table seen as a lattice: node n = i + ni*(j + nj*k)
// is reference row row_of[n].  Direction d (0 = i via N1/N3, 1 = j via
// N0/N2, 2 = k via N4/N5) is either periodic (the +d chain closes) or
// non-periodic with its ends pointing at themselves (the reference's
// outermost ghosts), in which case owned nodes (rows 1..sd_node, loc != 100)
// must lie at least three nodes inside each end and ghost rows carry
// loc 100.
struct LatticeMap {
    int ni = 0, nj = 0, nk = 0;
    int per = 7;                        // bit d: direction d periodic
    int locdirs = 0;                    // bit d: an owned node has a ghost within 2 along d
    std::vector<int32_t> row_of;        // n -> reference row
    std::vector<int32_t> n_of_row;      // reference row -> n (-1: not a lattice node)
    std::vector<unsigned char> loc;     // loc code of node n (non-periodic lattices)
    bool ghosted() const { return per != 7; }
    int extent(int d) const { return d == 0 ? ni : (d == 1 ? nj : nk); }
};

constexpr int kSlotPlus[3] = {1, 0, 4};
constexpr int kSlotMinus[3] = {3, 2, 5};

inline bool map_lattice(const cfd_geometry_t *g, LatticeMap &m)
{
    const int R = g->g_node;   // rows 1..R
    if (R < 1 || g->sd_node < 1 || g->sd_node > R) return false;
    auto nbr = [&](int r, int slot) { return nb_of(g->grid[r], slot); };
    int ext[3] = {0, 0, 0}, per = 0;
    int origin = 1;
    for (int d = 0; d < 3; ++d) {
        // periodic: the +d chain from row 1 closes on row 1
        int r = 1, len = 0;
        bool closed = false;
        while (len <= R) {
            r = nbr(r, kSlotPlus[d]);
            ++len;
            if (r < 1 || r > R) break;
            if (r == 1) {
                closed = true;
                break;
            }
        }
        if (closed) {
            ext[d] = len;
            per |= 1 << d;
        }
    }
    for (int d = 0; d < 3; ++d) {
        if (per >> d & 1) continue;
        // non-periodic: walk to the -d end (a row pointing at itself)
        int r = origin, steps = 0;
        while (true) {
            const int q = nbr(r, kSlotMinus[d]);
            if (q < 1 || q > R || ++steps > R) return false;
            if (q == r) break;
            r = q;
        }
        origin = r;
        int len = 1;
        while (true) {
            const int q = nbr(r, kSlotPlus[d]);
            if (q < 1 || q > R || len > R) return false;
            if (q == r) break;
            r = q;
            ++len;
        }
        ext[d] = len;
    }
    if ((long long)ext[0] * ext[1] * ext[2] != R) return false;
    m.ni = ext[0];
    m.nj = ext[1];
    m.nk = ext[2];
    m.per = per;
    m.row_of.assign(R, 0);
    m.n_of_row.assign(R + 1, -1);
    // rows by walking +i, +j, +k from the origin
    int rk = origin;
    for (int k = 0; k < m.nk; ++k) {
        int rj = rk;
        for (int j = 0; j < m.nj; ++j) {
            int ri = rj;
            for (int i = 0; i < m.ni; ++i) {
                const int n = i + m.ni * (j + m.nj * k);
                if (ri < 1 || ri > R || m.n_of_row[ri] >= 0) return false;
                m.row_of[n] = ri;
                m.n_of_row[ri] = n;
                ri = nbr(ri, kSlotPlus[0]);
            }
            rj = nbr(rj, kSlotPlus[1]);
        }
        rk = nbr(rk, kSlotPlus[2]);
    }
    // every neighbour is the lattice neighbour (wrapped or clamped)
    auto step = [&](int c, int o, int d) {
        const int e = m.extent(d);
        if (per >> d & 1) return ((c + o) % e + e) % e;
        return c + o < 0 ? 0 : (c + o >= e ? e - 1 : c + o);
    };
    const bool ghosted = per != 7;
    if (ghosted) m.loc.assign(R, 0);
    for (int k = 0; k < m.nk; ++k)
        for (int j = 0; j < m.nj; ++j)
            for (int i = 0; i < m.ni; ++i) {
                const int n = i + m.ni * (j + m.nj * k);
                const cfd_grid_t &row = g->grid[m.row_of[n]];
                const int c[3] = {i, j, k};
                for (int d = 0; d < 3; ++d)
                    for (int o : {-1, 1}) {
                        int cc[3] = {i, j, k};
                        cc[d] = step(c[d], o, d);
                        const int want = m.row_of[cc[0] + m.ni * (cc[1] + m.nj * cc[2])];
                        if (nb_of(row, o > 0 ? kSlotPlus[d] : kSlotMinus[d]) != want) return false;
                    }
                const bool owned = m.row_of[n] <= g->sd_node;
                if (!ghosted) {
                    if (row.loc != 0 || g->g_node != g->sd_node) return false;
                    continue;
                }
                if (owned == (row.loc == 100) || row.loc < 0 || row.loc > 100) return false;
                m.loc[n] = (unsigned char)row.loc;
                if (owned)
                    for (int d = 0; d < 3; ++d)
                        if (!(per >> d & 1) && (c[d] < 3 || c[d] > m.extent(d) - 4)) return false;
            }
    if (ghosted)
        for (int k = 0; k < m.nk; ++k)
            for (int j = 0; j < m.nj; ++j)
                for (int i = 0; i < m.ni; ++i) {
                    const int n = i + m.ni * (j + m.nj * k);
                    if (m.loc[n] == 100) continue;
                    const int c[3] = {i, j, k};
                    for (int d = 0; d < 3; ++d)
                        for (int o : {-2, -1, 1, 2}) {
                            int cc[3] = {i, j, k};
                            cc[d] = step(c[d], o, d);
                            if (m.loc[cc[0] + m.ni * (cc[1] + m.nj * cc[2])] == 100) m.locdirs |= 1 << d;
                        }
                }
    return true;
}

// The face-based path evaluates face n+1/2 from node n's +d data; the
// reference evaluates it again from node n+1's -d data.  Both must agree on
// every face the path computes.
inline bool faces_single_valued(const cfd_geometry_t *g, const LatticeMap &m)
{
    const double tol = 1e-13;
    auto close = [&](double a, double b, double scale) { return std::fabs(a - b) <= tol * scale; };
    for (int k = 0; k < m.nk; ++k)
        for (int j = 0; j < m.nj; ++j)
            for (int i = 0; i < m.ni; ++i) {
                const int n = i + m.ni * (j + m.nj * k);
                const int r = m.row_of[n];
                const double *mr = (const double *)&g->metric[r];
                const double *dd = (const double *)&g->deter[r];
                const int c[3] = {i, j, k};
                for (int d = 0; d < 3; ++d) {
                    if (!(m.per >> d & 1) && (c[d] < 2 || c[d] > m.extent(d) - 4)) continue;
                    const int nbr = nb_of(g->grid[r], kSlotPlus[d]);
                    const double *mn = (const double *)&g->metric[nbr];
                    const double *dn = (const double *)&g->deter[nbr];
                    double scale = 0;
                    for (int q = 0; q < 3; ++q) scale = std::fmax(scale, std::fabs(mr[9 * (1 + 2 * d) + 3 * d + q]));
                    for (int q = 0; q < 3; ++q)
                        if (!close(mr[9 * (1 + 2 * d) + 3 * d + q], mn[9 * (2 + 2 * d) + 3 * d + q], scale)) return false;
                    if (!close(dd[2 * d], dn[2 * d + 1], std::fabs(dd[2 * d]))) return false;
                }
            }
    return true;
}

// Geometry of a lattice as SoA host arrays: m9 [9][N], det [N], fm [3 dir][3
// comp][N] (metric of face n+1/2), fdet [3][N] (det of face n+1/2).
inline void lattice_geometry_soa(const cfd_geometry_t *g, const LatticeMap &map, std::vector<double> &m9,
                                 std::vector<double> &det, std::vector<double> &fm, std::vector<double> &fdet)
{
    const size_t N = map.row_of.size();
    m9.assign(9 * N, 0.0);
    det.assign(N, 0.0);
    fm.assign(9 * N, 0.0);
    fdet.assign(3 * N, 0.0);
    for (size_t n = 0; n < N; ++n) {
        const int r = map.row_of[n];
        const double *m = (const double *)&g->metric[r];
        const double *dd = (const double *)&g->deter[r];
        for (int q = 0; q < 9; ++q) m9[q * N + n] = m[q];
        det[n] = g->det[r];
        for (int d = 0; d < 3; ++d) {
            for (int c = 0; c < 3; ++c) fm[(d * 3 + c) * N + n] = m[9 * (1 + 2 * d) + 3 * d + c];
            fdet[d * N + n] = dd[2 * d];
        }
    }
}

}  // namespace cfd

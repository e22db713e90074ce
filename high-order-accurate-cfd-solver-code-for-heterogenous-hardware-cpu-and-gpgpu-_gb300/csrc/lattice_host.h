// lattice_host.h -- host-side checks that decide whether a reference
// neighbour table can run on the face-based lattice kernels, and the
// conversion of its geometry to the lattice layout.  The per-node passes run
// on up to 16 host threads: admitting a 160^3 lattice reads about 2 GB of
// reference geometry.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <memory>
#include <thread>
#include <vector>

#include "cfd_rhs.h"

namespace cfd {

// fn(begin, end) over [0, n) in contiguous chunks of at least 64 Ki items,
// on up to 16 threads; a thread that cannot be started runs its chunk on
// the calling thread.
template <class F>
inline void host_parallel_for(long long n, F fn)
{
    const unsigned hw = std::max(1u, std::min(std::thread::hardware_concurrency(), 16u));
    const long long T = std::max(1LL, std::min<long long>(hw, (n + 65535) / 65536));
    const long long chunk = (n + T - 1) / T;
    std::vector<std::thread> th;
    for (long long t = 1; t < T; ++t) {
        const long long b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        try {
            th.emplace_back(fn, b, e);
        } catch (...) {
            fn(b, e);
        }
    }
    fn(0LL, std::min(n, chunk));
    for (auto &x : th) x.join();
}

// std::vector element type without value-initialisation: the conversion
// writes every element, so the zero fill of a plain vector is wasted work.
template <class T>
struct NoInit {
    T v;
    NoInit() {}
};
using HostDoubles = std::vector<NoInit<double>>;
inline double *host_ptr(HostDoubles &v) { return &v.data()->v; }

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
    // rows by walking +i, +j, +k from the origin: the first row of every
    // (j, k) line, then the lines in parallel, then a serial pass that
    // rejects a row reached twice
    const int lines = m.nj * m.nk;
    std::vector<int32_t> first(lines);
    int rk = origin;
    for (int k = 0; k < m.nk; ++k) {
        int rj = rk;
        for (int j = 0; j < m.nj; ++j) {
            if (rj < 1 || rj > R) return false;
            first[j + m.nj * k] = rj;
            rj = nbr(rj, kSlotPlus[1]);
        }
        if (rk < 1 || rk > R) return false;
        rk = nbr(rk, kSlotPlus[2]);
    }
    std::atomic<bool> bad{false};
    host_parallel_for(lines, [&](long long l0, long long l1) {
        for (long long l = l0; l < l1 && !bad.load(std::memory_order_relaxed); ++l) {
            int ri = first[l];
            for (int i = 0; i < m.ni; ++i) {
                if (ri < 1 || ri > R) {
                    bad = true;
                    break;
                }
                m.row_of[i + (size_t)m.ni * l] = ri;
                ri = nbr(ri, kSlotPlus[0]);
            }
        }
    });
    if (bad) return false;
    for (int n = 0; n < R; ++n) {
        const int r = m.row_of[n];
        if (m.n_of_row[r] >= 0) return false;
        m.n_of_row[r] = n;
    }
    // every neighbour is the lattice neighbour (wrapped or clamped)
    auto step = [&](int c, int o, int d) {
        const int e = m.extent(d);
        if (per >> d & 1) return ((c + o) % e + e) % e;
        return c + o < 0 ? 0 : (c + o >= e ? e - 1 : c + o);
    };
    const bool ghosted = per != 7;
    if (ghosted) m.loc.assign(R, 0);
    // node n's coordinates
    auto coords = [&](long long n, int c[3]) {
        c[0] = (int)(n % m.ni);
        c[1] = (int)((n / m.ni) % m.nj);
        c[2] = (int)(n / ((long long)m.ni * m.nj));
    };
    host_parallel_for(R, [&](long long n0, long long n1) {
        for (long long n = n0; n < n1 && !bad.load(std::memory_order_relaxed); ++n) {
            int c[3];
            coords(n, c);
            const cfd_grid_t &row = g->grid[m.row_of[n]];
            bool ok = true;
            for (int d = 0; d < 3 && ok; ++d)
                for (int o : {-1, 1}) {
                    int cc[3] = {c[0], c[1], c[2]};
                    cc[d] = step(c[d], o, d);
                    const int want = m.row_of[cc[0] + m.ni * (cc[1] + (size_t)m.nj * cc[2])];
                    if (nb_of(row, o > 0 ? kSlotPlus[d] : kSlotMinus[d]) != want) ok = false;
                }
            const bool owned = m.row_of[n] <= g->sd_node;
            if (ok && !ghosted) ok = row.loc == 0 && g->g_node == g->sd_node;
            else if (ok) {
                ok = owned != (row.loc == 100) && row.loc >= 0 && row.loc <= 100;
                if (ok) m.loc[n] = (unsigned char)row.loc;
                if (ok && owned)
                    for (int d = 0; d < 3; ++d)
                        if (!(per >> d & 1) && (c[d] < 3 || c[d] > m.extent(d) - 4)) ok = false;
            }
            if (!ok) bad = true;
        }
    });
    if (bad) return false;
    if (ghosted) {
        std::atomic<int> dirs{0};
        host_parallel_for(R, [&](long long n0, long long n1) {
            int mine = 0;
            for (long long n = n0; n < n1; ++n) {
                if (m.loc[n] == 100) continue;
                int c[3];
                coords(n, c);
                for (int d = 0; d < 3; ++d)
                    for (int o : {-2, -1, 1, 2}) {
                        int cc[3] = {c[0], c[1], c[2]};
                        cc[d] = step(c[d], o, d);
                        if (m.loc[cc[0] + m.ni * (cc[1] + (size_t)m.nj * cc[2])] == 100) mine |= 1 << d;
                    }
            }
            dirs.fetch_or(mine);
        });
        m.locdirs = dirs.load();
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
    std::atomic<bool> bad{false};
    host_parallel_for((long long)m.row_of.size(), [&](long long n0, long long n1) {
        for (long long n = n0; n < n1 && !bad.load(std::memory_order_relaxed); ++n) {
            const int c[3] = {(int)(n % m.ni), (int)((n / m.ni) % m.nj), (int)(n / ((long long)m.ni * m.nj))};
            const int r = m.row_of[n];
            const double *mr = (const double *)&g->metric[r];
            const double *dd = (const double *)&g->deter[r];
            for (int d = 0; d < 3; ++d) {
                if (!(m.per >> d & 1) && (c[d] < 2 || c[d] > m.extent(d) - 4)) continue;
                const int nbr = nb_of(g->grid[r], kSlotPlus[d]);
                const double *mn = (const double *)&g->metric[nbr];
                const double *dn = (const double *)&g->deter[nbr];
                double scale = 0;
                for (int q = 0; q < 3; ++q) scale = std::fmax(scale, std::fabs(mr[9 * (1 + 2 * d) + 3 * d + q]));
                bool ok = close(dd[2 * d], dn[2 * d + 1], std::fabs(dd[2 * d]));
                for (int q = 0; q < 3; ++q)
                    ok = ok && close(mr[9 * (1 + 2 * d) + 3 * d + q], mn[9 * (2 + 2 * d) + 3 * d + q], scale);
                if (!ok) {
                    bad = true;
                    break;
                }
            }
        }
    });
    return !bad;
}

// Geometry of a lattice as SoA host arrays: m9 [9][N], det [N], fm [3 dir][3
// comp][N] (metric of face n+1/2), fdet [3][N] (det of face n+1/2).
inline void lattice_geometry_soa(const cfd_geometry_t *g, const LatticeMap &map, HostDoubles &m9v,
                                 HostDoubles &detv, HostDoubles &fmv, HostDoubles &fdetv)
{
    const size_t N = map.row_of.size();
    m9v.resize(9 * N);
    detv.resize(N);
    fmv.resize(9 * N);
    fdetv.resize(3 * N);
    double *m9 = host_ptr(m9v), *det = host_ptr(detv), *fm = host_ptr(fmv), *fdet = host_ptr(fdetv);
    host_parallel_for((long long)N, [&](long long n0, long long n1) {
        for (long long n = n0; n < n1; ++n) {
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
    });
}

}  // namespace cfd

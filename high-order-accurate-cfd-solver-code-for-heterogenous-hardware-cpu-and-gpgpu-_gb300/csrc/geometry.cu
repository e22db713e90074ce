// geometry.cu -- the geometry producer: the inputs the RHS path reads (node
// metrics, det, face metrics, face dets) from a node table, as the
// reference computes them once before its time loop.
//
// cfd_compact_metrics    Grid_Transformation.cpp:22-1045 (metric_term):
//                        x, y, z differentiated along every grid line by
//                        the sixth-order compact (Pade) scheme, det of the
//                        Jacobian, node metrics as cofactors / det.
// cfd_half_point_metrics Main.cpp:2369-2440: face metrics and face dets by
//                        the six-point midpoint rule of node values.
//
// One-off host work (the lines are independent and split across host
// threads); the arithmetic follows the reference's expressions in its
// order, and this file is compiled without FMA contraction of host code, so
// the results equal the reference's bit for bit.
#include <atomic>
#include <cstring>
#include <vector>

#include "internal.h"
#include "lattice_host.h"

namespace {

using cfd::host_parallel_for;
using cfd::nb_of;

// The three line families: the slot of the + neighbour (where a line
// starts: no neighbour there) and of the - neighbour it walks along.
// zeta: N1 / N3, eta: N0 / N2, xi: N4 / N5 (Grid_Transformation.cpp:29-36,
// 213-218, 328-334).
constexpr int kPlus[3] = {1, 0, 4};
constexpr int kMinus[3] = {3, 2, 5};

// The xi family starts only at rows with these loc codes (:329).
inline bool xi_start_loc(int loc) { return loc == 30 || loc == 31 || loc <= 27 || loc == 28; }

struct Line {
    int dir, start;
};

// Coefficients of one row of a line's tridiagonal system: lower a (times the
// + neighbour's derivative), diagonal d, upper b (the - neighbour's), and
// the right-hand sides of x, y, z.
struct Row {
    double a, d, b, c[3];
};

double coord(const cfd_grid_t &g, int k) { return k == 0 ? g.x : (k == 1 ? g.y : g.z); }

// Right-hand side and coefficients at position `step` of a line, the
// reference's cases in its order (later cases override earlier ones).
// p[0..5] are the row and its + neighbours at 1..5 steps, m[0..5] the row and
// its - neighbours; x(r) the coordinate k of row r.
template <class X>
void line_row(int step, const int p[6], const int m[6], double dz, X x, Row &R, int k)
{
    if (step > 1) {   // interior: alpha 1/3, a/2 = 7/9, b/4 = 1/36 (:46-52)
        R.b = 1.0 / 3.0;
        R.d = 1.0;
        R.a = 1.0 / 3.0;
        R.c[k] = (1.0 / dz) * ((-1.0 / 36.0) * x(m[2]) - (7.0 / 9.0) * x(m[1]) + (7.0 / 9.0) * x(p[1])
                               + (1.0 / 36.0) * x(p[2]));
    }
    if (step == 0 && p[1] == 0) {   // the + end, one-sided (:55-62)
        R.b = 5.0;
        R.d = 1.0;
        R.a = 0.0;
        R.c[k] = (1.0 / dz) * ((197.0 / 60.0) * x(m[0]) + (5.0 / 12.0) * x(m[1]) - (5.0) * x(m[2])
                               + (5.0 / 3.0) * x(m[3]) - (5.0 / 12.0) * x(m[4]) + (1.0 / 20.0) * x(m[5]));
    }
    if (step == 1) {   // one row in from the + end (:63-70)
        R.b = 2.0 / 11.0;
        R.d = 1.0;
        R.a = 2.0 / 11.0;
        R.c[k] = (1.0 / dz) * ((20.0 / 33.0) * x(p[1]) + (35.0 / 132.0) * x(m[0]) - (34.0 / 33.0) * x(m[1])
                               + (7.0 / 33.0) * x(m[2]) - (2.0 / 33.0) * x(m[3]) + (1.0 / 132.0) * x(m[4]));
    }
    if (step > 1 && m[2] == 0 && m[1] != 0) {   // one row in from the - end (:72-79)
        R.b = 2.0 / 11.0;
        R.d = 1.0;
        R.a = 2.0 / 11.0;
        R.c[k] = (1.0 / dz) * (-1.0)
                 * ((20.0 / 33.0) * x(m[1]) + (35.0 / 132.0) * x(p[0]) - (34.0 / 33.0) * x(p[1])
                    + (7.0 / 33.0) * x(p[2]) - (2.0 / 33.0) * x(p[3]) + (1.0 / 132.0) * x(p[4]));
    }
    if (step != 0 && m[1] == 0) {   // the - end (:80-87)
        R.b = 0.0;
        R.d = 1.0;
        R.a = 5.0;
        R.c[k] = (1.0 / dz) * (-1.0)
                 * ((197.0 / 60.0) * x(p[0]) + (5.0 / 12.0) * x(p[1]) - (5.0) * x(p[2]) + (5.0 / 3.0) * x(p[3])
                    - (5.0 / 12.0) * x(p[4]) + (1.0 / 20.0) * x(p[5]));
    }
}

// Solves one line into J (d x_k / d dir at [row * 3 + k]); false if the
// line is shorter than three rows or does not end.
bool solve_line(const cfd_grid_t *G, int n_rows, const Line &L, double dz, double *J, std::vector<Row> &rows,
                std::vector<int> &at, std::vector<double> &dp, std::vector<double> &cp)
{
    const int P = kPlus[L.dir], Mn = kMinus[L.dir];
    auto nb = [&](int r, int s) { return (r >= 0 && r < n_rows) ? nb_of(G[r], s) : 0; };
    rows.clear();
    at.clear();
    for (int r = L.start; r != 0; r = nb(r, Mn)) {
        if ((int)at.size() >= n_rows || r < 0 || r >= n_rows) return false;
        int p[6], m[6];
        p[0] = m[0] = r;
        for (int o = 1; o < 6; ++o) {
            p[o] = nb(p[o - 1], P);
            m[o] = nb(m[o - 1], Mn);
        }
        Row R{};
        const int step = (int)at.size();
        for (int k = 0; k < 3; ++k) line_row(step, p, m, dz, [&](int q) { return coord(G[q], k); }, R, k);
        rows.push_back(R);
        at.push_back(r);
    }
    const int M = (int)at.size() - 1;
    if (M < 2) return false;
    // elimination from the - end (:133-152)
    dp.assign(M + 1, 0.0);
    cp.assign(3 * (M + 1), 0.0);
    dp[M - 1] = rows[M - 1].d - ((rows[M - 1].b * rows[M].a) / rows[M].d);
    for (int k = 0; k < 3; ++k) cp[3 * (M - 1) + k] = rows[M - 1].c[k] - ((rows[M].c[k] * rows[M - 1].b) / rows[M].d);
    for (int s = M - 2; s >= 0; --s) {
        dp[s] = rows[s].d - ((rows[s].b * rows[s + 1].a) / dp[s + 1]);
        for (int k = 0; k < 3; ++k) cp[3 * s + k] = rows[s].c[k] - ((cp[3 * (s + 1) + k] * rows[s].b) / dp[s + 1]);
    }
    // substitution from the + end (:154-204); the + neighbour of the row at
    // step s is the row the walk visited at step s - 1
    for (int s = 0; s <= M; ++s) {
        double *Jr = J + 3 * (size_t)at[s];
        const double *Jp = s > 0 ? J + 3 * (size_t)nb(at[s], P) : nullptr;
        for (int k = 0; k < 3; ++k) {
            if (s == 0) Jr[k] = cp[k] / dp[0];
            else if (s < M) Jr[k] = (cp[3 * s + k] - rows[s].a * Jp[k]) / dp[s];
            else Jr[k] = (rows[s].c[k] - rows[M].a * Jp[k]) / rows[M].d;
        }
    }
    return true;
}

}  // namespace

extern "C" {

cfd_status_t cfd_compact_metrics(const cfd_grid_t *grid, int32_t n_rows, double del_zeta, double *det,
                                 cfd_metric_t *metric)
{
    if (!grid || !det || !metric || n_rows < 4 || !(del_zeta > 0.0)) return CFD_EINVAL;
    std::vector<Line> lines;
    for (int r = 1; r < n_rows; ++r) {
        if (grid[r].ID == 10) return CFD_EUNSUPPORTED;   // the reference's wake-cut branches
        for (int d = 0; d < 3; ++d) {
            if (nb_of(grid[r], kPlus[d]) != 0) continue;
            if (d == 2 && !xi_start_loc(grid[r].loc)) continue;
            lines.push_back(Line{d, r});
        }
    }
    // J[d][row][k] = d x_k / d dir_d; zero where no line passes (the
    // reference's zero-initialised Jacobian)
    std::vector<double> J((size_t)9 * n_rows, 0.0);
    std::atomic<bool> bad{false};
    host_parallel_for((long long)lines.size(), [&](long long l0, long long l1) {
        std::vector<Row> rows;
        std::vector<int> at;
        std::vector<double> dp, cp;
        for (long long l = l0; l < l1 && !bad.load(std::memory_order_relaxed); ++l)
            if (!solve_line(grid, n_rows, lines[l], del_zeta, J.data() + (size_t)3 * n_rows * lines[l].dir, rows, at,
                            dp, cp))
                bad = true;
    });
    if (bad) return CFD_EINVAL;   // a line shorter than three rows or without an end
    const double *Jz = J.data(), *Je = Jz + 3 * (size_t)n_rows, *Jx = Je + 3 * (size_t)n_rows;
    host_parallel_for(n_rows - 1, [&](long long b0, long long b1) {
        for (long long q = b0; q < b1; ++q) {
            const size_t r = (size_t)q + 1;
            const double x_zeta = Jz[3 * r], y_zeta = Jz[3 * r + 1], z_zeta = Jz[3 * r + 2];
            const double x_eta = Je[3 * r], y_eta = Je[3 * r + 1], z_eta = Je[3 * r + 2];
            const double x_xi = Jx[3 * r], y_xi = Jx[3 * r + 1], z_xi = Jx[3 * r + 2];
            // det (:447) and the cofactor metrics (:1029-1037)
            const double D = (((x_zeta) * ((y_eta * z_xi) - (y_xi * z_eta))) + ((x_eta) * ((y_xi * z_zeta) - (y_zeta * z_xi)))
                              + ((x_xi) * ((y_zeta * z_eta) - (y_eta * z_zeta))));
            det[r] = D;
            cfd_metric_t &m = metric[r];
            m.zeta_x = (1.0 / D) * (y_eta * z_xi - y_xi * z_eta);
            m.zeta_y = (1.0 / D) * (z_eta * x_xi - z_xi * x_eta);
            m.zeta_z = (1.0 / D) * (x_eta * y_xi - x_xi * y_eta);
            m.eta_x = (1.0 / D) * (y_xi * z_zeta - y_zeta * z_xi);
            m.eta_y = (1.0 / D) * (z_xi * x_zeta - z_zeta * x_xi);
            m.eta_z = (1.0 / D) * (x_xi * y_zeta - x_zeta * y_xi);
            m.xi_x = (1.0 / D) * (y_zeta * z_eta - y_eta * z_zeta);
            m.xi_y = (1.0 / D) * (z_zeta * x_eta - z_eta * x_zeta);
            m.xi_z = (1.0 / D) * (x_zeta * y_eta - x_eta * y_zeta);
        }
    });
    return CFD_OK;
}

cfd_status_t cfd_half_point_metrics(const cfd_grid_t *grid, int32_t n_rows, int32_t n_owned, const double *det,
                                    cfd_metric_t *metric, cfd_determ_t *deter)
{
    if (!grid || !det || !metric || !deter || n_owned < 1 || n_owned >= n_rows) return CFD_EINVAL;
    std::atomic<bool> bad{false};
    auto rule = [](double f0, double f1, double f2, double f3, double f4, double f5) {
        return (1.0 / 256.0) * (3.0 * (f0) - 25.0 * (f1) + 150.0 * (f2) + 150.0 * (f3) - 25.0 * (f4) + 3.0 * (f5));
    };
    // the face blocks are written and the node blocks read: node values into
    // a copy first, so that rows can be processed in any order
    std::vector<double> node9((size_t)9 * n_rows);
    for (int r = 0; r < n_rows; ++r) std::memcpy(&node9[(size_t)9 * r], &metric[r].zeta_x, 9 * sizeof(double));
    host_parallel_for(n_owned, [&](long long b0, long long b1) {
        for (long long q = b0; q < b1; ++q) {
            const int r = (int)q + 1;
            double *rowm = &metric[r].zeta_x, *rowd = &deter[r].ip;
            for (int d = 0; d < 3; ++d) {
                int s[7];   // rows at offsets -3..3 along d
                s[3] = r;
                for (int o = 1; o <= 3; ++o) {
                    const int up = s[3 + o - 1], dn = s[3 - o + 1];
                    s[3 + o] = (up >= 0 && up < n_rows) ? nb_of(grid[up], kPlus[d]) : -1;
                    s[3 - o] = (dn >= 0 && dn < n_rows) ? nb_of(grid[dn], kMinus[d]) : -1;
                }
                for (int o = 0; o < 7; ++o)
                    if (s[o] < 0 || s[o] >= n_rows) bad = true;
                if (bad) return;
                auto M = [&](int o, int c) { return node9[(size_t)9 * s[o] + c]; };
                double *plus = rowm + 9 * (1 + 2 * d), *minus = rowm + 9 * (2 + 2 * d);
                for (int c = 0; c < 9; ++c) {
                    plus[c] = rule(M(1, c), M(2, c), M(3, c), M(4, c), M(5, c), M(6, c));
                    minus[c] = rule(M(0, c), M(1, c), M(2, c), M(3, c), M(4, c), M(5, c));
                }
                rowd[2 * d] = rule(det[s[1]], det[s[2]], det[s[3]], det[s[4]], det[s[5]], det[s[6]]);
                rowd[2 * d + 1] = rule(det[s[0]], det[s[1]], det[s[2]], det[s[3]], det[s[4]], det[s[5]]);
            }
        }
    });
    return bad ? CFD_EINVAL : CFD_OK;
}

}  // extern "C"

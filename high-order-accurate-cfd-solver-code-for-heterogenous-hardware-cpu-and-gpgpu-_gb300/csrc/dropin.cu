// dropin.cu -- the three reference kernels on the reference's own layout.
//
// One thread per row (work-item), exactly the NDRange of the reference
// (Solver.cpp:31-38, local size 1 there).  Buffers are the packed AoS structs
// of include/cfd_rhs.h; device code reads them through aligned double/int
// views (every struct size is a multiple of 8 bytes) rather than through the
// packed types, which would force byte-wise loads.  Neighbour chains are
// bounds-checked: a row whose stencil leaves [0, n_rows) is skipped and the
// context's error word gets CFD_FLAG_BAD_INDEX.
//
// Arithmetic: the exact FP64 layer (physics_exact.cuh); this file is
// compiled with --fmad=false so that results follow the reference's
// evaluation order.
//
// Weno evaluates both faces of each direction at every row, so every
// interior face is computed twice from identical inputs (as row n's +1/2
// face and as row n+1's -1/2 face).  With a scratch buffer the launch is
// split: k_weno_plus computes each row's +1/2 face once and, where its plus
// neighbour p has this row as its minus neighbour and every input of p's
// -1/2 face is bit-identical (then so are the stencil rows; face metric,
// face det and Roe state are compared), also stores it as p's -1/2 face,
// stamped with the call's generation; k_weno_minus computes the -1/2 faces
// left unstamped (box edges, loc codes, inconsistent tables), and
// k_weno<true> reads both faces from the scratch, which keeps the FP64 face
// code and its registers out of it.  The results are the same bits either
// way.
// The drop-in's face kernel runs at 2 blocks of 128 per SM: too few warps
// to hide the integer product's latency, so the divisions' first quotient
// comes from the FP64 multiply (exact_div.cuh, CFD_XDIV_QPROD; the same bits
// either way).
#define CFD_XDIV_QPROD 0
#include <algorithm>

#include "internal.h"
#include "physics_exact.cuh"

namespace cfd {

// ---- aligned views of the packed reference structs ----
// GRID: 56 B = 7 doubles = 14 ints; x,y,z at doubles 0..2, N0..N5 at ints
// 6..11, ID at 12, loc at 13.
__device__ __forceinline__ int grid_nb(const int *g, int row, int which) { return g[14 * row + 6 + which]; }
__device__ __forceinline__ int grid_loc(const int *g, int row) { return g[14 * row + 13]; }
// neighbour slot of (+d) and (-d): d=0 -> N1/N3, d=1 -> N0/N2, d=2 -> N4/N5
__device__ __forceinline__ int plus_slot(int d) { return d == 0 ? 1 : (d == 1 ? 0 : 4); }
__device__ __forceinline__ int minus_slot(int d) { return d == 0 ? 3 : (d == 1 ? 2 : 5); }

// Chained neighbour gather (Weno.cl:159-226): idx[d][o+3], o = -3..3.
// Returns false if any index leaves [0, n_rows).
__device__ __forceinline__ bool gather_star(const int *grid, int gid, int n_rows, int idx[3][7])
{
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        idx[d][3] = gid;
        int p = gid, m = gid;
#pragma unroll
        for (int o = 1; o <= 3; ++o) {
            p = grid_nb(grid, p, plus_slot(d));
            m = grid_nb(grid, m, minus_slot(d));
            if ((unsigned)p >= (unsigned)n_rows || (unsigned)m >= (unsigned)n_rows) return false;
            idx[d][3 + o] = p;
            idx[d][3 - o] = m;
        }
    }
    return true;
}

// FLOW field offsets inside the 9-double row
enum { FU = 0, FV = 1, FW = 2, FP = 3, FT = 4, FRHO = 5, FMU = 6, FA = 7, FE = 8 };

// ------------------------------------------------------------------ U_Q --
// sqrt(rho) and total enthalpy of every row (U_Q.cl:60-65), once per row:
// sh[2*row], sh[2*row + 1].  k_uq<true> reads them for the row and its six
// neighbours instead of evaluating them seven times.
__global__ void __launch_bounds__(128) k_uq_node(const double *__restrict__ flow, int n_rows, double *__restrict__ sh)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    const double *f = flow + 9 * (size_t)row;
    const double rho = f[FRHO];
    sh[2 * (size_t)row] = sqrt(rho);
    sh[2 * (size_t)row + 1] = ex::enthalpy(rho, f[FU], f[FV], f[FW], f[FP]);
}

// U_Q.cl:36-125.
template <bool SH>
__global__ void __launch_bounds__(128) k_uq(double *__restrict__ U, double *__restrict__ Q,
                                            const int *__restrict__ grid, const double *__restrict__ det,
                                            const double *__restrict__ flow, double *__restrict__ roe, int n_items,
                                            int n_rows, unsigned *flags, const double *__restrict__ sh)
{
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= n_items) return;
    int nb[6];
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        nb[s] = grid_nb(grid, gid, s);
        if ((unsigned)nb[s] >= (unsigned)n_rows) {
            atomicOr(flags, CFD_FLAG_BAD_INDEX);
            return;
        }
    }
    const double *fi = flow + 9 * (size_t)gid;
    const double rho = fi[FRHO], u = fi[FU], v = fi[FV], w = fi[FW], p = fi[FP];
    const double si = SH ? sh[2 * (size_t)gid] : sqrt(rho);
    const double hi = SH ? sh[2 * (size_t)gid + 1] : ex::enthalpy(rho, u, v, w, p);
    // ROE block order ip, jp, kp, im, jm, km: block d is the +d face
    // (neighbour slot plus_slot(d)), block d + 3 the -d face (minus_slot(d)).
    //
    // With SH the Roe state of a face is evaluated once.  roe() is symmetric
    // in its two rows bit for bit (one product, and a sum of two products
    // over a sum: IEEE addition and multiplication commute), so the +d
    // block of row m equals the -d block of row q = plus(m) whenever
    // minus(q) == m.  Row m then also stores it as q's -d block, provided q
    // is a row of this launch, and row q skips that block: both rows test
    // the same predicate (m, q < n_items, plus(m) == q, minus(q) == m), so
    // every block has exactly one writer.
    double *r = roe + 36 * (size_t)gid;
#pragma unroll
    for (int b = 0; b < 6; ++b) {
        const int d = b % 3;
        const bool plus = b < 3;
        const int nr = nb[plus ? plus_slot(d) : minus_slot(d)];
        if (SH && !plus && nr < n_items && grid_nb(grid, nr, plus_slot(d)) == gid) continue;
        const double *fn = flow + 9 * (size_t)nr;
        const double rb = fn[FRHO], ub = fn[FU], vb = fn[FV], wb = fn[FW], pb = fn[FP];
        const double sb = SH ? sh[2 * (size_t)nr] : sqrt(rb);
        const double hb = SH ? sh[2 * (size_t)nr + 1] : ex::enthalpy(rb, ub, vb, wb, pb);
        double ra[5];
        ex::roe(sb, ub, vb, wb, hb, si, u, v, w, hi, ra);
        r[6 * b + 0] = ra[0];
        r[6 * b + 1] = ra[1];
        r[6 * b + 2] = ra[2];
        r[6 * b + 4] = ra[3];
        r[6 * b + 5] = ra[4];
        if (SH && plus && nr < n_items && grid_nb(grid, nr, minus_slot(d)) == gid) {
            double *rq = roe + 36 * (size_t)nr + 6 * (d + 3);
            rq[0] = ra[0];
            rq[1] = ra[1];
            rq[2] = ra[2];
            rq[4] = ra[3];
            rq[5] = ra[4];
        }
    }
    const double D = det[gid];
    const double ke = xdiv::scale2<-1>(rho) * (u * u + v * v + w * w);   // 0.5 rho, same bits
    double *Ur = U + 5 * (size_t)gid, *Qr = Q + 5 * (size_t)gid;
    Ur[0] = D * rho;
    Ur[1] = D * rho * u;
    Ur[2] = D * rho * v;
    Ur[3] = D * rho * w;
    const double E = ex::dv(p, 0.4) + ke;
    Ur[4] = D * E;
    Qr[0] = rho;
    Qr[1] = rho * u;
    Qr[2] = rho * v;
    Qr[3] = rho * w;
    Qr[4] = E;
}

// -------------------------------------------------------------- Viscous --
// Viscous.cl:23-643.
__global__ void __launch_bounds__(128) k_viscous(Phys P, const double *__restrict__ U, double *__restrict__ F,
                                                 double *__restrict__ E, double *__restrict__ G,
                                                 double *__restrict__ Fv, double *__restrict__ Ev,
                                                 double *__restrict__ Gv, const int *__restrict__ grid,
                                                 const double *__restrict__ metric, const double *__restrict__ det,
                                                 double *__restrict__ flow, int n_items, int n_rows, unsigned *flags)
{
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= n_items) return;
    int idx[3][7];
    if (!gather_star(grid, gid, n_rows, idx)) {
        atomicOr(flags, CFD_FLAG_BAD_INDEX);
        return;
    }
    double m[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) m[k] = metric[63 * (size_t)gid + k];
    const double D = det[gid];
    const double *fr = flow + 9 * (size_t)gid;
    const double prim[5] = {fr[FRHO], fr[FU], fr[FV], fr[FW], fr[FP]};
    double Fn[5], En[5], Gn[5];
    ex::node_flux(prim, m, D, Fn, En, Gn);
    double Fvn[5], Evn[5], Gvn[5];
    double mu;
    {
        double dU[3][5];
#pragma unroll 1
        for (int d = 0; d < 3; ++d) {
            int L[7];
#pragma unroll
            for (int o = 0; o < 7; ++o) L[o] = grid_loc(grid, idx[d][o]);
#pragma unroll
            for (int c = 0; c < 5; ++c) {
                double f[7];
#pragma unroll
                for (int o = 0; o < 7; ++o) f[o] = U[5 * (size_t)idx[d][o] + c];
                dU[d][c] = visc_deriv_ref(f, L);
            }
        }
        double Ui[5];
#pragma unroll
        for (int c = 0; c < 5; ++c) Ui[c] = U[5 * (size_t)gid + c];
        double KS[3];   // MTS test filter (Viscous.cl:493-495)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int c = d + 1;
            const double *um = U + 5 * (size_t)idx[d][2], *up = U + 5 * (size_t)idx[d][4];
            KS[d] = ex::ks(Ui[c], Ui[0], um[c], um[0], up[c], up[0]);
        }
        const ex::Visc V{P.mach, P.reynolds, P.prandtl, P.t_inf, P.les, P.cs};
        ex::viscous_node(dU, Ui, m, D, prim, KS, V, Fvn, Evn, Gvn, mu);
    }
    double *o;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        o = F + 5 * (size_t)gid; o[c] = Fn[c];
        o = E + 5 * (size_t)gid; o[c] = En[c];
        o = G + 5 * (size_t)gid; o[c] = Gn[c];
        o = Fv + 5 * (size_t)gid; o[c] = P.viscous ? Fvn[c] : 0.0;
        o = Ev + 5 * (size_t)gid; o[c] = P.viscous ? Evn[c] : 0.0;
        o = Gv + 5 * (size_t)gid; o[c] = P.viscous ? Gvn[c] : 0.0;
    }
    flow[9 * (size_t)gid + FMU] = mu;
}

// ----------------------------------------------------------------- Weno --
// Corrected face flux of row gid, direction d, side s (0: +1/2, 1: -1/2)
// from the row's own face data (metric block 1+2d+s, DETERM 2d+s, ROE
// block d+3s) over the stencil rows st[0..5] (offsets -2..3 for s = 0,
// -3..2 for s = 1), Weno.cl:336-3058.
__device__ __forceinline__ void face_side(const Phys &P, int gid, int d, int s, const int st[6],
                                          const double *__restrict__ deter, const double *__restrict__ Q,
                                          const double *__restrict__ metric, const double *__restrict__ roe,
                                          const double *__restrict__ NF, double Fh[5])
{
    const double *fm = metric + 63 * (size_t)gid + 9 * (1 + 2 * d + s) + 3 * d;
    const double det_f = deter[6 * (size_t)gid + 2 * d + s];
    const double *ra = roe + 36 * (size_t)gid + 6 * (d + 3 * s);
    const double rstate[5] = {ra[0], ra[1], ra[2], ra[4], ra[5]};
    double pts[6][5], nfv[6];
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int c = 0; c < 5; ++c) pts[k][c] = Q[5 * (size_t)st[k] + c];
    double Fhat[5];
    ex::face_flux(pts, fm[0], fm[1], fm[2], det_f, rstate, P.eps, Fhat);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
#pragma unroll
        for (int k = 0; k < 6; ++k) nfv[k] = NF[5 * (size_t)st[k] + c];
        Fh[c] = ex::corrected(Fhat[c], nfv);
    }
}

// Rows of offsets -2..3 of row n along d (chained neighbours); false if the
// chain leaves [0, n_rows).
__device__ __forceinline__ bool plus_line(const int *grid, int n, int n_rows, int d, int st[6])
{
    st[2] = n;
    int m = n, p = n;
#pragma unroll
    for (int o = 1; o <= 3; ++o) {
        p = grid_nb(grid, p, plus_slot(d));
        if ((unsigned)p >= (unsigned)n_rows) return false;
        st[2 + o] = p;
        if (o <= 2) {
            m = grid_nb(grid, m, minus_slot(d));
            if ((unsigned)m >= (unsigned)n_rows) return false;
            st[2 - o] = m;
        }
    }
    return true;
}

__device__ __forceinline__ bool same_bits(double a, double b) { return __double_as_longlong(a) == __double_as_longlong(b); }

// +1/2 face of every row gid < n_items along d = blockIdx.y whose stencil
// stays in the table: Fp[(d*5 + c)*ld + gid]; also p's -1/2 face
// Fm[(d*5 + c)*ld + p] with stamp[d*ld + p] = gen for the plus neighbour p
// whose minus neighbour is gid, when p's face data are gid's bit for bit.
// blocks per SM the +1/2-face kernel's register budget allows: 2 (GB300,
// TGV 128^3: drop-in 2.89e7 cell-updates/s against 2.85e7 at 3)
#ifndef CFD_WENO_PLUS_MIN_BLOCKS
#define CFD_WENO_PLUS_MIN_BLOCKS 2
#endif
__global__ void __launch_bounds__(128, CFD_WENO_PLUS_MIN_BLOCKS) k_weno_plus(Phys P, const double *__restrict__ deter,
                                                       const int *__restrict__ grid, const double *__restrict__ Q,
                                                       const double *__restrict__ metric,
                                                       const double *__restrict__ roe, const double *__restrict__ F,
                                                       const double *__restrict__ E, const double *__restrict__ G,
                                                       int n_items, int n_rows, double *__restrict__ Fp,
                                                       double *__restrict__ Fm, unsigned *__restrict__ stamp,
                                                       unsigned gen, long long ld)
{
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (gid >= n_items) return;
    int st[6];
    if (!plus_line(grid, gid, n_rows, d, st)) return;
    double Fh[5];
    face_side(P, gid, d, 0, st, deter, Q, metric, roe, d == 0 ? F : (d == 1 ? E : G), Fh);
#pragma unroll
    for (int c = 0; c < 5; ++c) Fp[(d * 5 + c) * ld + gid] = Fh[c];
    const int p = st[3];
    if ((unsigned)p >= (unsigned)n_items || grid_nb(grid, p, minus_slot(d)) != gid) return;
    // p's -1/2 face reads metric block 2+2d, DETERM 2d+1 and ROE block d+3 of p
    const double *fg = metric + 63 * (size_t)gid + 9 * (1 + 2 * d) + 3 * d;
    const double *fp = metric + 63 * (size_t)p + 9 * (2 + 2 * d) + 3 * d;
    const double *rg = roe + 36 * (size_t)gid + 6 * d, *rp = roe + 36 * (size_t)p + 6 * (d + 3);
    if (same_bits(fg[0], fp[0]) && same_bits(fg[1], fp[1]) && same_bits(fg[2], fp[2])
        && same_bits(deter[6 * (size_t)gid + 2 * d], deter[6 * (size_t)p + 2 * d + 1]) && same_bits(rg[0], rp[0])
        && same_bits(rg[1], rp[1]) && same_bits(rg[2], rp[2]) && same_bits(rg[4], rp[4]) && same_bits(rg[5], rp[5])) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Fm[(d * 5 + c) * ld + p] = Fh[c];
        stamp[d * ld + p] = gen;
    }
}

// Rows of offsets -3..2 of row n along d; false if the chain leaves
// [0, n_rows).
__device__ __forceinline__ bool minus_line(const int *grid, int n, int n_rows, int d, int st[6])
{
    st[3] = n;
    int m = n, p = n;
#pragma unroll
    for (int o = 1; o <= 3; ++o) {
        m = grid_nb(grid, m, minus_slot(d));
        if ((unsigned)m >= (unsigned)n_rows) return false;
        st[3 - o] = m;
        if (o <= 2) {
            p = grid_nb(grid, p, plus_slot(d));
            if ((unsigned)p >= (unsigned)n_rows) return false;
            st[3 + o] = p;
        }
    }
    return true;
}

// The -1/2 face of every row gid < n_items along each d that k_weno_plus
// did not stamp, from the row's own face data (metric block 2+2d, DETERM
// 2d+1, ROE block d+3): Fm and stamp = gen.  A grid-stride scan of the
// rows, direction by direction, with a resident-sized grid: on a periodic
// lattice every face is stamped and the pass only reads the stamps.
__global__ void __launch_bounds__(128, 2) k_weno_minus(Phys P, const double *__restrict__ deter,
                                                        const int *__restrict__ grid, const double *__restrict__ Q,
                                                        const double *__restrict__ metric,
                                                        const double *__restrict__ roe, const double *__restrict__ F,
                                                        const double *__restrict__ E, const double *__restrict__ G,
                                                        int n_items, int n_rows, double *__restrict__ Fm,
                                                        unsigned *__restrict__ stamp, unsigned gen, long long ld)
{
    const int stride = gridDim.x * blockDim.x;
    for (int d = 0; d < 3; ++d) {
        for (int gid = blockIdx.x * blockDim.x + threadIdx.x; gid < n_items; gid += stride) {
            if (stamp[d * ld + gid] == gen) continue;
            int st[6];
            if (!minus_line(grid, gid, n_rows, d, st)) continue;   // k_weno reports the row
            double Fh[5];
            face_side(P, gid, d, 1, st, deter, Q, metric, roe, d == 0 ? F : (d == 1 ? E : G), Fh);
#pragma unroll
            for (int c = 0; c < 5; ++c) Fm[(d * 5 + c) * ld + gid] = Fh[c];
            stamp[d * ld + gid] = gen;
        }
    }
}

// Weno.cl:36-3137: per row, both faces of each direction from the row's own
// face data (metric blocks, DETERM, ROE_AVERAGING), as the reference does.
// REUSE: the +1/2 faces come from k_weno_plus (Fp), the -1/2 faces from Fm
// (k_weno_plus or k_weno_minus; every row whose stencil stays in the table
// is stamped with this call's generation).
template <bool REUSE>
__global__ void __launch_bounds__(128) k_weno(Phys P, int j, double mach, double dt, const double *__restrict__ deter,
                                              const double *__restrict__ det, double *__restrict__ U0,
                                              double *__restrict__ U1, double *__restrict__ U2,
                                              const int *__restrict__ grid, const double *__restrict__ Q,
                                              const double *__restrict__ metric, const double *__restrict__ roe,
                                              const double *__restrict__ Fv, const double *__restrict__ Ev,
                                              const double *__restrict__ Gv, const double *__restrict__ F,
                                              const double *__restrict__ E, const double *__restrict__ G,
                                              double *__restrict__ flow, int n_items, int n_rows, unsigned *flags,
                                              double *__restrict__ L_out, const double *__restrict__ Fp,
                                              const double *__restrict__ Fm, const unsigned *__restrict__ stamp,
                                              unsigned gen, long long ld)
{
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= n_items) return;
    int idx[3][7];
    if (!gather_star(grid, gid, n_rows, idx)) {
        atomicOr(flags, CFD_FLAG_BAD_INDEX);
        return;
    }
    double dflux[3][5], dvis[3][5];
    bool bad = false;
    // direction d's flux and viscous differences (unrolled over d with the
    // faces from the scratch, a loop when the faces are evaluated here)
    auto direction = [&](const int d) {
        const double *NF = d == 0 ? F : (d == 1 ? E : G);
        const double *VF = d == 0 ? Fv : (d == 1 ? Ev : Gv);
        double Fh[2][5];
        if (REUSE) {
            if (stamp[d * ld + gid] != gen) {   // cannot happen when the star is in the table
                bad = true;
                return;
            }
#pragma unroll
            for (int c = 0; c < 5; ++c) {
                Fh[0][c] = Fp[(d * 5 + c) * ld + gid];
                Fh[1][c] = Fm[(d * 5 + c) * ld + gid];
            }
        } else {
#pragma unroll 1
            for (int s = 0; s < 2; ++s)   // stencil rows: offsets -2..3 (plus) or -3..2 (minus)
                face_side(P, gid, d, s, idx[d] + (s == 0 ? 1 : 0), deter, Q, metric, roe, NF, Fh[s]);
        }
        int Lc[7];
#pragma unroll
        for (int o = 0; o < 7; ++o) Lc[o] = grid_loc(grid, idx[d][o]);
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            dflux[d][c] = Fh[0][c] - Fh[1][c];
            double f[7];
#pragma unroll
            for (int o = 0; o < 7; ++o) f[o] = VF[5 * (size_t)idx[d][o] + c];
            dvis[d][c] = weno_visc_deriv_ref(f, Lc);
        }
    };
    if (REUSE) {
        direction(0);
        direction(1);
        direction(2);
    } else {
#pragma unroll 1
        for (int d = 0; d < 3; ++d) direction(d);
    }
    if (bad) {
        atomicOr(flags, CFD_FLAG_BAD_INDEX);
        return;
    }
    double L[5];
#pragma unroll
    for (int c = 0; c < 5; ++c)
        L[c] = (-1.0) * (dflux[0][c] + dflux[1][c] + dflux[2][c] + dvis[0][c] + dvis[1][c] + dvis[2][c]);
    if (L_out) {
#pragma unroll
        for (int c = 0; c < 5; ++c) L_out[5 * (size_t)gid + c] = L[c];
    }
    // SSP-RK3 stage and primitive recovery (Weno.cl:3084-3135)
    const size_t r5 = 5 * (size_t)gid;
    double u0[5], u1[5], u2[5], Un[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) { u0[c] = U0[r5 + c]; u1[c] = U1[r5 + c]; u2[c] = U2[r5 + c]; }
    double rho, u, v, w, e, p, t, a;
    ex::rk_and_primitives(j, dt, mach, det[gid], u0, u1, u2, L, Un, rho, u, v, w, e, p, t, a);
    double *Uo = j == 0 ? U1 : (j == 1 ? U2 : U0);
#pragma unroll
    for (int c = 0; c < 5; ++c) Uo[r5 + c] = Un[c];
    double *fo = flow + 9 * (size_t)gid;
    fo[FRHO] = rho;
    fo[FU] = u;
    fo[FV] = v;
    fo[FW] = w;
    fo[FE] = e;
    fo[FP] = p;
    fo[FT] = t;
    fo[FA] = a;
    if (gid > 0 && !(isfinite(rho) && isfinite(u) && isfinite(v) && isfinite(w) && isfinite(p)))
        atomicOr(flags, CFD_FLAG_NONFINITE);
}

int launch_uq(cudaStream_t st, double *U, double *Q, const int *grid, const double *det, const double *flow,
              double *roe, int n_items, int n_rows, unsigned *flags, double *node_scratch, long long scratch_rows)
{
    if (node_scratch && scratch_rows >= n_rows) {   // 2 of the 15 doubles per row
        k_uq_node<<<blocks_for(n_rows, 128), 128, 0, st>>>(flow, n_rows, node_scratch);
        k_uq<true><<<blocks_for(n_items, 128), 128, 0, st>>>(U, Q, grid, det, flow, roe, n_items, n_rows, flags,
                                                             node_scratch);
        return 2;
    }
    k_uq<false><<<blocks_for(n_items, 128), 128, 0, st>>>(U, Q, grid, det, flow, roe, n_items, n_rows, flags, nullptr);
    return 1;
}

void launch_viscous(cudaStream_t st, const Phys &P, const double *U, double *F, double *E, double *G, double *Fv,
                    double *Ev, double *Gv, const int *grid, const double *metric, const double *det, double *flow,
                    int n_items, int n_rows, unsigned *flags)
{
    k_viscous<<<blocks_for(n_items, 128), 128, 0, st>>>(P, U, F, E, G, Fv, Ev, Gv, grid, metric, det, flow, n_items,
                                                        n_rows, flags);
}

// Grid of k_weno_minus: two resident blocks of 128 per SM, at most one
// thread per row.
static unsigned minus_blocks(int n_items)
{
    const long long want = ((long long)n_items + 127) / 128;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess
        || sms <= 0) {
        cudaGetLastError();
        return (unsigned)std::max(1LL, want);
    }
    return (unsigned)std::max(1LL, std::min<long long>(want, 2LL * sms));
}

void launch_weno(cudaStream_t st, const Phys &P, int j, double mach, double dt, const double *deter,
                 const double *det, double *U0, double *U1, double *U2, const int *grid, const double *Q,
                 const double *metric, const double *roe, const double *Fv, const double *Ev, const double *Gv,
                 const double *F, const double *E, const double *G, double *flow, int n_items, int n_rows,
                 unsigned *flags, double *L_out, double *face_scratch, long long scratch_rows, unsigned gen)
{
    const unsigned nb = blocks_for(n_items, 128);
    if (face_scratch && scratch_rows >= n_items) {
        const long long ld = scratch_rows;
        double *Fp = face_scratch, *Fm = face_scratch + 15 * ld;
        unsigned *stamp = face_stamps(face_scratch, ld);
        k_weno_plus<<<dim3(nb, 3), 128, 0, st>>>(P, deter, grid, Q, metric, roe, F, E, G, n_items, n_rows, Fp, Fm,
                                                 stamp, gen, ld);
        k_weno_minus<<<minus_blocks(n_items), 128, 0, st>>>(P, deter, grid, Q, metric, roe, F, E, G, n_items, n_rows,
                                                             Fm, stamp, gen, ld);
        k_weno<true><<<nb, 128, 0, st>>>(P, j, mach, dt, deter, det, U0, U1, U2, grid, Q, metric, roe, Fv, Ev, Gv, F, E,
                                         G, flow, n_items, n_rows, flags, L_out, Fp, Fm, stamp, gen, ld);
    } else {
        k_weno<false><<<nb, 128, 0, st>>>(P, j, mach, dt, deter, det, U0, U1, U2, grid, Q, metric, roe, Fv, Ev, Gv, F,
                                          E, G, flow, n_items, n_rows, flags, L_out, nullptr, nullptr, nullptr, 0u, 0);
    }
}

}  // namespace cfd

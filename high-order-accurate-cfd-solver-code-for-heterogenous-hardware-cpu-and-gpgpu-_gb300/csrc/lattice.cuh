// lattice.cuh -- one periodic lattice as the device kernels see it: shape,
// constants, and pointers to its structure-of-arrays fields.  Shared by the
// single-lattice kernels (structured.cu, mixed.cu) and the batched
// persistent kernel (batch_*.cu), which holds one LatView per instance.
#pragma once

#include <cuda_runtime.h>

#include "physics.cuh"

namespace cfd {

// Field layout: every array is [component][N], n = i + ni*(j + nj*k).
//
// Mixed form: U0/U1/U2 hold each conserved value as an unevaluated sum of
// two FP32 numbers (hi + lo, about 48 significant bits) in the same bytes as
// the FP64 form's [5][N] doubles: hi at [c][N], lo at [5 + c][N].  Split
// form: U0/U1/U2 are the FP64 form's doubles, the stage intermediates FP32
// (Q32, R32, FEG32, V32) except the face fluxes Fh (FP64).
struct LatView {
    int ni, nj, nk, N;
    Phys P;
    double dt;
    float dt_hi, dt_lo;        // dt as hi + lo (mixed form)
    // geometry (FP64), and FP32 copies for the mixed form
    const double *m9, *det, *fm, *fdet;
    const float *fm32, *fdet32;
    const float *node32;       // [11][N] 9 node metrics, det, det^(-1/3) (mixed form)
    const float *idet32;       // [2][N] 1/det as hi, lo (mixed form)
    const double *idet64;      // [N] 1/det (split form)
    float *Whl;                // [10][N] hi/lo copy of the current stage's state (split form)
    // state
    double *prim9;             // FLOW fields u,v,w,p,t,rho,mu,a,e
    float *prim32;             // the same fields in FP32 (mixed form)
    double *U0, *U1, *U2;
    // FP64 stage intermediates
    double *Q, *FEG, *V, *sh, *Fh;
    // FP32 stage intermediates (mixed form)
    float *Q32, *R32, *FEG32, *V32, *Fh32;
    unsigned *flags;           // error word of this lattice
    double *Lout;              // optional [5][N] right-hand side output
    // Non-periodic directions: bit d of `per` set = direction d periodic.
    // A non-periodic direction carries at least three ghost layers on each
    // side; its stencils clamp at the box edge (the outermost ghosts'
    // outward neighbour is the node itself) and loc8 holds the reference's
    // loc codes (0 interior, 1..52 boundary, 100 ghost).  loc8 is null on a
    // fully periodic lattice.
    int per;
    const unsigned char *loc8;
    // bit d: some owned node has a ghost within two nodes along d, so the
    // loc-code branches matter there; along the other directions every
    // branch of the reference is the central one
    int locdirs;
    // bit d of locflag[n]: node n takes a non-central loc-code branch along d
    // (a node in the band next to the ghost layers); null: every node of a
    // locdir direction evaluates its branches
    const unsigned char *locflag;
    const int *row_of;         // node n -> reference row (null: row n + 1)
};

__device__ __forceinline__ bool lat_locdir(const LatView &g, int d) { return g.loc8 && ((g.locdirs >> d) & 1); }

constexpr unsigned char kLocGhost = 100;

enum { LF_U = 0, LF_V = 1, LF_W = 2, LF_P = 3, LF_T = 4, LF_RHO = 5, LF_MU = 6, LF_A = 7, LF_E = 8 };

// periodic wrap of x = i + o, 0 <= i < n; one correction when |o| <= 3 <= n
// (every stencil here), repeated for shorter extents
__device__ __forceinline__ int lwrap(int x, int n)
{
    if (n >= 3) {
        x += x < 0 ? n : 0;
        return x >= n ? x - n : x;
    }
    while (x < 0) x += n;
    while (x >= n) x -= n;
    return x;
}

__device__ __forceinline__ void lat_ijk(const LatView &g, int n, int &i, int &j, int &k)
{
    const unsigned un = (unsigned)n, uni = (unsigned)g.ni, unj = (unsigned)g.nj;
    const unsigned r = un / uni;
    i = (int)(un - r * uni);
    k = (int)(r / unj);
    j = (int)(r - (unsigned)k * unj);
}

// clamp of x = i + o into [0, n) (non-periodic directions)
__device__ __forceinline__ int lclamp(int x, int n) { return x < 0 ? 0 : (x >= n ? n - 1 : x); }

__device__ __forceinline__ bool lat_periodic(const LatView &g, int d) { return (g.per >> d) & 1; }

// node at offset o along direction d from (i,j,k)
__device__ __forceinline__ int lat_step(const LatView &g, int i, int j, int k, int d, int o)
{
    const bool p = lat_periodic(g, d);
    if (d == 0) i = p ? lwrap(i + o, g.ni) : lclamp(i + o, g.ni);
    else if (d == 1) j = p ? lwrap(j + o, g.nj) : lclamp(j + o, g.nj);
    else k = p ? lwrap(k + o, g.nk) : lclamp(k + o, g.nk);
    return i + g.ni * (j + g.nj * k);
}

__device__ __forceinline__ int lat_coord(int i, int j, int k, int d) { return d == 0 ? i : (d == 1 ? j : k); }

__device__ __forceinline__ int lat_extent(const LatView &g, int d) { return d == 0 ? g.ni : (d == 1 ? g.nj : g.nk); }
inline int lat_extent_h(const LatView &g, int d) { return d == 0 ? g.ni : (d == 1 ? g.nj : g.nk); }

// Face n+1/2 along a non-periodic d is needed (and its six-point stencil
// lies in the box) for coordinates 2 .. n_d-4.
__device__ __forceinline__ bool lat_face_needed(const LatView &g, int i, int j, int k, int d)
{
    if (lat_periodic(g, d)) return true;
    const int c = lat_coord(i, j, k, d);
    return c >= 2 && c <= lat_extent(g, d) - 4;
}

__device__ __forceinline__ bool lat_ghost(const LatView &g, int n) { return g.loc8 && g.loc8[n] == kLocGhost; }

__device__ __forceinline__ double *lat_U(const LatView &g, int q) { return q == 0 ? g.U0 : (q == 1 ? g.U1 : g.U2); }

// mixed form: the hi/lo view of U slot q ([10][N] floats)
__device__ __forceinline__ float *lat_W(const LatView &g, int q) { return reinterpret_cast<float *>(lat_U(g, q)); }

}  // namespace cfd

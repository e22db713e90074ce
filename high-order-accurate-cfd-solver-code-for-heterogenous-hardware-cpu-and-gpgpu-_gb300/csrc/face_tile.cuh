// face_tile.cuh -- shared-memory tiles of the FP32 face passes (mixed and
// split forms): a block of 128 threads covers TILE faces along the face
// direction D times 128 / TILE nodes across it (axis A), on one line of the
// third axis (B).  The block loads the stencil lines (TILE + 5 nodes along
// D) of Q, the Roe inputs (u, v, w, sqrt(rho), H) and the node fluxes along
// D once, coalesced along i, and every face reads its six points from there
// (the reference gathers each point per face, Weno.cl:159-328).
#pragma once

#include "lattice.cuh"
#include "physics.cuh"

namespace cfd {

constexpr int kFaceThreads = 128;

template <int D, int TILE>
struct FaceTile {
    static constexpr int kTile = TILE;                   // faces along D
    static constexpr int kWide = kFaceThreads / TILE;    // nodes across
    static constexpr int A = D == 0 ? 1 : 0;             // axis across
    static constexpr int B = D == 2 ? 1 : 2;             // axis of the block's line
    static constexpr int kLine = kTile + 5;              // staged nodes along D
    static constexpr int kStaged = kLine * kWide;
    // smem index of (position b along D, a across); i is the fast index
    static __device__ __forceinline__ int at(int b, int a) { return D == 0 ? a * kLine + b : b * kWide + a; }
    // thread -> (t along D, a across), consecutive threads consecutive in i
    static __device__ __forceinline__ void split(int x, int &t, int &a)
    {
        if (D == 0) {
            t = x % kTile;
            a = x / kTile;
        } else {
            t = x / kWide;
            a = x % kWide;
        }
    }
    // staged element m -> (b along D, a across)
    static __device__ __forceinline__ void staged(int m, int &b, int &a)
    {
        if (D == 0) {
            b = m % kLine;
            a = m / kLine;
        } else {
            b = m / kWide;
            a = m % kWide;
        }
    }
    static dim3 grid(const LatView &g)
    {
        return dim3((unsigned)((lat_extent_h(g, D) + kTile - 1) / kTile),
                    (unsigned)((lat_extent_h(g, A) + kWide - 1) / kWide), (unsigned)lat_extent_h(g, B));
    }
};

// coordinate c in [-2, n + TILE + 3) of a staged stencil line, wrapped
// (periodic) or clamped; the wrap subtracts instead of dividing (c is at
// most a few extents away from [0, n))
__device__ __forceinline__ int tile_coord(const LatView &g, int d, int c)
{
    const int n = lat_extent(g, d);
    if (lat_periodic(g, d)) {
        while (c < 0) c += n;
        while (c >= n) c -= n;
        return c;
    }
    return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

// The tile at face coordinate tD along D, node tA across (axis A), line cB
// of axis B: the single-lattice passes take it from blockIdx, the batched
// kernel from its item table.
struct TileAt {
    int tD, tA, cB;
};

template <class T>
__device__ __forceinline__ TileAt tile_of_block()
{
    return {(int)blockIdx.x * T::kTile, (int)blockIdx.y * T::kWide, (int)blockIdx.z};
}

// Stages the block's stencil lines of Q, the Roe inputs and the node fluxes
// along D (read-only in the face pass: non-coherent loads, unless RO is
// false because the same launch wrote them) into sQ/sR/sF, each
// [5][T::kStaged]; ends with __syncthreads().
template <class T, int D, bool RO = true>
__device__ __forceinline__ void stage_face_lines(const LatView &g, TileAt at, float *sQ, float *sR, float *sF)
{
    constexpr int S = T::kStaged;
    auto ld = [](const float *p) { return RO ? __ldg(p) : *p; };
    const int N = g.N;
    const int nA = lat_extent(g, T::A);
    const float *NF = g.FEG32 + (size_t)D * 5 * N;
    for (int m = threadIdx.x; m < S; m += blockDim.x) {
        int b, a;
        T::staged(m, b, a);
        int c[3];
        c[D] = tile_coord(g, D, at.tD + b - 2);
        c[T::A] = at.tA + a < nA ? at.tA + a : nA - 1;
        c[T::B] = at.cB;
        const int node = c[0] + g.ni * (c[1] + g.nj * c[2]);
        const int e = T::at(b, a);
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            sQ[q * S + e] = ld(g.Q32 + q * N + node);
            sR[q * S + e] = ld(g.R32 + q * N + node);
            sF[q * S + e] = ld(NF + q * N + node);
        }
    }
    __syncthreads();
}

// The face of this thread: its lattice node and position (t, a) in the
// tile; false if the thread has no face (past the lattice, or a face whose
// stencil leaves a non-periodic box).
template <class T, int D>
__device__ __forceinline__ bool tile_face(const LatView &g, TileAt at, int &n, int &t, int &a)
{
    T::split(threadIdx.x, t, a);
    int c[3];
    c[D] = at.tD + t;
    c[T::A] = at.tA + a;
    c[T::B] = at.cB;
    if (c[D] >= lat_extent(g, D) || c[T::A] >= lat_extent(g, T::A) || !lat_face_needed(g, c[0], c[1], c[2], D))
        return false;
    n = c[0] + g.ni * (c[1] + g.nj * c[2]);
    return true;
}

// The stencil of the face at tile position (t, a) from the staged lines:
// P[k] = (Q of point k, Q of point 5-k) and the Roe state r of the face.
template <class T>
__device__ __forceinline__ void tile_stencil(const float *sQ, const float *sR, int t, int a, float2 P[3][5],
                                             float r[5])
{
    constexpr int S = T::kStaged;
#pragma unroll
    for (int o = 0; o < 3; ++o)
#pragma unroll
        for (int q = 0; q < 5; ++q) P[o][q] = make_float2(sQ[q * S + T::at(t + o, a)], sQ[q * S + T::at(t + 5 - o, a)]);
    const int er = T::at(t + 3, a), el = T::at(t + 2, a);
    roe_average<float>(sR[3 * S + er], sR[er], sR[S + er], sR[2 * S + er], sR[4 * S + er], sR[3 * S + el], sR[el],
                       sR[S + el], sR[2 * S + el], sR[4 * S + el], r);
}

// The node fluxes f[0..5] of component q along D at tile position (t, a).
template <class T>
__device__ __forceinline__ void tile_node_fluxes(const float *sF, int q, int t, int a, float f[6])
{
    constexpr int S = T::kStaged;
#pragma unroll
    for (int o = 0; o < 6; ++o) f[o] = sF[q * S + T::at(t + o, a)];
}

// Shared floats one tile of T stages (Q, Roe inputs, node fluxes).
template <class T>
constexpr int tile_smem_floats()
{
    return 15 * T::kStaged;
}

}  // namespace cfd

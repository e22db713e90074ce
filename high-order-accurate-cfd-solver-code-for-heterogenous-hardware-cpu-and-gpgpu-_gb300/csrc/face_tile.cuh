// face_tile.cuh -- shared-memory tiles of the FP32 face passes (mixed and
// split forms): a block of 128 threads covers TILE faces along the face
// direction D times 128 / TILE nodes across it (axis A), on one line of the
// third axis (B).  The block loads the stencil lines (TILE + 5 nodes along
// D) of Q, the Roe inputs (u, v, w, sqrt(rho), H) and the node fluxes along
// D once, coalesced along i, and every face reads its six points from there
// (the reference gathers each point per face, Weno.cl:159-328).
#pragma once

#include "lattice.cuh"

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

// Stages the block's stencil lines of Q, the Roe inputs and the node fluxes
// along D (read-only in the face pass: non-coherent loads) into sQ/sR/sF,
// each [5][T::kStaged]; ends with __syncthreads().
template <class T, int D>
__device__ __forceinline__ void stage_face_lines(const LatView &g, float *sQ, float *sR, float *sF)
{
    constexpr int S = T::kStaged;
    const int N = g.N;
    const int tD = blockIdx.x * T::kTile, tA = blockIdx.y * T::kWide, cB = blockIdx.z;
    const int nA = lat_extent(g, T::A);
    const float *NF = g.FEG32 + (size_t)D * 5 * N;
    for (int m = threadIdx.x; m < S; m += blockDim.x) {
        int b, a;
        T::staged(m, b, a);
        int c[3];
        c[D] = tile_coord(g, D, tD + b - 2);
        c[T::A] = tA + a < nA ? tA + a : nA - 1;
        c[T::B] = cB;
        const int node = c[0] + g.ni * (c[1] + g.nj * c[2]);
        const int e = T::at(b, a);
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            sQ[q * S + e] = __ldg(g.Q32 + q * N + node);
            sR[q * S + e] = __ldg(g.R32 + q * N + node);
            sF[q * S + e] = __ldg(NF + q * N + node);
        }
    }
    __syncthreads();
}

// The face of this thread: its lattice coordinates, node, and position
// (t, a) in the tile; false if the thread has no face (past the lattice, or
// a face whose stencil leaves a non-periodic box).
template <class T, int D>
__device__ __forceinline__ bool tile_face(const LatView &g, int &n, int &t, int &a)
{
    T::split(threadIdx.x, t, a);
    int c[3];
    c[D] = blockIdx.x * T::kTile + t;
    c[T::A] = blockIdx.y * T::kWide + a;
    c[T::B] = blockIdx.z;
    if (c[D] >= lat_extent(g, D) || c[T::A] >= lat_extent(g, T::A) || !lat_face_needed(g, c[0], c[1], c[2], D))
        return false;
    n = c[0] + g.ni * (c[1] + g.nj * c[2]);
    return true;
}

}  // namespace cfd

// batch_kernel.cuh -- one persistent launch per RK stage over many lattices.
//
// Work is described by a tile table: tile t = (instance, first node, node
// count), tile size = block size, so one thread owns one node of a tile.
// A stage has two phases separated by a grid-wide barrier:
//   A  for every tile: viscous fluxes and the three face fluxes (4 work items
//      per tile, taken in order from a shared counter, so that blocks that
//      run at the same time share a tile's data and none waits long)
//   B  for every tile: RHS, RK stage, primitives, and the next stage's prep
//      (U_Q) on the new primitives
// The kernel is launched cooperatively (all blocks co-resident) with at most
// the occupancy limit of blocks; the barrier's wait is bounded by a
// %globaltimer deadline, after which it sets CFD_FLAG_TIMEOUT and the block
// returns instead of spinning.
//
// Ops supplies the per-node operations of one precision form
// (lattice_fp64.cuh or lattice_mixed.cuh); this header is included by the
// translation unit compiled with that form's flags.
#pragma once

#include "face_tile.cuh"
#include "lattice.cuh"

namespace cfd {

struct BatchTile {
    int inst;   // index into the LatView table
    int n0;     // first node of the tile
    int count;  // nodes in the tile (<= block size)
    int pad;
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Sense-reversing grid barrier over `nblocks` co-resident blocks.
// bar[0] = arrival count, bar[1] = generation.  Returns false (and sets the
// timeout bit) if the generation does not advance before the deadline.
// The last block to arrive also clears bar[3], the phase-A work counter
// (every block has stopped taking phase-A items when it arrives), so the
// next launch starts from item 0.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned nblocks, unsigned long long limit_ns,
                                             unsigned *gflags)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned *vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(bar + 3, 0u);
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (*vgen == gen) {
                if (global_ns() - t0 > limit_ns) {
                    atomicOr(gflags, 4u);   // CFD_FLAG_TIMEOUT
                    ok = 0;
                    break;
                }
                __nanosleep(200);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Next phase-A item of this block: blocks take items in order from a
// shared counter (bar[3]), so a block that finishes early takes more and
// no block idles long at the barrier (with a fixed item-to-block map some
// blocks ran phase A ~10 % longer than the rest and everyone waited).
__device__ __forceinline__ int next_item(unsigned *bar)
{
    __shared__ int s_w;
    __syncthreads();   // every thread is done with the previous item
    if (threadIdx.x == 0) s_w = (int)atomicAdd(bar + 3, 1u);
    __syncthreads();
    return s_w;
}

// Phase A's item order: kind-major (1: every tile's i faces, then every
// tile's j faces, then k, then the viscous items -- the blocks running at
// one time work on one direction, as the single-lattice passes do) or
// tile-major (0: the four kinds of a tile one after the other).  64
// vortices, tuned tiles: mixed 1.33e9 against 1.29e9 cell-updates/s, split
// 1.02e9 against 9.6e8.
#ifndef CFD_BATCH_KIND_MAJOR
#define CFD_BATCH_KIND_MAJOR 1
#endif

// Blocks of up to 256 threads (the tile sizes 32, 64, 128, 256); Ops::kMinBlocks
// bounds the registers so that many blocks stay resident (the mixed form is
// latency bound; the FP64 form keeps its registers).
template <class Ops>
__global__ void __launch_bounds__(256, Ops::kMinBlocks)
k_batch_stage(const LatView *__restrict__ views, const BatchTile *__restrict__ tiles, int ntiles, int jst,
              unsigned *bar, unsigned *gflags, unsigned long long limit_ns)
{
    // Item w: tile w % ntiles of kind w / ntiles (kind-major), or tile w >> 2
    // of kind w & 3 (the four items of a tile taken one after the other, by
    // different blocks at about the same time: they share the tile's data in
    // L2).
    const int items = 4 * ntiles;
    for (int w = next_item(bar); w < items; w = next_item(bar)) {
#if CFD_BATCH_KIND_MAJOR
        const BatchTile t = tiles[w % ntiles];
        const int kind = (w / ntiles + 1) & 3;   // i faces, j faces, k faces, then the viscous items
#else
        const BatchTile t = tiles[w >> 2];
        const int kind = w & 3;
#endif
        if ((int)threadIdx.x < t.count) {
            const LatView &g = views[t.inst];
            const int n = t.n0 + threadIdx.x;
            if (kind == 0) {
                if (g.P.viscous) Ops::visc(g, n, jst);
                else Ops::mu(g, n, jst);
            } else if (kind == 1) {
                Ops::template face<0>(g, n);
            } else if (kind == 2) {
                Ops::template face<1>(g, n);
            } else {
                Ops::template face<2>(g, n);
            }
        }
    }
    if (!grid_barrier(bar, gridDim.x, limit_ns, gflags)) return;
    for (int w = blockIdx.x; w < ntiles; w += gridDim.x) {
        const BatchTile t = tiles[w];
        if ((int)threadIdx.x < t.count) Ops::update(views[t.inst], t.n0 + threadIdx.x, jst);
    }
}

// One work item of phase A of the tiled form (the reduced-precision
// forms): kind 0 a viscous range of one lattice (a = first node, b = nodes),
// kind 1 + D a face tile along D (a = first face along D, b = first node
// across, c = line of the third axis; face_tile.cuh).
struct BatchItem {
    int inst, kind, a, b, c, pad;
};

// The persistent stage over items: phase A's face items stage their stencil
// lines in shared memory as the single-lattice face passes do (Ops::face_tile)
// instead of gathering each face's points through L1; phase B updates 1-D
// tiles (upd) of kFaceThreads nodes.  The item order (built on the host)
// rotates the kinds across rounds of the grid, as k_batch_stage does.
template <class Ops>
__global__ void __launch_bounds__(kFaceThreads, Ops::kMinBlocksTiled)
k_batch_stage_tiled(const LatView *__restrict__ views, const BatchItem *__restrict__ items, int nitems,
                    const BatchTile *__restrict__ upd, int nupd, int jst, unsigned *bar, unsigned *gflags,
                    unsigned long long limit_ns)
{
    __shared__ float smem[Ops::kTileSmemFloats];
    for (int w = next_item(bar); w < nitems; w = next_item(bar)) {
        const BatchItem it = items[w];
        const LatView &g = views[it.inst];
        const TileAt at{it.a, it.b, it.c};
        if (it.kind == 0) {
            if ((int)threadIdx.x < it.b) {
                if (g.P.viscous) Ops::visc(g, it.a + threadIdx.x, jst);
                else Ops::mu(g, it.a + threadIdx.x, jst);
            }
        } else if (it.kind == 1) {
            Ops::template face_tile<0>(g, at, smem);
        } else if (it.kind == 2) {
            Ops::template face_tile<1>(g, at, smem);
        } else {
            Ops::template face_tile<2>(g, at, smem);
        }
    }   // next_item synchronises the block before the next item restages smem
    if (!grid_barrier(bar, gridDim.x, limit_ns, gflags)) return;
    for (int w = blockIdx.x; w < nupd; w += gridDim.x) {
        const BatchTile t = upd[w];
        if ((int)threadIdx.x < t.count) Ops::update(views[t.inst], t.n0 + threadIdx.x, jst);
    }
}

// prep (U_Q) of stage 0 for one lattice, before its first stage
template <class Ops>
__global__ void k_batch_prep(LatView g)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < g.N) Ops::prep(g, n, 0);
}

}  // namespace cfd

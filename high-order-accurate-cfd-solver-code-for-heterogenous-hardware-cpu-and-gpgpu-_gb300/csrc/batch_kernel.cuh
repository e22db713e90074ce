// batch_kernel.cuh -- one persistent launch per RK stage over many lattices.
//
// Work is described by a tile table: tile t = (instance, first node, node
// count), tile size = block size, so one thread owns one node of a tile.
// A stage has two phases separated by a grid-wide barrier:
//   A  for every tile: viscous fluxes and the three face fluxes (4 work items
//      per tile, interleaved so that neighbouring blocks share a tile's data)
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

// Blocks of up to 256 threads (the tile sizes 64, 128, 256); Ops::kMinBlocks
// bounds the registers so that many blocks stay resident (the mixed form is
// latency bound; the FP64 form keeps its registers).
template <class Ops>
__global__ void __launch_bounds__(256, Ops::kMinBlocks)
k_batch_stage(const LatView *__restrict__ views, const BatchTile *__restrict__ tiles, int ntiles, int jst,
              unsigned *bar, unsigned *gflags, unsigned long long limit_ns)
{
    // Item w is tile w >> 2; the four items of a tile go to four neighbouring
    // blocks in the same round (they share the tile's data in L2).  The kind
    // is rotated by the round, (w & 3) + round, which is still a permutation
    // of the four kinds per tile: without it, a grid of a multiple of 4
    // blocks gives each block one kind for the whole phase, and the blocks
    // with the light viscous items idle at the barrier.
    const int items = 4 * ntiles;
    const int per_round = max(1, (int)gridDim.x >> 2);
    for (int w = blockIdx.x; w < items; w += gridDim.x) {
        const BatchTile t = tiles[w >> 2];
        const int kind = ((w & 3) + (w >> 2) / per_round) & 3;
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
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
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
        __syncthreads();   // the next item restages smem
    }
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

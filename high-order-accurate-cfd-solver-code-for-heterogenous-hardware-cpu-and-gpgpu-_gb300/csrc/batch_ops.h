// batch_ops.h -- host-side launch interface of the batched persistent kernel
// for the two precision forms (batch_fp64.cu, batch_mixed.cu).
#pragma once

#include <cuda_runtime.h>

#include "lattice.cuh"

namespace cfd {

struct BatchTile;
struct BatchItem;

// Face-tile shapes of the batched kernel's tiled form: faces along i x
// nodes across for i faces, faces along j or k for j and k faces
// (kFaceThreads faces per tile).  Shorter i tiles than the single-lattice
// pass: batched lattices are small (edges 32-96).
constexpr int kBatchTileI = 32;
constexpr int kBatchTileJK = 16;

struct BatchLaunch {
    const LatView *views;      // device table
    const BatchTile *tiles;    // device table
    int ntiles;
    int threads;               // = tile size
    int blocks;                // co-resident persistent grid
    unsigned *bar;             // device barrier words (2)
    unsigned *gflags;          // device error word of the batch
    unsigned long long limit_ns;
    cudaStream_t stream;
    // tiled form (reduced-precision forms): phase A items, phase B uses tiles
    const BatchItem *items = nullptr;
    int nitems = 0;
    int tiled = 0;
};

// One RK stage j (cooperative launch).  Returns the launch error.
cudaError_t batch_stage_fp64(const BatchLaunch &b, int j);
cudaError_t batch_stage_mixed(const BatchLaunch &b, int j);
cudaError_t batch_stage_split(const BatchLaunch &b, int j);
// Stage-0 prep of one lattice.
void batch_prep_fp64(const LatView &g, cudaStream_t st);
void batch_prep_mixed(const LatView &g, cudaStream_t st);
void batch_prep_split(const LatView &g, cudaStream_t st);
// Co-resident blocks per SM of the stage kernel at `threads` per block
// (tiled: the tiled form's kernel, kFaceThreads per block).
int batch_occupancy_fp64(int threads);
int batch_occupancy_mixed(int threads, bool tiled = false);
int batch_occupancy_split(int threads, bool tiled = false);

}  // namespace cfd

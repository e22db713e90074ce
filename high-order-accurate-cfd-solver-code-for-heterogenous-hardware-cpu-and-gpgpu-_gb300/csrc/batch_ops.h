// batch_ops.h -- host-side launch interface of the batched persistent kernel
// for the two precision forms (batch_fp64.cu, batch_mixed.cu).
#pragma once

#include <cuda_runtime.h>

#include "lattice.cuh"

namespace cfd {

struct BatchTile;

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
};

// One RK stage j (cooperative launch).  Returns the launch error.
cudaError_t batch_stage_fp64(const BatchLaunch &b, int j);
cudaError_t batch_stage_mixed(const BatchLaunch &b, int j);
cudaError_t batch_stage_split(const BatchLaunch &b, int j);
// Stage-0 prep of one lattice.
void batch_prep_fp64(const LatView &g, cudaStream_t st);
void batch_prep_mixed(const LatView &g, cudaStream_t st);
void batch_prep_split(const LatView &g, cudaStream_t st);
// Co-resident blocks per SM of the stage kernel at `threads` per block.
int batch_occupancy_fp64(int threads);
int batch_occupancy_mixed(int threads);
int batch_occupancy_split(int threads);

}  // namespace cfd

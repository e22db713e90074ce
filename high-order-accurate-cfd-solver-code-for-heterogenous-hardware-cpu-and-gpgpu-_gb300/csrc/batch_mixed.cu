// batch_mixed.cu -- the batched persistent stage kernel instantiated with the
// per-node operations of the mixed precision (FMA contraction, approximate FP32 division/sqrt) form.
#include "batch_kernel.cuh"
#include "batch_ops.h"
#include "internal.h"
#include "lattice_mixed.cuh"

namespace cfd {
namespace {

#ifndef CFD_MBATCH_MIN_BLOCKS
#define CFD_MBATCH_MIN_BLOCKS 3
#endif

struct Ops {
    static constexpr int kMinBlocks = CFD_MBATCH_MIN_BLOCKS;
    static __device__ __forceinline__ void prep(const LatView &g, int n, int q) { mx::init_node(g, n, q); }
    static __device__ __forceinline__ void visc(const LatView &g, int n, int q) { mx::visc_node<false>(g, n, q); }
    static __device__ __forceinline__ void mu(const LatView &g, int n, int q) { mx::mu_node(g, n, q); }
    template <int D>
    static __device__ __forceinline__ void face(const LatView &g, int n) { mx::face_node<D>(g, n); }
    // fluxes written by phase A of the same launch: coherent loads
    static __device__ __forceinline__ void update(const LatView &g, int n, int j) { mx::update_node<false, false>(g, n, j); }
};

}  // namespace

cudaError_t batch_stage_mixed(const BatchLaunch &b, int j)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b.blocks);
    cfg.blockDim = dim3(b.threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = b.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_batch_stage<Ops>, b.views, b.tiles, b.ntiles, j, b.bar, b.gflags, b.limit_ns);
}

void batch_prep_mixed(const LatView &g, cudaStream_t st)
{
    k_batch_prep<Ops><<<blocks_for(g.N, 128), 128, 0, st>>>(g);
}

int batch_occupancy_mixed(int threads)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_stage<Ops>, threads, 0) != cudaSuccess) return 0;
    return nb;
}

}  // namespace cfd

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

#ifndef CFD_MBATCH_TILED_MIN_BLOCKS
#define CFD_MBATCH_TILED_MIN_BLOCKS 6
#endif

template <int D>
using BTile = FaceTile<D, D == 0 ? kBatchTileI : kBatchTileJK>;

struct Ops {
    static constexpr int kMinBlocksTiled = CFD_MBATCH_TILED_MIN_BLOCKS;
    static constexpr int kTileSmemFloats =
        tile_smem_floats<BTile<0>>() > tile_smem_floats<BTile<1>>() ? tile_smem_floats<BTile<0>>() : tile_smem_floats<BTile<1>>();
    // the staged inputs were written by the previous launch: non-coherent loads
    template <int D>
    static __device__ __forceinline__ void face_tile(const LatView &g, TileAt at, float *smem)
    {
        mx::face_tile<BTile<D>, D>(g, at, smem);
    }
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
    cfg.blockDim = dim3(b.tiled ? kFaceThreads : b.threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = b.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (b.tiled)
        return cudaLaunchKernelEx(&cfg, k_batch_stage_tiled<Ops>, b.views, b.items, b.nitems, b.tiles, b.ntiles, j,
                                  b.bar, b.gflags, b.limit_ns);
    return cudaLaunchKernelEx(&cfg, k_batch_stage<Ops>, b.views, b.tiles, b.ntiles, j, b.bar, b.gflags, b.limit_ns);
}

void batch_prep_mixed(const LatView &g, cudaStream_t st)
{
    k_batch_prep<Ops><<<blocks_for(g.N, 128), 128, 0, st>>>(g);
}

int batch_occupancy_mixed(int threads, bool tiled)
{
    int nb = 0;
    const cudaError_t e = tiled ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_stage_tiled<Ops>,
                                                                               kFaceThreads, 0)
                                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_stage<Ops>, threads, 0);
    return e == cudaSuccess ? nb : 0;
}

}  // namespace cfd

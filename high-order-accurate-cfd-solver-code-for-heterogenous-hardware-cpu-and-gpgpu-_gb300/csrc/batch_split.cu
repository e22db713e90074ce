// batch_split.cu -- the batched persistent stage kernel instantiated with the
// per-node operations of the split precision form (lattice_split.cuh: FP64
// state, RK3 and face-flux metric products; FP32 characteristic WENO, LLF
// speed and viscous fluxes), compiled with FMA contraction and approximate
// FP32 division/sqrt.
#include "batch_kernel.cuh"
#include "batch_ops.h"
#include "internal.h"
#include "lattice_split.cuh"

namespace cfd {
namespace {

#ifndef CFD_SBATCH_MIN_BLOCKS
#define CFD_SBATCH_MIN_BLOCKS 3
#endif

#ifndef CFD_SBATCH_TILED_MIN_BLOCKS
#define CFD_SBATCH_TILED_MIN_BLOCKS 5
#endif

template <int D>
using BTile = FaceTile<D, D == 0 ? kBatchTileI : kBatchTileJK>;

struct Ops {
    static constexpr int kMinBlocksTiled = CFD_SBATCH_TILED_MIN_BLOCKS;
    static constexpr int kTileSmemFloats =
        tile_smem_floats<BTile<0>>() > tile_smem_floats<BTile<1>>() ? tile_smem_floats<BTile<0>>() : tile_smem_floats<BTile<1>>();
    // the staged inputs were written by the previous launch: non-coherent loads
    template <int D>
    static __device__ __forceinline__ void face_tile(const LatView &g, TileAt at, float *smem)
    {
        sp::face_tile<BTile<D>, D>(g, at, smem);
    }
    static constexpr int kMinBlocks = CFD_SBATCH_MIN_BLOCKS;
    static __device__ __forceinline__ void prep(const LatView &g, int n, int q) { sp::init_node(g, n, q); }
    // the viscous pass on the hi/lo read copy of the stage's state
    static __device__ __forceinline__ void visc(const LatView &g, int n, int) { mx::visc_node<false>(sp::hilo_view(g), n, 0); }
    static __device__ __forceinline__ void mu(const LatView &g, int n, int) { mx::mu_node(sp::hilo_view(g), n, 0); }
    template <int D>
    static __device__ __forceinline__ void face(const LatView &g, int n) { sp::face_node<D>(g, n); }
    // fluxes written by phase A of the same launch: coherent loads
    static __device__ __forceinline__ void update(const LatView &g, int n, int j) { sp::update_node<false, false>(g, n, j); }
};

}  // namespace

cudaError_t batch_stage_split(const BatchLaunch &b, int j)
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

void batch_prep_split(const LatView &g, cudaStream_t st)
{
    k_batch_prep<Ops><<<blocks_for(g.N, 128), 128, 0, st>>>(g);
}

int batch_occupancy_split(int threads, bool tiled)
{
    int nb = 0;
    const cudaError_t e = tiled ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_stage_tiled<Ops>,
                                                                               kFaceThreads, 0)
                                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_stage<Ops>, threads, 0);
    return e == cudaSuccess ? nb : 0;
}

}  // namespace cfd

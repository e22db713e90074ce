// batch_fp64.cu -- the batched persistent stage kernel instantiated with the
// per-node operations of the exact FP64 evaluation order (compiled with --fmad=false) form.
// The batched stage runs 8 warps per SM: too few to hide the integer
// product's latency, so the divisions' first quotient comes from the FP64
// multiply (exact_div.cuh, CFD_XDIV_QPROD; the same bits either way).
#define CFD_XDIV_QPROD 0
#include "batch_kernel.cuh"
#include "batch_ops.h"
#include "internal.h"
#include "lattice_fp64.cuh"

namespace cfd {
namespace {

// 1: shared reciprocals in the face flux (exact_div.cuh), as in the
// single-lattice kernels; 0: a division per quotient.  Same bits either
// way; with the quotients' rounding on the integer pipe the shared form is
// the faster here too (64 vortices: 2.30e7 against 2.15e7 cell-updates/s).
#ifndef CFD_FBATCH_SHARED_DIV
#define CFD_FBATCH_SHARED_DIV 1
#endif

struct Ops {
    static constexpr int kMinBlocks = 1;
    static __device__ __forceinline__ void prep(const LatView &g, int n, int q) { ex::prep_node(g, n, q); }
    static __device__ __forceinline__ void visc(const LatView &g, int n, int q) { ex::visc_node(g, n, q); }
    static __device__ __forceinline__ void mu(const LatView &g, int n, int q) { ex::mu_node(g, n, q); }
    template <int D>
    static __device__ __forceinline__ void face(const LatView &g, int n)
    {
        ex::face_node<D, CFD_FBATCH_SHARED_DIV != 0>(g, n);
    }
    static __device__ __forceinline__ void update(const LatView &g, int n, int j) { ex::update_node(g, n, j, true); }
};

}  // namespace

cudaError_t batch_stage_fp64(const BatchLaunch &b, int j)
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

void batch_prep_fp64(const LatView &g, cudaStream_t st)
{
    k_batch_prep<Ops><<<blocks_for(g.N, 128), 128, 0, st>>>(g);
}

int batch_occupancy_fp64(int threads)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_stage<Ops>, threads, 0) != cudaSuccess) return 0;
    return nb;
}

}  // namespace cfd

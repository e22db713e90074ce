// face_fp64_mb2.cu -- the FP64 lattice face passes at 2 blocks of 128 per SM
// (face_fp64.cuh).
// 2 blocks of 128 per SM: too few warps to hide the integer product's
// latency, so the divisions' first quotient comes from the FP64 multiply
// (exact_div.cuh, CFD_XDIV_QPROD; the same bits either way).
#define CFD_XDIV_QPROD 0
#include "face_fp64.cuh"

namespace cfd {

void fp64_face_pass_mb2(const LatView &g, int d, cudaStream_t st) { face_pass<2>(g, d, st); }

}  // namespace cfd

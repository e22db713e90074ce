// face_fp64_mb4.cu -- the FP64 lattice face passes at 4 blocks of 128 per SM
// (face_fp64.cuh).
#include "face_fp64.cuh"

namespace cfd {

void fp64_face_pass_mb4(const LatView &g, int d, cudaStream_t st) { face_pass<4>(g, d, st); }

}  // namespace cfd

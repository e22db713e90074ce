// face_fp64_mb3.cu -- the FP64 lattice face passes at 3 blocks of 128 per SM
// (face_fp64.cuh).
#include "face_fp64.cuh"

namespace cfd {

void fp64_face_pass_mb3(const LatView &g, int d, cudaStream_t st) { face_pass<3>(g, d, st); }

}  // namespace cfd

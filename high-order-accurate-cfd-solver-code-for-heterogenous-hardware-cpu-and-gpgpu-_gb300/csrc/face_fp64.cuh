// face_fp64.cuh -- the FP64 lattice face pass (one thread per face n+1/2
// along D: Roe average, LLF face flux and the sixth-order correction of
// lattice_fp64.cuh face_node) at a register budget MB, the blocks of 128
// threads per SM its launch bounds request.  face_fp64_mb2.cu, _mb3.cu and
// _mb4.cu each compile one budget (in parallel; the 2-block unit forms its
// divisions' first quotient and reciprocal on the FP64 pipe, the others on
// the integer pipe, exact_div.cuh); the solver times the three per
// direction at its second stage and keeps the fastest (the arithmetic is
// the same in each: the same bits).  Include only from translation units
// compiled with --fmad=false.
#pragma once

#include "internal.h"
#include "lattice_fp64.cuh"
#include "structured.h"

namespace cfd {
namespace {

template <int D, int MB>
__global__ void __launch_bounds__(128, MB) k_face(LatView g)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < g.N) ex::face_node<D>(g, n);
}

template <int MB>
void face_pass(const LatView &g, int d, cudaStream_t st)
{
    const unsigned nb = blocks_for(g.N, 128);
    if (d == 0)
        k_face<0, MB><<<nb, 128, 0, st>>>(g);
    else if (d == 1)
        k_face<1, MB><<<nb, 128, 0, st>>>(g);
    else
        k_face<2, MB><<<nb, 128, 0, st>>>(g);
}

}  // namespace
}  // namespace cfd

// exact_div_gpu.cu -- cfd::xdiv::div(x, b, 1/b) on the GPU against the GPU's
// own IEEE division x / b, bit for bit, on the pairs of div_cases.h.
//
//   exact_div_gpu <rounds> <seed>
#include <cstdio>
#include <cstdlib>

#include "div_cases.h"
#include "exact_div.cuh"

__global__ void k_div(const double *x, const double *b, int n, double *want, double *got)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double y = 1.0 / b[i];
    want[i] = x[i] / b[i];
    got[i] = cfd::xdiv::div(x[i], b[i], y);
}

int main(int argc, char **argv)
{
    const long rounds = argc > 1 ? std::atol(argv[1]) : 100000;
    const uint64_t seed = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1;
    std::vector<double> X, B;
    divcases::make(rounds, seed, X, B);
    const int n = (int)X.size();
    double *dx, *db, *dw, *dg;
    const size_t bytes = (size_t)n * sizeof(double);
    if (cudaMalloc(&dx, bytes) || cudaMalloc(&db, bytes) || cudaMalloc(&dw, bytes) || cudaMalloc(&dg, bytes)) {
        std::printf("cudaMalloc failed\n");
        return 2;
    }
    cudaMemcpy(dx, X.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(db, B.data(), bytes, cudaMemcpyHostToDevice);
    k_div<<<(n + 255) / 256, 256>>>(dx, db, n, dw, dg);
    std::vector<double> W(n), G(n);
    cudaMemcpy(W.data(), dw, bytes, cudaMemcpyDeviceToHost);
    cudaMemcpy(G.data(), dg, bytes, cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaDeviceSynchronize();
    long fails = 0, host_diff = 0;
    for (int i = 0; i < n; ++i) {
        const bool same = divcases::to_bits(G[i]) == divcases::to_bits(W[i]) || (std::isnan(G[i]) && std::isnan(W[i]));
        fails += !same;
        volatile double hx = X[i], hb = B[i];
        const double h = hx / hb;
        host_diff += !(divcases::to_bits(h) == divcases::to_bits(W[i]) || (std::isnan(h) && std::isnan(W[i])));
    }
    std::printf("exact_div_gpu: %d cases, %ld mismatches against the GPU division, %ld GPU/host division "
                "differences (%s)\n", n, fails, host_diff, cudaGetErrorString(e));
    cudaFree(dx);
    cudaFree(db);
    cudaFree(dw);
    cudaFree(dg);
    return (fails == 0 && e == cudaSuccess) ? 0 : 1;
}

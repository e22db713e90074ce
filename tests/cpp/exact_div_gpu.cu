// exact_div_gpu.cu -- cfd::xdiv::div(x, b, 1/b) on the GPU against the GPU's
// own IEEE division x / b, bit for bit, on the pairs of div_cases.h,
// cfd::xdiv::scale2<K>(x) against the GPU's x * 2^K on every x, pow2_over,
// and the integer-pipe reciprocal (rcp_int) and single division (divide).
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

// the reciprocal of b[i] with its rounding on the integer pipe
// (xdiv::rcp_int where it accepts b, else the division) and x / b through
// xdiv::divide, against the GPU's 1.0 / b and x / b: out[2 * i + k]
__global__ void k_rcp(const double *x, const double *b, int n, double *want, double *got)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool ok;
    const double y = cfd::xdiv::rcp_int(b[i], ok);
    got[2 * i + 0] = ok ? y : 1.0 / b[i];
    want[2 * i + 0] = 1.0 / b[i];
    got[2 * i + 1] = cfd::xdiv::divide(x[i], b[i]);
    want[2 * i + 1] = x[i] / b[i];
}

// out[6 * i + k]: scale2 of x[i] by 2, 4, 8, 1/2, 1/4, 1/8 (got) and the
// FP64 products (want)
__global__ void k_scale(const double *x, int n, const double *c, double *want, double *got)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    got[6 * i + 0] = cfd::xdiv::scale2<1>(v);
    got[6 * i + 1] = cfd::xdiv::scale2<2>(v);
    got[6 * i + 2] = cfd::xdiv::scale2<3>(v);
    got[6 * i + 3] = cfd::xdiv::scale2<-1>(v);
    got[6 * i + 4] = cfd::xdiv::scale2<-2>(v);
    got[6 * i + 5] = cfd::xdiv::scale2<-3>(v);
    for (int k = 0; k < 6; ++k) want[6 * i + k] = v * c[k];
}

// out[3 * i + k]: pow2_over of x[i] for 2^-4, 2^-1, 2^3 (got) and the FP64
// divisions (want)
__global__ void k_pow2_over(const double *x, int n, const double *c, double *want, double *got)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    got[3 * i + 0] = cfd::xdiv::pow2_over<-4>(v);
    got[3 * i + 1] = cfd::xdiv::pow2_over<-1>(v);
    got[3 * i + 2] = cfd::xdiv::pow2_over<3>(v);
    for (int k = 0; k < 3; ++k) want[3 * i + k] = c[k] / v;
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
    // scale2 on every x and b (2n operands, 6 factors each)
    const double cs[6] = {2.0, 4.0, 8.0, 0.5, 0.25, 0.125};
    std::vector<double> V(X);
    V.insert(V.end(), B.begin(), B.end());
    const int m = (int)V.size();
    double *dv, *dc, *sw, *sg;
    long sfails = 0;
    cudaError_t e2 = cudaSuccess;
    if (cudaMalloc(&dv, m * sizeof(double)) || cudaMalloc(&dc, sizeof cs) || cudaMalloc(&sw, 6 * (size_t)m * 8)
        || cudaMalloc(&sg, 6 * (size_t)m * 8)) {
        std::printf("cudaMalloc failed\n");
        return 2;
    }
    cudaMemcpy(dv, V.data(), m * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(dc, cs, sizeof cs, cudaMemcpyHostToDevice);
    k_scale<<<(m + 255) / 256, 256>>>(dv, m, dc, sw, sg);
    std::vector<double> SW(6 * (size_t)m), SG(6 * (size_t)m);
    cudaMemcpy(SW.data(), sw, SW.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(SG.data(), sg, SG.size() * 8, cudaMemcpyDeviceToHost);
    e2 = cudaDeviceSynchronize();
    for (size_t i = 0; i < SW.size(); ++i)
        sfails += !(divcases::to_bits(SG[i]) == divcases::to_bits(SW[i]) || (std::isnan(SG[i]) && std::isnan(SW[i])));
    std::printf("scale2: %zu cases, %ld scale2 mismatches (%s)\n", SW.size(), sfails, cudaGetErrorString(e2));
    // pow2_over on every x and b (3 numerators each), reusing the buffers
    const double pc[3] = {0.0625, 0.5, 8.0};
    cudaMemcpy(dc, pc, sizeof pc, cudaMemcpyHostToDevice);
    k_pow2_over<<<(m + 255) / 256, 256>>>(dv, m, dc, sw, sg);
    std::vector<double> PW(3 * (size_t)m), PG(3 * (size_t)m);
    cudaMemcpy(PW.data(), sw, PW.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(PG.data(), sg, PG.size() * 8, cudaMemcpyDeviceToHost);
    const cudaError_t e3 = cudaDeviceSynchronize();
    long pfails = 0;
    for (size_t i = 0; i < PW.size(); ++i)
        pfails += !(divcases::to_bits(PG[i]) == divcases::to_bits(PW[i]) || (std::isnan(PG[i]) && std::isnan(PW[i])));
    std::printf("pow2_over: %zu cases, %ld pow2_over mismatches (%s)\n", PW.size(), pfails, cudaGetErrorString(e3));
    sfails += pfails;
    if (e3 != cudaSuccess) e2 = e3;
    // reciprocals and single divisions on the pairs (x, b), reusing the buffers (2n <= 6m entries)
    k_rcp<<<(n + 255) / 256, 256>>>(dx, db, n, sw, sg);
    std::vector<double> RW(2 * (size_t)n), RG(2 * (size_t)n);
    cudaMemcpy(RW.data(), sw, RW.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(RG.data(), sg, RG.size() * 8, cudaMemcpyDeviceToHost);
    const cudaError_t e4 = cudaDeviceSynchronize();
    long rfails = 0;
    for (size_t i = 0; i < RW.size(); ++i)
        rfails += !(divcases::to_bits(RG[i]) == divcases::to_bits(RW[i]) || (std::isnan(RG[i]) && std::isnan(RW[i])));
    std::printf("rcp/divide: %zu cases, %ld rcp mismatches (%s)\n", RW.size(), rfails, cudaGetErrorString(e4));
    sfails += rfails;
    if (e4 != cudaSuccess) e2 = e4;
    cudaFree(dv);
    cudaFree(dc);
    cudaFree(sw);
    cudaFree(sg);
    cudaFree(dx);
    cudaFree(db);
    cudaFree(dw);
    cudaFree(dg);
    return (fails == 0 && sfails == 0 && e == cudaSuccess && e2 == cudaSuccess) ? 0 : 1;
}

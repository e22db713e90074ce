// probe.cu -- measured arithmetic peaks (cfd_probe_flops), a public
// diagnostic: the FP64 path is bounded by the FP64 pipe and the reduced
// forms partly by FP32, so their roofline denominators are measured here:
// independent FMA chains (8 per thread, no memory traffic), timed with CUDA
// events.  HBM bandwidth and tensor throughput are measured elsewhere.
#include "internal.h"

namespace cfd {
namespace {

template <class T>
__global__ void __launch_bounds__(256) k_fma_chain(int iters, T b, T c, T *out)
{
    T a0 = (T)threadIdx.x * (T)1e-3, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
    T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
        a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
    const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == (T)-12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;   // keeps the chains live
}

template <class T>
cfd_status_t run_probe(cfd_ctx *ctx, int iters, double *flops)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256, blocks = sms * 8;
    T *out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(T) * (size_t)threads * blocks);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "probe alloc");
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(t0, ctx->stream);
        k_fma_chain<T><<<blocks, threads, 0, ctx->stream>>>(iters, (T)0.999999, (T)1e-7, out);
        cudaEventRecord(t1, ctx->stream);
        e = cudaEventSynchronize(t1);
        if (e != cudaSuccess) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, t0, t1);
        if (ms < best) best = ms;
    }
    ctx->launches += 3;
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFree(out);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "probe run");
    *flops = 2.0 * 8.0 * (double)iters * threads * blocks / (best * 1e-3);
    return CFD_OK;
}

}  // namespace
}  // namespace cfd

extern "C" cfd_status_t cfd_probe_flops(cfd_ctx_t *ctx, int32_t fp64, double *flops_per_s)
{
    if (!ctx || !flops_per_s) return CFD_EINVAL;
    cfd_status_t s = cfd::use_device(ctx);
    if (s != CFD_OK) return s;
    return fp64 ? cfd::run_probe<double>(ctx, 2048, flops_per_s) : cfd::run_probe<float>(ctx, 65536, flops_per_s);
}

// probe.cu -- public diagnostics.  cfd_probe_flops: measured arithmetic
// peaks; the FP64 path is bounded by the FP64 pipe and the reduced forms
// partly by FP32, so their roofline denominators are measured here:
// independent FMA chains (8 per thread, no memory traffic), timed with CUDA
// events.  HBM bandwidth and tensor throughput are measured elsewhere.
// cfd_probe_emu64: the integer-pipe binary64 routines (emu64.cuh) against
// the hardware instructions on seeded operands.
#include "emu64.cuh"
#include "exact_div.cuh"
#include "internal.h"

namespace cfd {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// A seeded binary64 operand of class cls: 0 everyday magnitudes, 1 the full
// exponent range, 2 sparse significands (rounding ties), 3 zeros,
// subnormals, infinities, NaN and the ends of the range, 4 around the
// binary32 range (for the conversions); 5 (second operand only) close to
// minus the first (cancellation).
__device__ double operand(uint64_t &st, int cls, double first, bool second)
{
    const uint64_t r = mix64(st++), r2 = mix64(st++);
    const uint64_t sign = (r2 & 1u) << 63;
    uint64_t man = r & emu::kFrac, ex;
    switch (cls) {
    case 0: ex = 1000 + (r2 >> 8) % 47; break;
    case 1: ex = 1 + (r2 >> 8) % 2046; break;
    case 2:
        man &= mix64(st++) & mix64(st++);
        ex = 980 + (r2 >> 8) % 87;
        break;
    case 3: {
        const int k = (int)((r2 >> 8) % 8);
        if (k == 0) return 0.0;
        if (k == 1) return -0.0;
        if (k == 2) return emu::f64(sign | man);
        if (k == 3) return emu::f64(sign | (0x7ffULL << 52));
        if (k == 4) return emu::f64(0x7ff8000000000000ULL | man);
        ex = k == 5 ? 1 + (r2 >> 12) % 60 : (k == 6 ? 2046 - (r2 >> 12) % 60 : 1000 + (r2 >> 8) % 47);
        break;
    }
    case 4: ex = 860 + (r2 >> 8) % 330; break;
    default: {
        if (!second) {
            ex = 1000 + (r2 >> 8) % 47;
            break;
        }
        const uint64_t uo = emu::u64(first);
        const uint64_t eo = ((uo >> 52) & 0x7ff) + (uint64_t)((r2 >> 8) % 3) - 1;
        const uint64_t pert = (r >> 3) & ((1ull << ((r2 >> 16) % 53)) - 1);
        return emu::f64(((~uo) & emu::kSign) | (eo << 52) | (((uo & emu::kFrac) ^ pert) & emu::kFrac));
    }
    }
    return emu::f64(sign | (ex << 52) | man);
}

__device__ __forceinline__ bool same64(double x, double y) { return (x != x && y != y) || emu::u64(x) == emu::u64(y); }
__device__ __forceinline__ bool same32(float x, float y)
{
    return (x != x && y != y) || __float_as_uint(x) == __float_as_uint(y);
}

// per thread `per` operand pairs of class cls; bad[0..4] count the
// mismatches of f2d, d2f (and the hi/lo split), add/sub, mul and the
// division from a shared reciprocal (xdiv::quotient_int_v, both ways of
// forming its first quotient, where it accepts the operands; xdiv::div) and
// the reciprocal (rcp_int and rcp_int_i, rcp, divide)
__global__ void k_emu_check(int cls, uint64_t seed, int per, unsigned long long *bad)
{
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t st = mix64(seed ^ (t * 0x632be59bd9b4e019ULL) ^ ((uint64_t)cls << 56));
    unsigned long long nb[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < per; ++i) {
        const double a = operand(st, cls, 0.0, false);
        const double b = operand(st, cls, a, true);
        const float fa = __uint_as_float((uint32_t)mix64(st++));   // every binary32 bit pattern
        nb[0] += !same64(emu::f2d(fa), (double)fa) + !same64(emu::f2d(__double2float_rn(a)), (double)__double2float_rn(a));
        nb[1] += !same32(emu::d2f(a), __double2float_rn(a)) + !same32(emu::d2f(b), __double2float_rn(b));
        {
            float h, l;
            emu::hi_lo(a, h, l);
            const float hn = __double2float_rn(a);
            const float ln = __double2float_rn(__dsub_rn(a, (double)hn));
            nb[1] += !same32(h, hn) + !same32(l, ln);
        }
        nb[2] += !same64(emu::add(a, b), __dadd_rn(a, b)) + !same64(emu::sub(a, b), __dsub_rn(a, b));
        nb[3] += !same64(emu::mul(a, b), __dmul_rn(a, b));
        {
            const double y = 1.0 / b;
            bool ok;
            const double q = xdiv::quotient_int_v<1>(a, b, y, ok);   // first quotient: integer product
            nb[4] += ok && !same64(q, a / b);
            const double qf = xdiv::quotient_int_v<0>(a, b, y, ok);  // first quotient: FP64 product
            nb[4] += ok && !same64(qf, a / b);
            nb[4] += !same64(xdiv::div(a, b, y), a / b);
            const double yi = xdiv::rcp_int(b, ok);   // Newton step on the FP64 pipe
            nb[4] += ok && !same64(yi, y);
            const double yj = xdiv::rcp_int_i(b, ok);   // on the integer pipe
            nb[4] += ok && !same64(yj, y);
            nb[4] += !same64(xdiv::rcp(b), y) + !same64(xdiv::divide(a, b), a / b);
        }
    }
    for (int k = 0; k < 5; ++k)
        if (nb[k]) atomicAdd(bad + k, nb[k]);
}

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

extern "C" cfd_status_t cfd_probe_emu64(cfd_ctx_t *ctx, int64_t n_per_class, uint64_t seed, int64_t mismatches[5])
{
    if (!ctx || !mismatches || n_per_class < 1) return CFD_EINVAL;
    cfd_status_t s = cfd::use_device(ctx);
    if (s != CFD_OK) return s;
    const int threads = 256;
    const int per = 64;
    const long long blocks = (n_per_class + (long long)threads * per - 1) / ((long long)threads * per);
    if (blocks > (1LL << 30)) return CFD_EINVAL;
    unsigned long long *bad = nullptr;
    cudaError_t e = cudaMalloc(&bad, 5 * sizeof(unsigned long long));
    if (e != cudaSuccess) return cfd::cuda_fail(ctx, e, "cfd_probe_emu64 alloc");
    cudaMemsetAsync(bad, 0, 5 * sizeof(unsigned long long), ctx->stream);
    for (int cls = 0; cls < 6; ++cls) cfd::k_emu_check<<<(unsigned)blocks, threads, 0, ctx->stream>>>(cls, seed, per, bad);
    ctx->launches += 6;
    unsigned long long h[5] = {0, 0, 0, 0, 0};
    e = cudaMemcpyAsync(h, bad, sizeof h, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(bad);
    if (e != cudaSuccess) return cfd::cuda_fail(ctx, e, "cfd_probe_emu64");
    for (int k = 0; k < 5; ++k) mismatches[k] = (int64_t)h[k];
    return CFD_OK;
}

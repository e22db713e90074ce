// mixed.cu -- face-flux kernels of the mixed-precision form.
//
// Characteristic projection, WENO weights and the LLF split run in FP32
// (physics.cuh, templated on the compute type, FMA-friendly rewrites: one
// division per WENO side, reciprocal of rho reused); the stencil inputs, the
// Roe state inputs and the sixth-order correction stay FP64 and the result is
// accumulated in FP64 by the FP64 update kernel.  Compiled with FMA
// contraction on.
#include "internal.h"
#include "structured.h"

namespace cfd {

namespace {

__device__ __forceinline__ int wrapm(int x, int n)
{
    x %= n;
    return x < 0 ? x + n : x;
}

enum { MU_ = 0, MV_ = 1, MW_ = 2 };

template <int D>
__global__ void __launch_bounds__(128) k_face_mixed(int ni, int nj, int nk, float eps, const double *__restrict__ Q,
                                                    const double *__restrict__ prim9, const double *__restrict__ sh,
                                                    const double *__restrict__ fm, const double *__restrict__ fdet,
                                                    const double *__restrict__ FEG, double *__restrict__ Fh)
{
    const long long N = (long long)ni * nj * nk;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int i = (int)(n % ni);
    const long long r_ = n / ni;
    const int j = (int)(r_ % nj), k = (int)(r_ / nj);
    long long s[6];
#pragma unroll
    for (int o = 0; o < 6; ++o) {
        const int ii = D == 0 ? wrapm(i + o - 2, ni) : i;
        const int jj = D == 1 ? wrapm(j + o - 2, nj) : j;
        const int kk = D == 2 ? wrapm(k + o - 2, nk) : k;
        s[o] = (long long)ii + (long long)ni * ((long long)jj + (long long)nj * kk);
    }
    float pts[6][5];
#pragma unroll
    for (int o = 0; o < 6; ++o)
#pragma unroll
        for (int c = 0; c < 5; ++c) pts[o][c] = (float)Q[c * N + s[o]];
    float roe[5];
    {
        const long long l = s[2], r = s[3];
        roe_average<float>((float)sh[r], (float)prim9[MU_ * N + r], (float)prim9[MV_ * N + r],
                           (float)prim9[MW_ * N + r], (float)sh[N + r], (float)sh[l], (float)prim9[MU_ * N + l],
                           (float)prim9[MV_ * N + l], (float)prim9[MW_ * N + l], (float)sh[N + l], roe);
    }
    float Fhat[5];
    llf_face_flux<float>(pts, (float)fm[(D * 3 + 0) * N + n], (float)fm[(D * 3 + 1) * N + n],
                         (float)fm[(D * 3 + 2) * N + n], (float)fdet[D * N + n], roe, eps, Fhat);
    const double *NF = FEG + (size_t)D * 5 * N;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        double f[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) f[o] = NF[c * N + s[o]];
        Fh[(D * 5 + c) * N + n] = (double)Fhat[c] + face_correction(f);
    }
}

}  // namespace

void launch_faces_mixed(const StructuredLaunch &S, cudaEvent_t *ev)
{
    const long long N = (long long)S.ni * S.nj * S.nk;
    const unsigned nb = blocks_for(N, 128);
    const float e = (float)S.P.eps;
    k_face_mixed<0><<<nb, 128, 0, S.stream>>>(S.ni, S.nj, S.nk, e, S.Q, S.prim9, S.sh, S.fm, S.fdet, S.FEG, S.Fh);
    if (ev) cudaEventRecord(ev[0], S.stream);
    k_face_mixed<1><<<nb, 128, 0, S.stream>>>(S.ni, S.nj, S.nk, e, S.Q, S.prim9, S.sh, S.fm, S.fdet, S.FEG, S.Fh);
    if (ev) cudaEventRecord(ev[1], S.stream);
    k_face_mixed<2><<<nb, 128, 0, S.stream>>>(S.ni, S.nj, S.nk, e, S.Q, S.prim9, S.sh, S.fm, S.fdet, S.FEG, S.Fh);
    if (ev) cudaEventRecord(ev[2], S.stream);
}

}  // namespace cfd

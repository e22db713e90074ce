// static_stage.cu -- one SSP-RK3 stage on a periodic lattice that allocates
// no device memory.
//
// Some callers cannot call cudaMalloc while they advance a solution: code
// that runs inside a host framework owning a fixed device-memory pool, a
// real-time loop where an allocation (and the implicit device synchronisation
// that cudaMalloc/cudaFree may cause) is not allowed, or a plugin that is only
// handed buffers.  For them, cfd_lattice_stage_static runs the same kernels
// as the resident solver's structured path, but keeps every intermediate of
// the stage (structure-of-arrays copies of the inputs, node fluxes, viscous
// fluxes, face fluxes, the error word) in one library-owned array declared
// below, sized for at most CFD_STATIC_MAX_NODES lattice nodes.
//
// The array exists once per GPU that loads the library and stays allocated
// until the process exits.  All calls share it: two calls whose work
// overlaps on the GPU (different streams, or different host threads using
// the same device) race on it and produce garbage; callers must serialise
// them.  Host code cannot use the array's name as a device address, so the
// first call on each device looks the address up with cudaGetSymbolAddress
// (with that device current) and caches it; make that first call before any
// stream capture begins.  The cached address belongs to the device's
// current context: after cudaDeviceReset the process must not call the
// entry point again.
#include <mutex>

#include "internal.h"
#include "structured.h"

namespace cfd {
namespace {

// doubles per lattice node held in the scratch array:
//   geometry SoA 22 (9 node metrics, det, 3x3 face metrics, 3 face dets),
//   FLOW 9, U0/U1/U2 15, Q 5, node fluxes 15, viscous fluxes 15,
//   sqrt(rho) and H 2, face fluxes 15, L 5
constexpr size_t kPerNode = 22 + 9 + 15 + 5 + 15 + 15 + 2 + 15 + 5;   // 103
constexpr size_t kFlagDoubles = 32;                                    // 256 B for the error word
constexpr size_t kScratchDoubles = (size_t)CFD_STATIC_MAX_NODES * kPerNode + kFlagDoubles;

static __device__ __align__(256) double g_stage_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device).
cfd_status_t scratch_address(double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return CFD_ECUDA;
    if (dev < 0 || dev >= kMaxDevices) return CFD_EUNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_stage_scratch);
        if (e != cudaSuccess || !p) return CFD_ECUDA;
        g_scratch_addr[dev] = (double *)p;
    }
    *out = g_scratch_addr[dev];
    return CFD_OK;
}

// rows 1..N of an AoS buffer (row stride `stride` doubles, columns
// offset..offset+ncomp-1) <-> SoA [ncomp][N]
__global__ void k_cols_to_soa(const double *__restrict__ aos, int stride, int offset, int ncomp, long long N,
                              double *__restrict__ soa)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * ncomp) return;
    const long long n = t / ncomp;
    const int c = (int)(t % ncomp);
    soa[c * N + n] = aos[(n + 1) * stride + offset + c];
}

__global__ void k_soa_to_cols(const double *__restrict__ soa, int stride, int offset, int ncomp, long long N,
                              double *__restrict__ aos)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * ncomp) return;
    const long long n = t / ncomp;
    const int c = (int)(t % ncomp);
    aos[(n + 1) * stride + offset + c] = soa[c * N + n];
}

void to_soa(cudaStream_t st, const double *aos, int stride, int offset, int ncomp, long long N, double *soa)
{
    k_cols_to_soa<<<blocks_for(N * ncomp, 256), 256, 0, st>>>(aos, stride, offset, ncomp, N, soa);
}

void from_soa(cudaStream_t st, const double *soa, int stride, int offset, int ncomp, long long N, double *aos)
{
    k_soa_to_cols<<<blocks_for(N * ncomp, 256), 256, 0, st>>>(soa, stride, offset, ncomp, N, aos);
}

}  // namespace
}  // namespace cfd

extern "C" cfd_status_t cfd_lattice_stage_static(void *cuda_stream, int32_t ni, int32_t nj, int32_t nk, int32_t j,
                                                 double del_t, const cfd_params_t *params, const double *det,
                                                 const cfd_determ_t *deter, const cfd_metric_t *metric,
                                                 cfd_column_t *U0, cfd_column_t *U1, cfd_column_t *U2,
                                                 cfd_flow_t *FLOW, cfd_column_t *L_out)
{
    using namespace cfd;
    if (ni < 1 || nj < 1 || nk < 1 || j < 0 || j > 2) return CFD_EINVAL;
    const long long N = (long long)ni * nj * nk;
    if (N > CFD_STATIC_MAX_NODES) return CFD_EINVAL;   // beyond the static scratch array
    if (!det || !deter || !metric || !U0 || !U1 || !U2 || !FLOW) return CFD_EINVAL;
    if (params && params->precision != CFD_PREC_FP64) return CFD_EUNSUPPORTED;   // FP64 form only
    if (cudaPeekAtLastError() != cudaSuccess) return CFD_ECUDA;   // an earlier error, left for the caller
    double *base = nullptr;
    cfd_status_t s = scratch_address(&base);
    if (s != CFD_OK) return s;
    cudaStream_t st = (cudaStream_t)cuda_stream;

    // carve the scratch array (N nodes used, SoA [component][N])
    double *p = base;
    auto take = [&](size_t comps) {
        double *q = p;
        p += comps * (size_t)N;
        return q;
    };
    StructuredLaunch S{};
    S.ni = ni;
    S.nj = nj;
    S.nk = nk;
    S.stream = st;
    S.P = make_phys(params);
    S.mixed = 0;
    double *m9 = take(9), *dt_ = take(1), *fm = take(9), *fdet = take(3);
    S.m9 = m9;
    S.det = dt_;
    S.fm = fm;
    S.fdet = fdet;
    S.prim9 = take(9);
    S.U[0] = take(5);
    S.U[1] = take(5);
    S.U[2] = take(5);
    S.Q = take(5);
    S.FEG = take(15);
    S.V = take(15);
    S.sh = take(2);
    S.Fh = take(15);
    double *Lsoa = take(5);
    S.flags = (unsigned *)(base + (size_t)CFD_STATIC_MAX_NODES * kPerNode);

    // the error word must start at zero; every other region is written
    // before it is read within this call
    cudaError_t e = cudaMemsetAsync(S.flags, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return CFD_ECUDA;

    // reference layout (rows 1..N) -> SoA
    to_soa(st, det, 1, 0, 1, N, dt_);
    to_soa(st, (const double *)metric, 63, 0, 9, N, m9);
    for (int d = 0; d < 3; ++d) {
        to_soa(st, (const double *)metric, 63, 9 * (1 + 2 * d) + 3 * d, 3, N, fm + (size_t)3 * d * N);
        to_soa(st, (const double *)deter, 6, 2 * d, 1, N, fdet + (size_t)d * N);
    }
    to_soa(st, (const double *)FLOW, 9, 0, 9, N, S.prim9);
    to_soa(st, (const double *)U0, 5, 0, 5, N, S.U[0]);
    to_soa(st, (const double *)U1, 5, 0, 5, N, S.U[1]);
    to_soa(st, (const double *)U2, 5, 0, 5, N, S.U[2]);

    structured_stage(S, j, del_t, L_out ? Lsoa : nullptr);

    // results back into the caller's buffers: FLOW, U_j (U_Q's output),
    // the U the stage advanced, and L
    cfd_column_t *Ucaller[3] = {U0, U1, U2};
    const int advanced = j == 0 ? 1 : (j == 1 ? 2 : 0);
    from_soa(st, S.prim9, 9, 0, 9, N, (double *)FLOW);
    from_soa(st, S.U[j], 5, 0, 5, N, (double *)Ucaller[j]);
    from_soa(st, S.U[advanced], 5, 0, 5, N, (double *)Ucaller[advanced]);
    if (L_out) from_soa(st, Lsoa, 5, 0, 5, N, (double *)L_out);

    // peek, not get: a failed launch stays readable by the caller's own checks
    e = cudaPeekAtLastError();
    if (e != cudaSuccess) return CFD_ECUDA;
    unsigned flags = 0;
    e = cudaMemcpyAsync(&flags, S.flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return CFD_ECUDA;
    if (flags & CFD_FLAG_NONFINITE) return CFD_ENONFINITE;
    return CFD_OK;
}

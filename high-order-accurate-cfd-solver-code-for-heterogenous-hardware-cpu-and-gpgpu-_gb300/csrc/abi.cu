// abi.cu -- context, buffers and the three drop-in entry points of the C ABI.
#include <cstring>

#include "internal.h"

namespace cfd {

cfd_status_t fail(cfd_ctx *ctx, cfd_status_t s, const std::string &msg)
{
    if (ctx) ctx->last_error = msg;
    return s;
}

cfd_status_t cuda_fail(cfd_ctx *ctx, cudaError_t e, const char *what)
{
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(ctx, e == cudaErrorMemoryAllocation ? CFD_ENOMEM : CFD_ECUDA, msg);
}

cfd_status_t use_device(cfd_ctx *ctx)
{
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != ctx->device) {
        cudaError_t e = cudaSetDevice(ctx->device);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
    }
    return CFD_OK;
}

cfd_status_t flags_to_status(cfd_ctx *ctx, unsigned flags)
{
    if (flags & CFD_FLAG_BAD_INDEX) return fail(ctx, CFD_EINVAL, "neighbour index outside [0, n_rows)");
    if (flags & CFD_FLAG_TIMEOUT) return fail(ctx, CFD_ETIMEOUT, "bounded device wait expired");
    if (flags & CFD_FLAG_NONFINITE) return fail(ctx, CFD_ENONFINITE, "non-finite value in the advanced state");
    return CFD_OK;
}

cfd_status_t drain(cfd_ctx *ctx)
{
    cudaError_t e = cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "flag readback");
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
    unsigned f = *ctx->h_flags;
    if (f) {
        e = cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "flag reset");
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
    }
    return flags_to_status(ctx, f);
}

cfd_status_t after_launch(cfd_ctx *ctx, const char *what)
{
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    if (ctx->async) return CFD_OK;
    return drain(ctx);
}

bool is_device_pointer(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

Phys make_phys(const cfd_params_t *p)
{
    cfd_params_t d;
    cfd_params_default(&d);
    if (!p) p = &d;
    Phys P;
    P.mach = p->mach;
    P.reynolds = p->reynolds;
    P.prandtl = p->prandtl;
    P.t_inf = p->t_inf;
    P.eps = p->weno_eps;
    P.viscous = p->viscous;
    P.les = p->les;
    return P;
}

}  // namespace cfd

using namespace cfd;

extern "C" {

void cfd_params_default(cfd_params_t *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->mach = 1.5;
    p->reynolds = 500.0;
    p->prandtl = 0.72;
    p->t_inf = 273.0;
    p->weno_eps = 10e-8;
    p->viscous = 1;
    p->les = 1;
    p->precision = CFD_PREC_FP64;
}

const char *cfd_status_string(cfd_status_t s)
{
    switch (s) {
    case CFD_OK: return "ok";
    case CFD_EINVAL: return "invalid argument";
    case CFD_ENONFINITE: return "non-finite state";
    case CFD_ETIMEOUT: return "device wait timed out";
    case CFD_ECUDA: return "CUDA error";
    case CFD_ENOMEM: return "out of device memory";
    case CFD_EUNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

const char *cfd_last_error(const cfd_ctx_t *ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

cfd_status_t cfd_ctx_create(cfd_ctx_t **out, int device)
{
    if (!out) return CFD_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return CFD_ECUDA;
    }
    if (device < 0 || device >= n) return CFD_EINVAL;
    cfd_ctx *ctx = new cfd_ctx();
    ctx->device = device;
    cfd_status_t s = use_device(ctx);
    if (s != CFD_OK) { delete ctx; return s; }
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_flags, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_flags, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_flags, sizeof(unsigned));
    if (e != cudaSuccess) {
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        if (ctx->d_flags) cudaFree(ctx->d_flags);
        delete ctx;
        return e == cudaErrorMemoryAllocation ? CFD_ENOMEM : CFD_ECUDA;
    }
    ctx->own_stream = true;
    *out = ctx;
    return CFD_OK;
}

cfd_status_t cfd_ctx_destroy(cfd_ctx_t *ctx)
{
    if (!ctx) return CFD_EINVAL;
    use_device(ctx);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->d_flags) cudaFree(ctx->d_flags);
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->d_face) cudaFree(ctx->d_face);
    delete ctx;
    return CFD_OK;
}

cfd_status_t cfd_ctx_set_stream(cfd_ctx_t *ctx, void *stream)
{
    if (!ctx) return CFD_EINVAL;
    if (ctx->own_stream && ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    ctx->stream = (cudaStream_t)stream;
    ctx->own_stream = false;
    return CFD_OK;
}

cfd_status_t cfd_ctx_set_async(cfd_ctx_t *ctx, int async)
{
    if (!ctx) return CFD_EINVAL;
    ctx->async = async != 0;
    return CFD_OK;
}

cfd_status_t cfd_ctx_synchronize(cfd_ctx_t *ctx)
{
    if (!ctx) return CFD_EINVAL;
    cfd_status_t s = use_device(ctx);
    if (s != CFD_OK) return s;
    return drain(ctx);
}

cfd_status_t cfd_ctx_set_rows(cfd_ctx_t *ctx, int32_t n_rows)
{
    if (!ctx || n_rows <= 0) return fail(ctx, CFD_EINVAL, "n_rows must be positive");
    ctx->n_rows = n_rows;
    // cfd_weno's face scratch; without it (no memory) cfd_weno evaluates
    // both faces per row, with the same results
    if (ctx->face_rows < n_rows) {
        cfd_status_t s = use_device(ctx);
        if (s != CFD_OK) return s;
        if (ctx->d_face) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->d_face);
        }
        ctx->d_face = nullptr;
        ctx->face_rows = 0;
        if (cudaMalloc(&ctx->d_face, (size_t)n_rows * 15 * sizeof(double)) == cudaSuccess)
            ctx->face_rows = n_rows;
        else {
            cudaGetLastError();
            ctx->d_face = nullptr;
        }
    }
    return CFD_OK;
}

cfd_status_t cfd_ctx_set_face_reuse(cfd_ctx_t *ctx, int on)
{
    if (!ctx) return CFD_EINVAL;
    ctx->face_reuse = on != 0;
    return CFD_OK;
}

uint64_t cfd_ctx_launch_count(const cfd_ctx_t *ctx) { return ctx ? ctx->launches : 0; }

cfd_status_t cfd_buffer_alloc(cfd_ctx_t *ctx, size_t bytes, void **dev)
{
    if (!ctx || !dev || bytes == 0) return fail(ctx, CFD_EINVAL, "cfd_buffer_alloc: bad argument");
    cfd_status_t s = use_device(ctx);
    if (s != CFD_OK) return s;
    cudaError_t e = cudaMalloc(dev, bytes);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc");
    return CFD_OK;
}

cfd_status_t cfd_buffer_free(cfd_ctx_t *ctx, void *dev)
{
    if (!ctx) return CFD_EINVAL;
    use_device(ctx);
    cudaError_t e = cudaFree(dev);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaFree");
    return CFD_OK;
}

cfd_status_t cfd_buffer_write(cfd_ctx_t *ctx, void *dst, const void *src, size_t bytes)
{
    if (!ctx || !dst || !src) return fail(ctx, CFD_EINVAL, "cfd_buffer_write: null pointer");
    cfd_status_t s = use_device(ctx);
    if (s != CFD_OK) return s;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpyAsync H2D");
    if (!ctx->async) {
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
    }
    return CFD_OK;
}

cfd_status_t cfd_buffer_read(cfd_ctx_t *ctx, void *dst, const void *src, size_t bytes)
{
    if (!ctx || !dst || !src) return fail(ctx, CFD_EINVAL, "cfd_buffer_read: null pointer");
    cfd_status_t s = use_device(ctx);
    if (s != CFD_OK) return s;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpyAsync D2H");
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
    return CFD_OK;
}

static cfd_status_t check_launch_args(cfd_ctx_t *ctx, int32_t n_items, std::initializer_list<const void *> ptrs,
                                      const char *who)
{
    if (!ctx) return CFD_EINVAL;
    if (ctx->n_rows <= 0) return fail(ctx, CFD_EINVAL, std::string(who) + ": call cfd_ctx_set_rows first");
    if (n_items <= 0 || n_items > ctx->n_rows)
        return fail(ctx, CFD_EINVAL, std::string(who) + ": n_items must be in [1, n_rows]");
    cfd_status_t s = use_device(ctx);
    if (s != CFD_OK) return s;
    for (const void *p : ptrs)
        if (!is_device_pointer(p)) return fail(ctx, CFD_EINVAL, std::string(who) + ": buffers must be device pointers");
    return CFD_OK;
}

cfd_status_t cfd_uq(cfd_ctx_t *ctx, cfd_column_t *U_C, cfd_column_t *Q_C, const cfd_grid_t *Grid_P, const double *det,
                    cfd_flow_t *FLOW, cfd_roe_t *ROE_AVER, int32_t n_items)
{
    cfd_status_t s = check_launch_args(ctx, n_items, {U_C, Q_C, Grid_P, det, FLOW, ROE_AVER}, "cfd_uq");
    if (s != CFD_OK) return s;
    launch_uq(ctx->stream, (double *)U_C, (double *)Q_C, (const int *)Grid_P, det, (const double *)FLOW,
              (double *)ROE_AVER, n_items, ctx->n_rows, ctx->d_flags);
    return after_launch(ctx, "cfd_uq launch");
}

cfd_status_t cfd_viscous(cfd_ctx_t *ctx, cfd_column_t *U_C, cfd_column_t *F_C, cfd_column_t *E_C, cfd_column_t *G_C,
                         cfd_column_t *Fv_C, cfd_column_t *Ev_C, cfd_column_t *Gv_C, const cfd_grid_t *Grid_P,
                         const cfd_metric_t *metric, const double *det, cfd_flow_t *FLOW, int32_t n_items,
                         const cfd_params_t *params)
{
    cfd_status_t s = check_launch_args(ctx, n_items, {U_C, F_C, E_C, G_C, Fv_C, Ev_C, Gv_C, Grid_P, metric, det, FLOW},
                                       "cfd_viscous");
    if (s != CFD_OK) return s;
    launch_viscous(ctx->stream, make_phys(params), (const double *)U_C, (double *)F_C, (double *)E_C, (double *)G_C,
                   (double *)Fv_C, (double *)Ev_C, (double *)Gv_C, (const int *)Grid_P, (const double *)metric, det,
                   (double *)FLOW, n_items, ctx->n_rows, ctx->d_flags);
    return after_launch(ctx, "cfd_viscous launch");
}

cfd_status_t cfd_weno(cfd_ctx_t *ctx, int32_t j, double Mach, double del_t, const cfd_determ_t *deter,
                      const double *det, cfd_column_t *U0, cfd_column_t *U1, cfd_column_t *U2,
                      const cfd_grid_t *Grid_P, cfd_column_t *Q_C, const cfd_metric_t *metric, cfd_roe_t *ROE_AVER,
                      cfd_column_t *Fv, cfd_column_t *Ev, cfd_column_t *Gv, cfd_column_t *F, cfd_column_t *E,
                      cfd_column_t *G, cfd_flow_t *FLOW, int32_t n_items, const cfd_params_t *params,
                      cfd_column_t *L_out)
{
    if (j < 0 || j > 2) return fail(ctx, CFD_EINVAL, "cfd_weno: stage j must be 0, 1 or 2");
    cfd_status_t s = check_launch_args(
        ctx, n_items, {deter, det, U0, U1, U2, Grid_P, Q_C, metric, ROE_AVER, Fv, Ev, Gv, F, E, G, FLOW}, "cfd_weno");
    if (s != CFD_OK) return s;
    if (L_out && !is_device_pointer(L_out)) return fail(ctx, CFD_EINVAL, "cfd_weno: L_out must be a device pointer");
    launch_weno(ctx->stream, make_phys(params), j, Mach, del_t, (const double *)deter, det, (double *)U0, (double *)U1,
                (double *)U2, (const int *)Grid_P, (const double *)Q_C, (const double *)metric,
                (const double *)ROE_AVER, (const double *)Fv, (const double *)Ev, (const double *)Gv,
                (const double *)F, (const double *)E, (const double *)G, (double *)FLOW, n_items, ctx->n_rows,
                ctx->d_flags, (double *)L_out, ctx->face_reuse ? ctx->d_face : nullptr, ctx->face_rows);
    ctx->launches += weno_launches(ctx->face_reuse ? ctx->d_face : nullptr, ctx->face_rows, n_items) - 1;
    return after_launch(ctx, "cfd_weno launch");
}

}  // extern "C"

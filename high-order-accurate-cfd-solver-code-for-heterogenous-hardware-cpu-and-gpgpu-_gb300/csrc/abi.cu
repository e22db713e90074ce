// abi.cu -- context, buffers and the three drop-in entry points of the C ABI.
#include <cstring>

#include "boundary.h"
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
    P.cs = p->smagorinsky_cs;
    return P;
}

}  // namespace cfd

using namespace cfd;

namespace cfd {

cfd_status_t stage_in(cfd_ctx *ctx, BufArg *a, int n, const char *who)
{
    for (int i = 0; i < n; ++i) {
        BufArg &b = a[i];
        if (!b.user) return fail(ctx, CFD_EINVAL, std::string(who) + ": null buffer");
        if (is_device_pointer(b.user)) {
            b.dev = b.user;
            continue;
        }
        const size_t bytes = (size_t)(b.rows > 0 ? b.rows : ctx->n_rows) * b.row_bytes;
        auto it = ctx->mirrors.find(b.user);
        if (it == ctx->mirrors.end() || it->second.second < bytes) {
            if (it != ctx->mirrors.end()) {
                cudaStreamSynchronize(ctx->stream);
                cudaFree(it->second.first);
                ctx->mirrors.erase(it);
            }
            void *d = nullptr;
            cudaError_t e = cudaMalloc(&d, bytes);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "device mirror of a host buffer");
            it = ctx->mirrors.emplace(b.user, std::make_pair(d, bytes)).first;
        }
        b.dev = it->second.first;
        b.host = true;
        cudaError_t e = cudaMemcpyAsync(b.dev, b.user, bytes, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "host buffer copy in");
    }
    return CFD_OK;
}

cfd_status_t stage_out(cfd_ctx *ctx, const BufArg *a, int n, cfd_status_t launch_status)
{
    if (launch_status == CFD_ECUDA || launch_status == CFD_ENOMEM) return launch_status;
    bool any = false;
    for (int i = 0; i < n; ++i)
        if (a[i].host && a[i].written) {
            const size_t bytes = (size_t)(a[i].rows > 0 ? a[i].rows : ctx->n_rows) * a[i].row_bytes;
            cudaError_t e = cudaMemcpyAsync(a[i].user, a[i].dev, bytes, cudaMemcpyDeviceToHost, ctx->stream);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "host buffer copy out");
            any = true;
        }
    if (any) {
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
    }
    return launch_status;
}

}  // namespace cfd

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
    p->smagorinsky_cs = 0.1;
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
    for (auto &m : ctx->mirrors) cudaFree(m.second.first);
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
        void *buf = nullptr;
        if (cudaMalloc(&buf, face_scratch_bytes(n_rows)) == cudaSuccess) {
            double *f = static_cast<double *>(buf);
            if (cudaMemset(face_stamps(f, n_rows), 0, (size_t)n_rows * 3 * sizeof(unsigned)) == cudaSuccess) {
                ctx->d_face = f;
                ctx->face_rows = n_rows;
            } else {
                cudaFree(buf);
            }
        }
        cudaGetLastError();   // a failed allocation only disables the sharing
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

static cfd_status_t check_launch_args(cfd_ctx_t *ctx, int32_t n_items, const char *who)
{
    if (!ctx) return CFD_EINVAL;
    if (ctx->n_rows <= 0) return fail(ctx, CFD_EINVAL, std::string(who) + ": call cfd_ctx_set_rows first");
    if (n_items <= 0 || n_items > ctx->n_rows)
        return fail(ctx, CFD_EINVAL, std::string(who) + ": n_items must be in [1, n_rows]");
    return use_device(ctx);
}


cfd_status_t cfd_uq(cfd_ctx_t *ctx, cfd_column_t *U_C, cfd_column_t *Q_C, const cfd_grid_t *Grid_P, const double *det,
                    cfd_flow_t *FLOW, cfd_roe_t *ROE_AVER, int32_t n_items)
{
    cfd_status_t s = check_launch_args(ctx, n_items, "cfd_uq");
    if (s != CFD_OK) return s;
    BufArg a[] = {{U_C, 40, true}, {Q_C, 40, true}, {(void *)Grid_P, 56, false}, {(void *)det, 8, false},
                  {FLOW, 72, false}, {ROE_AVER, 288, true}};
    if ((s = stage_in(ctx, a, 6, "cfd_uq")) != CFD_OK) return s;
    ctx->launches += launch_uq(ctx->stream, (double *)a[0].dev, (double *)a[1].dev, (const int *)a[2].dev,
                               (const double *)a[3].dev, (const double *)a[4].dev, (double *)a[5].dev, n_items,
                               ctx->n_rows, ctx->d_flags, ctx->face_reuse ? ctx->d_face : nullptr,
                               ctx->face_rows) - 1;
    return stage_out(ctx, a, 6, after_launch(ctx, "cfd_uq launch"));
}

cfd_status_t cfd_viscous(cfd_ctx_t *ctx, cfd_column_t *U_C, cfd_column_t *F_C, cfd_column_t *E_C, cfd_column_t *G_C,
                         cfd_column_t *Fv_C, cfd_column_t *Ev_C, cfd_column_t *Gv_C, const cfd_grid_t *Grid_P,
                         const cfd_metric_t *metric, const double *det, cfd_flow_t *FLOW, int32_t n_items,
                         const cfd_params_t *params)
{
    cfd_status_t s = check_launch_args(ctx, n_items, "cfd_viscous");
    if (s != CFD_OK) return s;
    BufArg a[] = {{U_C, 40, false},  {F_C, 40, true},    {E_C, 40, true},           {G_C, 40, true},
                  {Fv_C, 40, true},  {Ev_C, 40, true},   {Gv_C, 40, true},          {(void *)Grid_P, 56, false},
                  {(void *)metric, 504, false}, {(void *)det, 8, false}, {FLOW, 72, true}};
    if ((s = stage_in(ctx, a, 11, "cfd_viscous")) != CFD_OK) return s;
    launch_viscous(ctx->stream, make_phys(params), (const double *)a[0].dev, (double *)a[1].dev, (double *)a[2].dev,
                   (double *)a[3].dev, (double *)a[4].dev, (double *)a[5].dev, (double *)a[6].dev,
                   (const int *)a[7].dev, (const double *)a[8].dev, (const double *)a[9].dev, (double *)a[10].dev,
                   n_items, ctx->n_rows, ctx->d_flags);
    return stage_out(ctx, a, 11, after_launch(ctx, "cfd_viscous launch"));
}

cfd_status_t cfd_weno(cfd_ctx_t *ctx, int32_t j, double Mach, double del_t, const cfd_determ_t *deter,
                      const double *det, cfd_column_t *U0, cfd_column_t *U1, cfd_column_t *U2,
                      const cfd_grid_t *Grid_P, cfd_column_t *Q_C, const cfd_metric_t *metric, cfd_roe_t *ROE_AVER,
                      cfd_column_t *Fv, cfd_column_t *Ev, cfd_column_t *Gv, cfd_column_t *F, cfd_column_t *E,
                      cfd_column_t *G, cfd_flow_t *FLOW, int32_t n_items, const cfd_params_t *params,
                      cfd_column_t *L_out)
{
    if (!ctx) return CFD_EINVAL;
    if (j < 0 || j > 2) return fail(ctx, CFD_EINVAL, "cfd_weno: stage j must be 0, 1 or 2");
    cfd_status_t s = check_launch_args(ctx, n_items, "cfd_weno");
    if (s != CFD_OK) return s;
    BufArg a[] = {{(void *)deter, 48, false}, {(void *)det, 8, false},     {U0, 40, j == 2},
                  {U1, 40, j == 0},           {U2, 40, j == 1},            {(void *)Grid_P, 56, false},
                  {Q_C, 40, false},           {(void *)metric, 504, false}, {ROE_AVER, 288, false},
                  {Fv, 40, false},            {Ev, 40, false},             {Gv, 40, false},
                  {F, 40, false},             {E, 40, false},              {G, 40, false},
                  {FLOW, 72, true}};
    if ((s = stage_in(ctx, a, 16, "cfd_weno")) != CFD_OK) return s;
    BufArg l[] = {{L_out, 40, true}};
    if (L_out && (s = stage_in(ctx, l, 1, "cfd_weno")) != CFD_OK) return s;
    double *const face = ctx->face_reuse ? ctx->d_face : nullptr;
    launch_weno(ctx->stream, make_phys(params), j, Mach, del_t, (const double *)a[0].dev, (const double *)a[1].dev,
                (double *)a[2].dev, (double *)a[3].dev, (double *)a[4].dev, (const int *)a[5].dev,
                (const double *)a[6].dev, (const double *)a[7].dev, (const double *)a[8].dev,
                (const double *)a[9].dev, (const double *)a[10].dev, (const double *)a[11].dev,
                (const double *)a[12].dev, (const double *)a[13].dev, (const double *)a[14].dev, (double *)a[15].dev,
                n_items, ctx->n_rows, ctx->d_flags, L_out ? (double *)l[0].dev : nullptr, face, ctx->face_rows,
                next_face_gen(ctx->face_gen));
    ctx->launches += weno_launches(face, ctx->face_rows, n_items) - 1;
    s = stage_out(ctx, a, 16, after_launch(ctx, "cfd_weno launch"));
    return L_out ? stage_out(ctx, l, 1, s) : s;
}

cfd_status_t cfd_rk3_step(cfd_ctx_t *ctx, double Mach, double del_t, const cfd_determ_t *deter, const double *det,
                          cfd_column_t *U0, cfd_column_t *U1, cfd_column_t *U2, const cfd_grid_t *Grid_P,
                          cfd_column_t *Q_C, const cfd_metric_t *metric, cfd_roe_t *ROE_AVER, cfd_column_t *Fv,
                          cfd_column_t *Ev, cfd_column_t *Gv, cfd_column_t *F, cfd_column_t *E, cfd_column_t *G,
                          cfd_flow_t *FLOW, int32_t g_node, int32_t sd_node, const cfd_params_t *params,
                          const cfd_bc_t *bc, int32_t nsteps)
{
    if (!ctx) return CFD_EINVAL;
    if (nsteps < 1) return fail(ctx, CFD_EINVAL, "cfd_rk3_step: nsteps must be at least 1");
    if (sd_node < 1 || sd_node > g_node) return fail(ctx, CFD_EINVAL, "cfd_rk3_step: need 1 <= sd_node <= g_node");
    cfd_status_t s = check_launch_args(ctx, g_node + 1, "cfd_rk3_step");
    if (s != CFD_OK) return s;
    if (bc && bc->n_rows != ctx->n_rows)
        return fail(ctx, CFD_EINVAL, "cfd_rk3_step: boundary lists were made for another table");
    BufArg a[] = {{(void *)deter, 48, false}, {(void *)det, 8, false},     {U0, 40, true},
                  {U1, 40, true},             {U2, 40, true},              {(void *)Grid_P, 56, false},
                  {Q_C, 40, true},            {(void *)metric, 504, false}, {ROE_AVER, 288, true},
                  {Fv, 40, true},             {Ev, 40, true},              {Gv, 40, true},
                  {F, 40, true},              {E, 40, true},               {G, 40, true},
                  {FLOW, 72, true}};
    if ((s = stage_in(ctx, a, 16, "cfd_rk3_step")) != CFD_OK) return s;
    const Phys P = make_phys(params);
    double *const face = ctx->face_reuse ? ctx->d_face : nullptr;
    double *U[3] = {(double *)a[2].dev, (double *)a[3].dev, (double *)a[4].dev};
    const int *grid = (const int *)a[5].dev;
    const double *dt_ = (const double *)a[0].dev, *dd = (const double *)a[1].dev, *met = (const double *)a[7].dev;
    double *Q = (double *)a[6].dev, *roe = (double *)a[8].dev, *flow = (double *)a[15].dev;
    double *Fv_ = (double *)a[9].dev, *Ev_ = (double *)a[10].dev, *Gv_ = (double *)a[11].dev;
    double *F_ = (double *)a[12].dev, *E_ = (double *)a[13].dev, *G_ = (double *)a[14].dev;
    uint64_t n = 0;
    for (int step = 0; step < nsteps; ++step)
        for (int j = 0; j < 3; ++j) {   // Solver.cpp:365-658, j passed per stage
            n += launch_uq(ctx->stream, U[j], Q, grid, dd, flow, roe, g_node + 1, ctx->n_rows, ctx->d_flags, face,
                           ctx->face_rows);
            launch_viscous(ctx->stream, P, U[j], F_, E_, G_, Fv_, Ev_, Gv_, grid, met, dd, flow, g_node + 1,
                           ctx->n_rows, ctx->d_flags);
            launch_weno(ctx->stream, P, j, Mach, del_t, dt_, dd, U[0], U[1], U[2], grid, Q, met, roe, Fv_, Ev_, Gv_,
                        F_, E_, G_, flow, sd_node + 1, ctx->n_rows, ctx->d_flags, nullptr, face, ctx->face_rows,
                        next_face_gen(ctx->face_gen));
            n += 1 + weno_launches(face, ctx->face_rows, sd_node + 1);
            if (bc) {
                bc_apply_aos(ctx->stream, bc->dev, flow, Mach);
                n += bc->dev.launches();
            }
        }
    ctx->launches += n - 1;
    return stage_out(ctx, a, 16, after_launch(ctx, "cfd_rk3_step launches"));
}

}  // extern "C"

// solver.cu -- resident solver object: the reference host loop
// (Solver.cpp:356-658, stages U_Q -> Viscous -> Weno(j)) run on the device
// with the state kept in device memory between stages and steps.
//
// Path selection at create time:
//   CFD_PATH_STRUCTURED  the neighbour table is an (i,j,k) lattice --
//                        periodic, or with non-periodic directions padded by
//                        ghost layers (lattice_host.h) -- with single-valued
//                        face data -> face-based SoA kernels (structured.cu,
//                        mixed.cu)
//   CFD_PATH_GATHER      anything else -> the drop-in kernels on the
//                        reference layout (dropin.cu), the same code the
//                        cfd_uq/cfd_viscous/cfd_weno entry points run
// With cfd_solver_set_boundary the reference's boundary routine
// (Flow_Initialisation.cpp, boundary.cu) runs after every stage, as the host
// loop calls it (Solver.cpp:658).
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "boundary.h"
#include "internal.h"
#include "lattice_host.h"
#include "structured.h"

struct cfd_solver {
    cfd_ctx *ctx = nullptr;
    cfd_params_t prm{};
    cfd::Phys P{};
    int path = CFD_PATH_GATHER;
    int32_t g_node = 0, sd_node = 0, n_rows = 0;
    int ni = 0, nj = 0, nk = 0;
    bool mixed = false;         // a reduced-precision form (mixed or split): U slots tracked below
    int form = CFD_PREC_FP64;   // cfd_precision_t
    std::vector<void *> allocs;
    uint64_t bytes = 0;
    // gather path (reference layout, device)
    int *grid = nullptr;
    double *det = nullptr, *deter = nullptr, *metric = nullptr, *flow = nullptr;
    double *U[3] = {nullptr, nullptr, nullptr};
    double *Q = nullptr, *F = nullptr, *E = nullptr, *G = nullptr, *Fv = nullptr, *Ev = nullptr, *Gv = nullptr;
    double *roe = nullptr, *L = nullptr;
    double *face = nullptr;     // gather path: the Weno pass's face scratch (face_scratch_bytes(n_rows))
    unsigned face_gen = 0;
    // structured path
    cfd::StructuredLaunch S{};
    double *stage9 = nullptr;   // AoS staging, rows 0..N, 9 doubles
    double *stage5 = nullptr;   // AoS staging, rows 0..N, 5 doubles
    double *Lsoa = nullptr;
    // mixed form: the U slot holding the current state (-1: the uploaded FP64
    // FLOW is current) and the stage whose U_Q outputs are ready (-1: none)
    int cur_slot = -1;
    int prep_ready = -1;
    cfd::LatticeMap map;        // lattice path: rows <-> nodes
    cfd::BcDevice bc;           // boundary routine after every stage
    bool has_bc = false;
    int fp64_tune = -1;         // FP64 lattice: stages before the face passes' budgets are timed (-1: none)
};

namespace {

using namespace cfd;

cfd_status_t dalloc(cfd_solver *s, size_t bytes, void **p)
{
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "cudaMalloc (solver)");
    s->allocs.push_back(*p);
    s->bytes += bytes;
    return CFD_OK;
}

template <class T>
cfd_status_t dalloc_t(cfd_solver *s, size_t count, T **p)
{
    return dalloc(s, count * sizeof(T), (void **)p);
}

cfd_status_t upload(cfd_solver *s, void *dst, const void *src, size_t bytes)
{
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "cudaMemcpyAsync H2D (solver)");
    return CFD_OK;
}

cfd_status_t create_gather(cfd_solver *s, const cfd_geometry_t *g)
{
    const size_t R = (size_t)s->n_rows;
    cfd_status_t st;
    if ((st = dalloc_t(s, R * 14, &s->grid)) || (st = dalloc_t(s, R, &s->det)) || (st = dalloc_t(s, R * 6, &s->deter))
        || (st = dalloc_t(s, R * 63, &s->metric)) || (st = dalloc_t(s, R * 9, &s->flow)))
        return st;
    for (int q = 0; q < 3; ++q)
        if ((st = dalloc_t(s, R * 5, &s->U[q]))) return st;
    double **c5[] = {&s->Q, &s->F, &s->E, &s->G, &s->Fv, &s->Ev, &s->Gv, &s->L};
    for (double **p : c5)
        if ((st = dalloc_t(s, R * 5, p))) return st;
    if ((st = dalloc_t(s, R * 36, &s->roe)) || (st = dalloc(s, face_scratch_bytes((long long)R), (void **)&s->face)))
        return st;
    cudaMemsetAsync(face_stamps(s->face, (long long)R), 0, R * 3 * sizeof(unsigned), s->ctx->stream);
    for (int q = 0; q < 3; ++q) cudaMemsetAsync(s->U[q], 0, R * 5 * sizeof(double), s->ctx->stream);
    for (double **p : c5) cudaMemsetAsync(*p, 0, R * 5 * sizeof(double), s->ctx->stream);
    cudaMemsetAsync(s->roe, 0, R * 36 * sizeof(double), s->ctx->stream);
    if ((st = upload(s, s->grid, g->grid, R * sizeof(cfd_grid_t))) || (st = upload(s, s->det, g->det, R * 8))
        || (st = upload(s, s->deter, g->deter, R * 48)) || (st = upload(s, s->metric, g->metric, R * 504)))
        return st;
    cudaError_t e = cudaStreamSynchronize(s->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "solver create sync");
    return CFD_OK;
}

cfd_status_t tune_face_tiles(cfd_solver *s);
cfd_status_t tune_fp64_faces(cfd_solver *s, int j);

cfd_status_t create_structured(cfd_solver *s, const cfd_geometry_t *g)
{
    const size_t N = (size_t)s->ni * s->nj * s->nk;
    StructuredLaunch &S = s->S;
    S.per = s->map.per;
    S.locdirs = s->map.locdirs;
    S.ni = s->ni;
    S.nj = s->nj;
    S.nk = s->nk;
    S.stream = s->ctx->stream;
    S.P = s->P;
    S.mixed = s->form;
    S.flags = s->ctx->d_flags;
    double *m9, *det, *fm, *fdet;
    cfd_status_t st;
    if ((st = dalloc_t(s, 9 * N, &m9)) || (st = dalloc_t(s, N, &det)) || (st = dalloc_t(s, 9 * N, &fm))
        || (st = dalloc_t(s, 3 * N, &fdet)) || (st = dalloc_t(s, 9 * N, &S.prim9))
        || (st = dalloc_t(s, 9 * (N + 1), &s->stage9)) || (st = dalloc_t(s, 5 * (N + 1), &s->stage5))
        || (st = dalloc_t(s, 5 * N, &s->Lsoa)))
        return st;
    for (int q = 0; q < 3; ++q)
        if ((st = dalloc_t(s, 5 * N, &S.U[q]))) return st;
    if (s->form == CFD_PREC_SPLIT) {   // FP32 stage intermediates, FP64 face fluxes
        if ((st = dalloc_t(s, 5 * N, &S.Q32)) || (st = dalloc_t(s, 5 * N, &S.R32)) || (st = dalloc_t(s, 15 * N, &S.FEG32))
            || (st = dalloc_t(s, 15 * N, &S.V32)) || (st = dalloc_t(s, 15 * N, &S.Fh))
            || (st = dalloc_t(s, 9 * N, &S.fm32)) || (st = dalloc_t(s, 11 * N, &S.node32))
            || (st = dalloc_t(s, N, &S.idet64)) || (st = dalloc_t(s, 9 * N, &S.prim32))
            || (st = dalloc_t(s, 10 * N, &S.Whl)))
            return st;
        cudaMemsetAsync(S.V32, 0, 15 * N * sizeof(float), S.stream);
    } else if (s->mixed) {   // FP32 stage intermediates
        if ((st = dalloc_t(s, 5 * N, &S.Q32)) || (st = dalloc_t(s, 5 * N, &S.R32)) || (st = dalloc_t(s, 15 * N, &S.FEG32))
            || (st = dalloc_t(s, 15 * N, &S.V32)) || (st = dalloc_t(s, 15 * N, &S.Fh32))
            || (st = dalloc_t(s, 9 * N, &S.fm32)) || (st = dalloc_t(s, 3 * N, &S.fdet32))
            || (st = dalloc_t(s, 11 * N, &S.node32)) || (st = dalloc_t(s, 2 * N, &S.idet32))
            || (st = dalloc_t(s, 9 * N, &S.prim32)))
            return st;
        cudaMemsetAsync(S.V32, 0, 15 * N * sizeof(float), S.stream);
    } else {          // FP64 stage intermediates
        if ((st = dalloc_t(s, 5 * N, &S.Q)) || (st = dalloc_t(s, 15 * N, &S.FEG)) || (st = dalloc_t(s, 15 * N, &S.V))
            || (st = dalloc_t(s, 2 * N, &S.sh)) || (st = dalloc_t(s, 15 * N, &S.Fh)))
            return st;
        cudaMemsetAsync(S.V, 0, 15 * N * sizeof(double), S.stream);
    }
    for (int q = 0; q < 3; ++q) cudaMemsetAsync(S.U[q], 0, 5 * N * sizeof(double), S.stream);
    cudaMemsetAsync(s->stage5, 0, 5 * (N + 1) * sizeof(double), S.stream);
    cudaMemsetAsync(s->stage9, 0, 9 * (N + 1) * sizeof(double), S.stream);
    // geometry AoS -> SoA on the host (one-off)
    HostDoubles h, hd, hf, hfd;
    lattice_geometry_soa(g, s->map, h, hd, hf, hfd);
    if ((st = upload(s, m9, host_ptr(h), 9 * N * 8)) || (st = upload(s, det, host_ptr(hd), N * 8))
        || (st = upload(s, fm, host_ptr(hf), 9 * N * 8)) || (st = upload(s, fdet, host_ptr(hfd), 3 * N * 8)))
        return st;
    S.m9 = m9;
    S.det = det;
    S.fm = fm;
    S.fdet = fdet;
    bool identity = true;
    for (size_t n = 0; n < N && identity; ++n) identity = s->map.row_of[n] == (int32_t)n + 1;
    if (!identity) {
        int *row_of;
        if ((st = dalloc_t(s, N, &row_of)) || (st = upload(s, row_of, s->map.row_of.data(), N * sizeof(int))))
            return st;
        S.row_of = row_of;
    }
    if (s->map.ghosted()) {
        unsigned char *loc8;
        if ((st = dalloc_t(s, N, &loc8)) || (st = upload(s, loc8, s->map.loc.data(), N))) return st;
        S.loc8 = loc8;
        {   // the nodes that take a non-central loc-code branch (LatView::locflag)
            std::vector<unsigned char> flag(N, 0);
            const LatticeMap &m = s->map;
            for (int k = 0; k < m.nk; ++k)
                for (int j = 0; j < m.nj; ++j)
                    for (int i = 0; i < m.ni; ++i) {
                        const int c[3] = {i, j, k};
                        unsigned char f = 0;
                        for (int d = 0; d < 3; ++d) {
                            if (!((m.locdirs >> d) & 1)) continue;
                            const int ext = m.extent(d);
                            const bool per = (m.per >> d) & 1;
                            int L7[7];
                            for (int o = 0; o < 7; ++o) {
                                int x = c[d] + o - 3;
                                x = per ? (x + ext) % ext : (x < 0 ? 0 : (x >= ext ? ext - 1 : x));
                                int cc[3] = {i, j, k};
                                cc[d] = x;
                                L7[o] = m.loc[(size_t)cc[0] + (size_t)m.ni * (cc[1] + (size_t)m.nj * cc[2])];
                            }
                            if (visc_branch(L7) != 5 || weno_visc_branch(L7) != 5) f |= (unsigned char)(1u << d);
                        }
                        flag[(size_t)i + (size_t)m.ni * (j + (size_t)m.nj * k)] = f;
                    }
            unsigned char *locflag;
            if ((st = dalloc_t(s, N, &locflag)) || (st = upload(s, locflag, flag.data(), N))) return st;
            S.locflag = locflag;
        }
    }
    if (s->mixed) {
        if (s->form == CFD_PREC_SPLIT) {
            split_geometry(S);
            s->ctx->launches += kSplitGeometryLaunches;
        } else {
            mixed_geometry(S);
            s->ctx->launches += kMixedGeometryLaunches;
        }
        if (cudaStreamCreateWithFlags(&S.side, cudaStreamNonBlocking) != cudaSuccess
            || cudaEventCreateWithFlags(&S.fork, cudaEventDisableTiming) != cudaSuccess
            || cudaEventCreateWithFlags(&S.join, cudaEventDisableTiming) != cudaSuccess)
            return cuda_fail(s->ctx, cudaGetLastError(), "solver side stream");
        for (int f = 0; f < 2; ++f)
            if (cudaStreamCreateWithFlags(&S.face_side[f], cudaStreamNonBlocking) != cudaSuccess
                || cudaEventCreateWithFlags(&S.face_join[f], cudaEventDisableTiming) != cudaSuccess)
                return cuda_fail(s->ctx, cudaGetLastError(), "solver face streams");
    }
    cudaError_t e = cudaStreamSynchronize(S.stream);   // host vectors go out of scope
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "solver create sync");
    if (s->mixed) return tune_face_tiles(s);
    s->fp64_tune = 1;   // on the second stage's real inputs (tune_fp64_faces)
    return CFD_OK;
}

// Face-tile widths of the mixed and split face passes, timed once per form
// and lattice shape in this process (candidates: 32, 64, 128 faces along i;
// 8, 16, 32 along j and k, which share one width).  The passes run on a
// uniform state in the FP32 face inputs, which the first stage overwrites;
// every width evaluates the same arithmetic, so the choice changes no
// result.
std::mutex g_tile_mutex;
std::map<std::array<int, 7>, std::pair<int, int>> g_tile_cache;

cfd_status_t tune_face_tiles(cfd_solver *s)
{
    StructuredLaunch &S = s->S;
    const std::array<int, 7> key = {s->form, S.ni, S.nj, S.nk, S.per, S.loc8 ? 1 : 0, s->ctx->device};
    {
        std::lock_guard<std::mutex> lock(g_tile_mutex);
        auto it = g_tile_cache.find(key);
        if (it != g_tile_cache.end()) {
            S.tile_i = it->second.first;
            S.tile_jk = it->second.second;
            return CFD_OK;
        }
    }
    cudaStream_t st = s->ctx->stream;
    auto pass = [&](int d, int tile) {
        if (s->form == CFD_PREC_SPLIT) split_face_pass(S, d, tile, st);
        else mixed_face_pass(S, d, tile, st);
    };
    reduced_uniform_inputs(S, st);
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess) {
        const cudaError_t ce = cudaGetLastError();
        if (t0) cudaEventDestroy(t0);
        return cuda_fail(s->ctx, ce, "face-tile tuner events");
    }
    auto time_ms = [&](std::initializer_list<int> dirs, int tile) {
        for (int d : dirs) pass(d, tile);   // warm-up
        cudaEventRecord(t0, st);
        for (int r = 0; r < 3; ++r)
            for (int d : dirs) pass(d, tile);
        cudaEventRecord(t1, st);
        float ms = 1e30f;
        if (cudaEventSynchronize(t1) == cudaSuccess) cudaEventElapsedTime(&ms, t0, t1);
        s->ctx->launches += 4 * dirs.size();
        return ms;
    };
    float best_i = 1e30f, best_jk = 1e30f;
    int ti = S.tile_i, tjk = S.tile_jk;
    for (int c : {32, 64, 128}) {
        const float ms = time_ms({0}, c);
        if (ms < best_i) best_i = ms, ti = c;
    }
    for (int c : {8, 16, 32}) {
        const float ms = time_ms({1, 2}, c);
        if (ms < best_jk) best_jk = ms, tjk = c;
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "face-tile tuner");
    S.tile_i = ti;
    S.tile_jk = tjk;
    std::lock_guard<std::mutex> lock(g_tile_mutex);
    g_tile_cache[key] = {ti, tjk};
    return CFD_OK;
}

// Register budgets of the FP64 face passes (2, 3 or 4 blocks of 128 per
// SM, per direction), timed once per lattice shape in this process, at the
// solver's second stage: that stage's prep runs first (it runs again in the
// stage itself, writing the same values), then each budget's face pass on
// the real inputs (their output, the face fluxes, is rewritten by the
// stage).  A uniform state does not do: the exact divisions take data-
// dependent paths, and budgets timed on one mispredicted the NACA0012 and
// shocked-slab lattices by 10 %.  Nor does the first stage of an impulsive
// start, whose state is still exactly uniform (zeros and ones everywhere)
// where every later stage carries rounding-level differences.  The best
// budget depends on the shape; every budget gives the same bits.
std::mutex g_fp64_face_mutex;
std::map<std::array<int, 6>, std::array<int, 3>> g_fp64_face_cache;

std::array<int, 6> fp64_face_key(const cfd_solver *s)
{
    const StructuredLaunch &S = s->S;
    return {S.ni, S.nj, S.nk, S.per, S.loc8 ? 1 : 0, s->ctx->device};
}

cfd_status_t tune_fp64_faces(cfd_solver *s, int j)
{
    s->fp64_tune = -1;
    StructuredLaunch &S = s->S;
    const std::array<int, 6> key = fp64_face_key(s);
    {
        std::lock_guard<std::mutex> lock(g_fp64_face_mutex);
        auto it = g_fp64_face_cache.find(key);
        if (it != g_fp64_face_cache.end()) {
            for (int d = 0; d < 3; ++d) S.face_mb[d] = it->second[d];
            return CFD_OK;
        }
    }
    cudaStream_t st = s->ctx->stream;
    fp64_prep_pass(S, j);
    s->ctx->launches += 1;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess) {
        const cudaError_t ce = cudaGetLastError();
        if (t0) cudaEventDestroy(t0);
        return cuda_fail(s->ctx, ce, "FP64 face tuner events");
    }
    std::array<int, 3> pick = {S.face_mb[0], S.face_mb[1], S.face_mb[2]};
    for (int d = 0; d < 3; ++d) {
        float best = 1e30f;
        for (int mb : {2, 3, 4}) {
            fp64_face_pass(S, d, mb, st);   // warm-up
            cudaEventRecord(t0, st);
            for (int r = 0; r < 2; ++r) fp64_face_pass(S, d, mb, st);
            cudaEventRecord(t1, st);
            float ms = 1e30f;
            if (cudaEventSynchronize(t1) == cudaSuccess) cudaEventElapsedTime(&ms, t0, t1);
            s->ctx->launches += 3;
            if (ms < best) best = ms, pick[d] = mb;
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "FP64 face tuner");
    for (int d = 0; d < 3; ++d) S.face_mb[d] = pick[d];
    std::lock_guard<std::mutex> lock(g_fp64_face_mutex);
    g_fp64_face_cache[key] = pick;
    return CFD_OK;
}

// where stage j's U_Q comes from (mixed form; the FP64 form always preps)
int prep_source(const cfd_solver *s, int j)
{
    if (!s->mixed) return kPrepFromFlow;
    if (s->prep_ready == j) return kPrepNone;
    return s->cur_slot < 0 ? kPrepFromFlow : s->cur_slot;
}

cfd_status_t run_stage(cfd_solver *s, int j, double dt, bool want_L)
{
    cfd_ctx *ctx = s->ctx;
    s->S.stream = ctx->stream;   // the context's stream may have been replaced
    if (s->path == CFD_PATH_STRUCTURED) {
        if (s->fp64_tune == 0) {
            const cfd_status_t st = tune_fp64_faces(s, j);
            if (st != CFD_OK) return st;
        } else if (s->fp64_tune > 0) {
            --s->fp64_tune;
        }
        ctx->launches += structured_stage(s->S, j, dt, want_L ? s->Lsoa : nullptr, nullptr, nullptr, prep_source(s, j));
        if (s->mixed) s->cur_slot = s->prep_ready = j == 2 ? 0 : j + 1;
        if (s->has_bc) {
            if (s->form == CFD_PREC_SPLIT)
                bc_apply_split(ctx->stream, s->bc, make_view(s->S, dt, nullptr), s->cur_slot, s->P.mach);
            else if (s->mixed)
                bc_apply_mixed(ctx->stream, s->bc, make_view(s->S, dt, nullptr), s->cur_slot, s->P.mach);
            else
                bc_apply_soa(ctx->stream, s->bc, s->S.prim9, (int)((long long)s->ni * s->nj * s->nk), s->P.mach);
            ctx->launches += s->bc.launches();
        }
    } else {
        double *Uj = s->U[j];
        const int nu = launch_uq(ctx->stream, Uj, s->Q, s->grid, s->det, s->flow, s->roe, s->g_node + 1, s->n_rows,
                                 ctx->d_flags, s->face, s->n_rows);
        launch_viscous(ctx->stream, s->P, Uj, s->F, s->E, s->G, s->Fv, s->Ev, s->Gv, s->grid, s->metric, s->det,
                       s->flow, s->g_node + 1, s->n_rows, ctx->d_flags);
        launch_weno(ctx->stream, s->P, j, s->P.mach, dt, s->deter, s->det, s->U[0], s->U[1], s->U[2], s->grid, s->Q,
                    s->metric, s->roe, s->Fv, s->Ev, s->Gv, s->F, s->E, s->G, s->flow, s->sd_node + 1, s->n_rows,
                    ctx->d_flags, want_L ? s->L : nullptr, s->face, s->n_rows, next_face_gen(s->face_gen));
        ctx->launches += nu + 1 + weno_launches(s->face, s->n_rows, s->sd_node + 1);
        if (s->has_bc) {
            bc_apply_aos(ctx->stream, s->bc, s->flow, s->P.mach);
            ctx->launches += s->bc.launches();
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "stage launch");
    return CFD_OK;
}

}  // namespace

extern "C" {

cfd_status_t cfd_solver_create(cfd_ctx_t *ctx, const cfd_geometry_t *geom, const cfd_params_t *params,
                               int32_t force_path, cfd_solver_t **out)
{
    if (!ctx || !geom || !out) return CFD_EINVAL;
    *out = nullptr;
    if (!geom->grid || !geom->det || !geom->deter || !geom->metric)
        return fail(ctx, CFD_EINVAL, "cfd_solver_create: null geometry array");
    if (geom->g_node < 1 || geom->sd_node < 1 || geom->sd_node > geom->g_node)
        return fail(ctx, CFD_EINVAL, "cfd_solver_create: need 1 <= sd_node <= g_node");
    if (force_path < -1 || force_path > 1) return fail(ctx, CFD_EINVAL, "cfd_solver_create: bad force_path");
    const int32_t n_rows = geom->g_node + 1;
    for (int32_t r = 0; r < n_rows; ++r)
        for (int slot = 0; slot < 6; ++slot) {
            const int v = nb_of(geom->grid[r], slot);
            if (v < 0 || v >= n_rows)
                return fail(ctx, CFD_EINVAL, "cfd_solver_create: neighbour index outside [0, g_node]");
        }
    cfd_status_t st = use_device(ctx);
    if (st != CFD_OK) return st;
    cfd_solver *s = new cfd_solver();
    s->ctx = ctx;
    cfd_params_default(&s->prm);
    if (params) s->prm = *params;
    s->P = make_phys(&s->prm);
    if (s->prm.precision < CFD_PREC_FP64 || s->prm.precision > CFD_PREC_SPLIT) {
        delete s;
        return fail(ctx, CFD_EINVAL, "cfd_solver_create: unknown precision");
    }
    s->form = s->prm.precision;
    s->mixed = s->form != CFD_PREC_FP64;
    s->g_node = geom->g_node;
    s->sd_node = geom->sd_node;
    s->n_rows = n_rows;
    bool lattice = force_path != CFD_PATH_GATHER && map_lattice(geom, s->map) && faces_single_valued(geom, s->map);
    if (force_path == CFD_PATH_STRUCTURED && !lattice) {
        delete s;
        return fail(ctx, CFD_EINVAL, "cfd_solver_create: table is not a lattice with single-valued faces");
    }
    if (lattice && (long long)s->map.ni * s->map.nj * s->map.nk > kLatticeMaxNodes) {
        // beyond the face-based kernels' 32-bit addressing: the gather path
        // (64-bit row offsets) takes the FP64 form
        if (force_path == CFD_PATH_STRUCTURED || s->mixed) {
            delete s;
            return fail(ctx, CFD_EUNSUPPORTED, "cfd_solver_create: lattice larger than 143,165,576 nodes");
        }
        lattice = false;
    }
    s->path = lattice ? CFD_PATH_STRUCTURED : CFD_PATH_GATHER;
    if (s->mixed && s->path != CFD_PATH_STRUCTURED) {
        delete s;
        return fail(ctx, CFD_EUNSUPPORTED, "cfd_solver_create: the mixed and split forms need the structured path");
    }
    s->ni = lattice ? s->map.ni : 0;
    s->nj = lattice ? s->map.nj : 0;
    s->nk = lattice ? s->map.nk : 0;
    st = s->path == CFD_PATH_STRUCTURED ? create_structured(s, geom) : create_gather(s, geom);
    if (st != CFD_OK) {
        cfd_solver_destroy(s);
        return st;
    }
    *out = s;
    return CFD_OK;
}

cfd_status_t cfd_solver_destroy(cfd_solver_t *s)
{
    if (!s) return CFD_EINVAL;
    use_device(s->ctx);
    cudaStreamSynchronize(s->ctx->stream);
    if (s->S.side) {
        cudaStreamSynchronize(s->S.side);
        cudaStreamDestroy(s->S.side);
    }
    if (s->S.fork) cudaEventDestroy(s->S.fork);
    if (s->S.join) cudaEventDestroy(s->S.join);
    for (int f = 0; f < 2; ++f) {
        if (s->S.face_side[f]) {
            cudaStreamSynchronize(s->S.face_side[f]);
            cudaStreamDestroy(s->S.face_side[f]);
        }
        if (s->S.face_join[f]) cudaEventDestroy(s->S.face_join[f]);
    }
    bc_free(s->bc);
    for (void *p : s->allocs) cudaFree(p);
    delete s;
    return CFD_OK;
}

cfd_status_t cfd_solver_set_boundary(cfd_solver_t *s, const cfd_bc_t *bc)
{
    if (!s) return CFD_EINVAL;
    cfd_status_t st = use_device(s->ctx);
    if (st != CFD_OK) return st;
    cudaStreamSynchronize(s->ctx->stream);
    bc_free(s->bc);
    s->has_bc = false;
    if (!bc) return CFD_OK;
    if (bc->n_rows != s->n_rows) return fail(s->ctx, CFD_EINVAL, "cfd_solver_set_boundary: table size differs");
    BcPlan plan;
    if (s->path == CFD_PATH_STRUCTURED) {
        if (!bc_remap(bc->plan, s->map.n_of_row, plan))
            return fail(s->ctx, CFD_EUNSUPPORTED, "cfd_solver_set_boundary: a boundary row is not a lattice node");
    } else {
        plan = bc->plan;
    }
    cudaError_t e = bc_upload(plan, s->bc, s->ctx->stream);
    if (e != cudaSuccess) {
        bc_free(s->bc);
        return cuda_fail(s->ctx, e, "cfd_solver_set_boundary upload");
    }
    s->has_bc = true;
    return CFD_OK;
}

cfd_status_t cfd_solver_info(const cfd_solver_t *s, cfd_solver_info_t *info)
{
    if (!s || !info) return CFD_EINVAL;
    std::memset(info, 0, sizeof *info);
    info->path = s->path;
    info->ni = s->ni;
    info->nj = s->nj;
    info->nk = s->nk;
    info->precision = s->form;
    info->device_bytes = s->bytes;
    info->face_tile_i = s->mixed && s->path == CFD_PATH_STRUCTURED ? s->S.tile_i : 0;
    info->face_tile_jk = s->mixed && s->path == CFD_PATH_STRUCTURED ? s->S.tile_jk : 0;
    if (!s->mixed && s->path == CFD_PATH_STRUCTURED)
        for (int d = 0; d < 3; ++d) info->face_blocks[d] = s->S.face_mb[d];
    return CFD_OK;
}

cfd_status_t cfd_solver_set_face_tiles(cfd_solver_t *s, int32_t tile_i, int32_t tile_jk)
{
    if (!s) return CFD_EINVAL;
    if (!(s->mixed && s->path == CFD_PATH_STRUCTURED)) return fail(s->ctx, CFD_EUNSUPPORTED, "face tiles: mixed or split lattice only");
    if ((tile_i != 0 && tile_i != 32 && tile_i != 64 && tile_i != 128)
        || (tile_jk != 0 && tile_jk != 8 && tile_jk != 16 && tile_jk != 32))
        return fail(s->ctx, CFD_EINVAL, "face tiles: tile_i in {32, 64, 128}, tile_jk in {8, 16, 32}");
    cfd_status_t st = use_device(s->ctx);
    if (st != CFD_OK) return st;
    cudaStreamSynchronize(s->ctx->stream);
    if (tile_i) s->S.tile_i = tile_i;
    if (tile_jk) s->S.tile_jk = tile_jk;
    return CFD_OK;
}

cfd_status_t cfd_solver_set_face_blocks(cfd_solver_t *s, int32_t blocks_i, int32_t blocks_j, int32_t blocks_k)
{
    if (!s) return CFD_EINVAL;
    if (s->mixed || s->path != CFD_PATH_STRUCTURED)
        return fail(s->ctx, CFD_EUNSUPPORTED, "face blocks: FP64 lattice only");
    const int32_t b[3] = {blocks_i, blocks_j, blocks_k};
    for (int d = 0; d < 3; ++d)
        if (b[d] != 0 && (b[d] < 2 || b[d] > 4)) return fail(s->ctx, CFD_EINVAL, "face blocks: 2, 3 or 4 (0 keeps)");
    cfd_status_t st = use_device(s->ctx);
    if (st != CFD_OK) return st;
    cudaStreamSynchronize(s->ctx->stream);
    for (int d = 0; d < 3; ++d)
        if (b[d]) s->S.face_mb[d] = b[d];
    s->fp64_tune = -1;   // the caller's choice stands
    return CFD_OK;
}

cfd_status_t cfd_solver_set_flow(cfd_solver_t *s, const cfd_flow_t *flow_host)
{
    if (!s || !flow_host) return CFD_EINVAL;
    cfd_status_t st = use_device(s->ctx);
    if (st != CFD_OK) return st;
    const size_t R = (size_t)s->n_rows;
    if (s->path == CFD_PATH_GATHER) {
        st = upload(s, s->flow, flow_host, R * sizeof(cfd_flow_t));
    } else {
        const long long N = (long long)s->ni * s->nj * s->nk;
        s->S.stream = s->ctx->stream;
        s->prep_ready = -1;
        s->cur_slot = -1;
        st = upload(s, s->stage9, flow_host, R * sizeof(cfd_flow_t));
        if (st == CFD_OK) aos_to_soa(s->ctx->stream, s->stage9, 9, 9, N, s->S.prim9, s->S.row_of);
    }
    if (st != CFD_OK) return st;
    return drain(s->ctx);
}

cfd_status_t cfd_solver_get_flow(cfd_solver_t *s, cfd_flow_t *flow_host)
{
    if (!s || !flow_host) return CFD_EINVAL;
    cfd_status_t st = use_device(s->ctx);
    if (st != CFD_OK) return st;
    const size_t R = (size_t)s->n_rows;
    const double *src = s->flow;
    if (s->path == CFD_PATH_STRUCTURED) {
        s->S.stream = s->ctx->stream;
        if (s->mixed && s->cur_slot >= 0) {   // FP64 FLOW of the current state
            if (s->form == CFD_PREC_SPLIT)
                split_flow_out(make_view(s->S, 0.0, nullptr), s->cur_slot, s->S.stream);
            else
                mixed_flow_out(make_view(s->S, 0.0, nullptr), s->cur_slot, s->S.stream);
            s->ctx->launches += 1;
        }
        soa_to_aos(s->ctx->stream, s->S.prim9, 9, 9, (long long)s->ni * s->nj * s->nk, s->stage9, s->S.row_of);
        src = s->stage9;
    }
    cudaError_t e = cudaMemcpyAsync(flow_host, src, R * sizeof(cfd_flow_t), cudaMemcpyDeviceToHost, s->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "cudaMemcpyAsync D2H (flow)");
    return drain(s->ctx);
}

cfd_status_t cfd_solver_get_u0(cfd_solver_t *s, cfd_column_t *u0_host)
{
    if (!s || !u0_host) return CFD_EINVAL;
    cfd_status_t st = use_device(s->ctx);
    if (st != CFD_OK) return st;
    const size_t R = (size_t)s->n_rows;
    const double *src = s->U[0];
    if (s->path == CFD_PATH_STRUCTURED) {
        if (s->form == CFD_PREC_MIXED)
            mixed_u_out(make_view(s->S, 0.0, nullptr), 0, s->stage5, s->ctx->stream);
        else
            soa_to_aos(s->ctx->stream, s->S.U[0], 5, 5, (long long)s->ni * s->nj * s->nk, s->stage5, s->S.row_of);
        src = s->stage5;
    }
    cudaError_t e = cudaMemcpyAsync(u0_host, src, R * sizeof(cfd_column_t), cudaMemcpyDeviceToHost, s->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "cudaMemcpyAsync D2H (U0)");
    return drain(s->ctx);
}

cfd_status_t cfd_solver_step(cfd_solver_t *s, double del_t, int32_t nsteps)
{
    if (!s || nsteps < 0 || !std::isfinite(del_t)) return CFD_EINVAL;
    cfd_status_t st = use_device(s->ctx);
    if (st != CFD_OK) return st;
    for (int n = 0; n < nsteps; ++n)
        for (int j = 0; j < 3; ++j)
            if ((st = run_stage(s, j, del_t, false)) != CFD_OK) return st;
    if (s->ctx->async) return CFD_OK;
    return drain(s->ctx);
}

cfd_status_t cfd_solver_stage(cfd_solver_t *s, int32_t j, double del_t, cfd_column_t *L_host)
{
    if (!s || j < 0 || j > 2) return CFD_EINVAL;
    cfd_status_t st = use_device(s->ctx);
    if (st != CFD_OK) return st;
    if ((st = run_stage(s, j, del_t, L_host != nullptr)) != CFD_OK) return st;
    if (L_host) {
        const size_t R = (size_t)s->n_rows;
        const double *src = s->L;
        if (s->path == CFD_PATH_STRUCTURED) {
            soa_to_aos(s->ctx->stream, s->Lsoa, 5, 5, (long long)s->ni * s->nj * s->nk, s->stage5, s->S.row_of);
            src = s->stage5;
        }
        cudaError_t e = cudaMemcpyAsync(L_host, src, R * sizeof(cfd_column_t), cudaMemcpyDeviceToHost, s->ctx->stream);
        if (e != cudaSuccess) return cuda_fail(s->ctx, e, "cudaMemcpyAsync D2H (L)");
    }
    return drain(s->ctx);
}

cfd_status_t cfd_solver_profile_stage(cfd_solver_t *s, int32_t j, double del_t, cfd_kernel_time_t *out,
                                      int32_t max_out, int32_t *n_out)
{
    if (!s || !out || !n_out || j < 0 || j > 2 || max_out <= 0) return CFD_EINVAL;
    cfd_status_t st = use_device(s->ctx);
    if (st != CFD_OK) return st;
    cudaStream_t stream = s->ctx->stream;
    s->S.stream = stream;
    std::vector<cudaEvent_t> ev(kMaxStageLaunches + 2);
    for (auto &e : ev) cudaEventCreate(&e);
    const char *snames[kMaxStageLaunches + 1] = {};
    int nk = 3;
    if (s->path == CFD_PATH_STRUCTURED && s->fp64_tune >= 0 && (st = tune_fp64_faces(s, j)) != CFD_OK) {
        for (auto &e : ev) cudaEventDestroy(e);
        return st;
    }
    if (s->path == CFD_PATH_STRUCTURED) {
        nk = structured_stage(s->S, j, del_t, nullptr, ev.data(), snames, prep_source(s, j));
        if (s->mixed) s->cur_slot = s->prep_ready = j == 2 ? 0 : j + 1;
    } else {
        cudaEventRecord(ev[0], stream);
        double *Uj = s->U[j];
        const int nu = launch_uq(stream, Uj, s->Q, s->grid, s->det, s->flow, s->roe, s->g_node + 1, s->n_rows,
                                 s->ctx->d_flags, s->face, s->n_rows);
        cudaEventRecord(ev[1], stream);
        launch_viscous(stream, s->P, Uj, s->F, s->E, s->G, s->Fv, s->Ev, s->Gv, s->grid, s->metric, s->det, s->flow,
                       s->g_node + 1, s->n_rows, s->ctx->d_flags);
        cudaEventRecord(ev[2], stream);
        launch_weno(stream, s->P, j, s->P.mach, del_t, s->deter, s->det, s->U[0], s->U[1], s->U[2], s->grid, s->Q,
                    s->metric, s->roe, s->Fv, s->Ev, s->Gv, s->F, s->E, s->G, s->flow, s->sd_node + 1, s->n_rows,
                    s->ctx->d_flags, nullptr, s->face, s->n_rows, next_face_gen(s->face_gen));
        cudaEventRecord(ev[3], stream);
        snames[0] = "uq";
        snames[1] = "viscous";
        snames[2] = "weno";
        // uq: per-row pass + Roe kernel; weno: plus faces + update
        s->ctx->launches += (nu - 1) + weno_launches(s->face, s->n_rows, s->sd_node + 1) - 1;
    }
    s->ctx->launches += nk;
    if (s->has_bc) {   // the boundary routine as one timed entry
        if (s->path != CFD_PATH_STRUCTURED)
            bc_apply_aos(stream, s->bc, s->flow, s->P.mach);
        else if (s->form == CFD_PREC_SPLIT)
            bc_apply_split(stream, s->bc, make_view(s->S, del_t, nullptr), s->cur_slot, s->P.mach);
        else if (s->mixed)
            bc_apply_mixed(stream, s->bc, make_view(s->S, del_t, nullptr), s->cur_slot, s->P.mach);
        else
            bc_apply_soa(stream, s->bc, s->S.prim9, (int)((long long)s->ni * s->nj * s->nk), s->P.mach);
        s->ctx->launches += s->bc.launches();
        cudaEventRecord(ev[nk + 1], stream);
        snames[nk] = "boundary";
        ++nk;
    }
    cudaError_t e = cudaEventSynchronize(ev[nk]);
    if (e == cudaSuccess) {
        const int n = nk < max_out ? nk : max_out;
        for (int i = 0; i < n; ++i) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
            const char *nm = snames[i] ? snames[i] : "?";
            std::strncpy(out[i].name, nm, sizeof out[i].name - 1);
            out[i].name[sizeof out[i].name - 1] = 0;
            out[i].ms = ms;
        }
        *n_out = n;
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "profile stage");
    return drain(s->ctx);
}

}  // extern "C"

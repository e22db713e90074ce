// batch.cu -- many independent lattices advanced together: one persistent,
// cooperative launch per RK stage over a tile table of all instances
// (batch_kernel.cuh), one RK step captured as a CUDA graph, and a tuner that
// times tile sizes on the live batch (state saved and restored around the
// trials).  Instances are admitted against a device-memory budget, keep
// their state resident, and can be added and removed between steps; this is
// the engine under the serving loop.
#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "batch_kernel.cuh"
#include "batch_ops.h"
#include "internal.h"
#include "lattice_host.h"
#include "structured.h"

namespace {

using namespace cfd;

constexpr int kMaxSlots = 4096;

struct BatchInst {
    bool active = false;
    bool held = false;          // resident, but not advanced by cfd_batch_step
    bool in_table = false;      // in the tile table of the last rebuild
    bool stepped = false;       // advanced by a step queued since the last finish()
    bool interrupted = false;   // a barrier timeout cut one of its steps short
    int32_t g_node = 0;
    int ni = 0, nj = 0, nk = 0, N = 0;
    cfd_params_t prm{};
    double dt = 0.0;
    std::vector<void *> allocs;
    uint64_t bytes = 0;
    LatView view{};
    double *stage9 = nullptr;   // AoS FLOW staging rows 0..N
    double *stage5 = nullptr;   // AoS column staging rows 0..N
};

}  // namespace

struct cfd_batch {
    cfd_ctx *ctx = nullptr;
    int precision = CFD_PREC_FP64;
    uint64_t capacity = 0, used = 0;
    std::vector<BatchInst> slots;
    LatView *d_views = nullptr;
    size_t views_cap = 0;
    BatchTile *d_tiles = nullptr;
    size_t tiles_cap = 0;
    int ntiles = 0;
    // tiled form (reduced-precision batches): phase A items (viscous ranges
    // and shared-memory face tiles); d_tiles then holds phase B's 1-D tiles
    bool face_tiles = false;
    BatchItem *d_items = nullptr;
    size_t items_cap = 0;
    int nitems = 0;
    int n_views = 0;
    unsigned *d_words = nullptr;          // [0..1] barrier, [2] batch flags, [3] phase-A work counter, [4..] per-slot flags
    int threads = 128;
    int blocks_override = 0;
    long long wait_limit_ns = -1;         // barrier deadline (< 0: 5 s + 50 ns per node)
    int blocks = 0;
    bool dirty = true;
    bool use_graph = true;
    bool graph_ok = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    uint64_t total_nodes = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};   // ends of the last two cfd_batch_step_async calls
    bool ev_live[2] = {false, false};
    int ev_next = 0;
};

namespace {

unsigned *bar_words(cfd_batch *b) { return b->d_words; }
unsigned *batch_flags(cfd_batch *b) { return b->d_words + 2; }
unsigned *slot_flags(cfd_batch *b, int slot) { return b->d_words + 4 + slot; }

uint64_t instance_bytes(int precision, int64_t N)
{
    const uint64_t doubles = (22 + 9 + 15) * (uint64_t)N + 14 * (uint64_t)(N + 1);
    // mixed: FP32 face/node geometry (12 + 10 + 2), prim32 (9), stage intermediates (55)
    if (precision == CFD_PREC_MIXED) return doubles * 8 + (12 + 11 + 2 + 9 + 55) * (uint64_t)N * 4;
    // split: FP32 face metrics (9), node geometry (11), prim32 (9), Q32/R32/FEG32/V32 (40) and the hi/lo
    // state copy (10); FP64 1/det and Fh (16)
    if (precision == CFD_PREC_SPLIT) return (doubles + 16 * (uint64_t)N) * 8 + (9 + 11 + 9 + 40 + 10) * (uint64_t)N * 4;
    return (doubles + 52 * (uint64_t)N) * 8;
}

void drop_graph(cfd_batch *b)
{
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->gexec = nullptr;
    b->graph = nullptr;
    b->graph_ok = false;
}

void free_instance(BatchInst &I)
{
    for (void *p : I.allocs) cudaFree(p);
    I.allocs.clear();
    I = BatchInst();
}

template <class T>
cfd_status_t ialloc(cfd_batch *b, BatchInst &I, size_t count, T **p)
{
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cudaMalloc (batch instance)");
    I.allocs.push_back(*p);
    I.bytes += count * sizeof(T);
    return CFD_OK;
}

// The face tiles of direction D of lattice view v (FaceTile<D, tile>::grid).
template <int D>
void face_tile_items(const LatView &g, int v, std::vector<BatchItem> &out)
{
    using T = FaceTile<D, D == 0 ? kBatchTileI : kBatchTileJK>;
    const dim3 gr = T::grid(g);
    for (unsigned z = 0; z < gr.z; ++z)
        for (unsigned y = 0; y < gr.y; ++y)
            for (unsigned x = 0; x < gr.x; ++x)
                out.push_back(BatchItem{v, 1 + D, (int)x * T::kTile, (int)y * T::kWide, (int)z, 0});
}

// Phase A items of the tiled form in the order the blocks take them (from
// the shared counter): kind-major as the 1-D form (CFD_BATCH_KIND_MAJOR),
// else position w has kind (w % G + w / G) mod 4 while that kind has items
// left (else the next kind that has), so that the blocks running at one
// time work on every kind of the same region.
std::vector<BatchItem> order_items(std::vector<BatchItem> q[4], int G)
{
    size_t total = 0, head[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; ++k) total += q[k].size();
    std::vector<BatchItem> out;
    out.reserve(total);
    if (CFD_BATCH_KIND_MAJOR) {   // as the 1-D form: i, j, k faces, then the viscous ranges
        for (int k : {1, 2, 3, 0}) out.insert(out.end(), q[k].begin(), q[k].end());
        return out;
    }
    for (size_t w = 0; w < total; ++w) {
        const int k0 = (int)(((w % G) + (w / G)) & 3);
        for (int t = 0; t < 4; ++t) {
            const int k = (k0 + t) & 3;
            if (head[k] < q[k].size()) {
                out.push_back(q[k][head[k]++]);
                break;
            }
        }
    }
    return out;
}

cfd_status_t rebuild(cfd_batch *b)
{
    std::vector<LatView> views;
    std::vector<BatchTile> tiles;
    std::vector<BatchItem> kinds[4];
    const bool tiled = b->face_tiles && b->precision != CFD_PREC_FP64;
    const int T = tiled ? kFaceThreads : b->threads;
    uint64_t nodes = 0;
    for (size_t s = 0; s < b->slots.size(); ++s) {
        BatchInst &I = b->slots[s];
        I.in_table = I.active && !I.held;
        if (!I.in_table) continue;
        const int v = (int)views.size();
        views.push_back(I.view);
        for (int n0 = 0; n0 < I.N; n0 += T) tiles.push_back(BatchTile{v, n0, std::min(T, I.N - n0), 0});
        if (tiled) {
            for (int n0 = 0; n0 < I.N; n0 += T) kinds[0].push_back(BatchItem{v, 0, n0, std::min(T, I.N - n0), 0, 0});
            face_tile_items<0>(I.view, v, kinds[1]);
            face_tile_items<1>(I.view, v, kinds[2]);
            face_tile_items<2>(I.view, v, kinds[3]);
        }
        nodes += (uint64_t)I.N;
    }
    cudaStream_t st = b->ctx->stream;
    cudaError_t e = cudaSuccess;
    if (views.size() > b->views_cap) {
        if (b->d_views) cudaFree(b->d_views);
        b->views_cap = std::max<size_t>(views.size(), 2 * b->views_cap);
        e = cudaMalloc(&b->d_views, b->views_cap * sizeof(LatView));
        if (e != cudaSuccess) return cuda_fail(b->ctx, e, "batch view table");
    }
    if (tiles.size() > b->tiles_cap) {
        if (b->d_tiles) cudaFree(b->d_tiles);
        b->tiles_cap = std::max<size_t>(tiles.size(), 2 * b->tiles_cap);
        e = cudaMalloc(&b->d_tiles, b->tiles_cap * sizeof(BatchTile));
        if (e != cudaSuccess) return cuda_fail(b->ctx, e, "batch tile table");
    }
    if (!views.empty()) e = cudaMemcpyAsync(b->d_views, views.data(), views.size() * sizeof(LatView), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !tiles.empty())
        e = cudaMemcpyAsync(b->d_tiles, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "batch table upload");
    b->ntiles = (int)tiles.size();
    b->n_views = (int)views.size();
    b->total_nodes = nodes;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int occ = b->precision == CFD_PREC_MIXED   ? batch_occupancy_mixed(T, tiled)
                    : b->precision == CFD_PREC_SPLIT ? batch_occupancy_split(T, tiled)
                                                     : batch_occupancy_fp64(T);
    if (occ <= 0) return fail(b->ctx, CFD_EUNSUPPORTED, "batch: stage kernel does not fit at this tile size");
    int blocks = occ * sms;
    if (b->blocks_override > 0) blocks = std::min(blocks, b->blocks_override);
    size_t n_a = 4 * (size_t)std::max(b->ntiles, 1);   // phase A items
    if (tiled) n_a = std::max<size_t>(1, kinds[0].size() + kinds[1].size() + kinds[2].size() + kinds[3].size());
    blocks = std::max(1, (int)std::min<size_t>((size_t)blocks, n_a));
    b->blocks = blocks;
    b->nitems = 0;
    if (tiled) {
        const std::vector<BatchItem> items = order_items(kinds, blocks);
        if (items.size() > b->items_cap) {
            if (b->d_items) cudaFree(b->d_items);
            b->items_cap = std::max<size_t>(items.size(), 2 * b->items_cap);
            e = cudaMalloc(&b->d_items, b->items_cap * sizeof(BatchItem));
            if (e != cudaSuccess) return cuda_fail(b->ctx, e, "batch item table");
        }
        if (!items.empty())
            e = cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(b->ctx, e, "batch item table upload");
        b->nitems = (int)items.size();
    }
    drop_graph(b);
    b->dirty = false;
    return CFD_OK;
}

BatchLaunch launch_of(cfd_batch *b)
{
    BatchLaunch L{};
    L.views = b->d_views;
    L.tiles = b->d_tiles;
    L.ntiles = b->ntiles;
    L.threads = b->threads;
    L.blocks = b->blocks;
    L.tiled = b->nitems > 0 ? 1 : 0;
    L.items = b->d_items;
    L.nitems = b->nitems;
    L.bar = bar_words(b);
    L.gflags = batch_flags(b);
    // generous deadline for the barrier: 5 s + 50 ns per node of the batch
    L.limit_ns = b->wait_limit_ns >= 0 ? (unsigned long long)b->wait_limit_ns
                                       : 5000000000ULL + 50ULL * b->total_nodes;
    L.stream = b->ctx->stream;
    return L;
}

cudaError_t launch_step(cfd_batch *b)
{
    const BatchLaunch L = launch_of(b);
    for (int j = 0; j < 3; ++j) {
        cudaError_t e = b->precision == CFD_PREC_MIXED   ? batch_stage_mixed(L, j)
                        : b->precision == CFD_PREC_SPLIT ? batch_stage_split(L, j)
                                                         : batch_stage_fp64(L, j);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void try_capture(cfd_batch *b)
{
    cudaStream_t st = b->ctx->stream;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        b->use_graph = false;
        return;
    }
    cudaError_t le = launch_step(b);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (le != cudaSuccess || ce != cudaSuccess || !g) {
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        b->use_graph = false;
        return;
    }
    cudaGraphExec_t ge = nullptr;
    if (cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(g);
        b->use_graph = false;
        return;
    }
    b->graph = g;
    b->gexec = ge;
    b->graph_ok = true;
}

// Waits for the stream; batch-level flags become the status, per-slot flags
// stay readable through cfd_batch_slot_status.
//
// A barrier timeout: the blocks that gave up skipped phase B of that stage,
// so the state of every instance in the launched tile table is part old,
// part new.  Those instances are marked interrupted (cfd_batch_step refuses
// to advance them until cfd_batch_set_flow restores them or they are
// removed), and the batch words are cleared so that the timeout is reported
// once.  The barrier itself needs no repair: every block counts its arrival
// before it waits, and the last one resets the count and advances the
// generation, so the words are consistent after every launch.
cfd_status_t finish(cfd_batch *b)
{
    std::vector<unsigned> w(4 + b->slots.size());
    cudaError_t e = cudaMemcpyAsync(w.data(), b->d_words, w.size() * sizeof(unsigned), cudaMemcpyDeviceToHost,
                                    b->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "batch finish");
    const bool timeout = (w[2] & CFD_FLAG_TIMEOUT) != 0;
    std::string which;
    for (size_t s = 0; s < b->slots.size(); ++s) {
        BatchInst &I = b->slots[s];
        if (timeout && I.active && I.stepped) {
            I.interrupted = true;
            which += (which.empty() ? "" : ",") + std::to_string(s);
        }
        I.stepped = false;
    }
    if (timeout) {
        e = cudaMemsetAsync(b->d_words, 0, 4 * sizeof(unsigned), b->ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->ctx->stream);
        if (e != cudaSuccess) return cuda_fail(b->ctx, e, "batch finish (clear timeout)");
        return fail(b->ctx, CFD_ETIMEOUT,
                    "batch: grid barrier deadline expired; slots " + which
                        + " interrupted (restore with cfd_batch_set_flow or remove)");
    }
    for (size_t s = 0; s < b->slots.size(); ++s)
        if (b->slots[s].active && (w[4 + s] & CFD_FLAG_NONFINITE))
            return fail(b->ctx, CFD_ENONFINITE, "batch: non-finite state in slot " + std::to_string(s));
    return CFD_OK;
}

// Per-instance arrays that a step changes, for the tuner's save/restore.
std::vector<std::pair<void *, size_t>> mutable_arrays(const BatchInst &I, int precision)
{
    const size_t N = (size_t)I.N;
    std::vector<std::pair<void *, size_t>> v = {{I.view.prim9, 9 * N * 8}, {I.view.U0, 5 * N * 8},
                                                {I.view.U1, 5 * N * 8}, {I.view.U2, 5 * N * 8}};
    if (precision == CFD_PREC_SPLIT) v.push_back({I.view.Whl, 10 * N * 4});
    if (precision == CFD_PREC_MIXED || precision == CFD_PREC_SPLIT) {
        v.push_back({I.view.prim32, 9 * N * 4});
        v.push_back({I.view.Q32, 5 * N * 4});
        v.push_back({I.view.R32, 5 * N * 4});
        v.push_back({I.view.FEG32, 15 * N * 4});
    } else {
        v.push_back({I.view.Q, 5 * N * 8});
        v.push_back({I.view.FEG, 15 * N * 8});
        v.push_back({I.view.sh, 2 * N * 8});
    }
    return v;
}

}  // namespace

extern "C" {

uint64_t cfd_batch_instance_bytes(int32_t precision, int64_t nodes) { return instance_bytes(precision, nodes); }

cfd_status_t cfd_batch_create(cfd_ctx_t *ctx, int32_t precision, uint64_t capacity_bytes, cfd_batch_t **out)
{
    if (!ctx || !out || precision < CFD_PREC_FP64 || precision > CFD_PREC_SPLIT) return CFD_EINVAL;
    *out = nullptr;
    cfd_status_t s = use_device(ctx);
    if (s != CFD_OK) return s;
    cfd_batch *b = new cfd_batch();
    b->ctx = ctx;
    b->precision = precision;
    if (capacity_bytes == 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        capacity_bytes = (uint64_t)(0.85 * (double)fr);
    }
    b->capacity = capacity_bytes;
    cudaError_t e = cudaMalloc(&b->d_words, (4 + kMaxSlots) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(b->d_words, 0, (4 + kMaxSlots) * sizeof(unsigned));
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(ctx, e, "batch create");
    }
    *out = b;
    return CFD_OK;
}

cfd_status_t cfd_batch_destroy(cfd_batch_t *b)
{
    if (!b) return CFD_EINVAL;
    use_device(b->ctx);
    cudaStreamSynchronize(b->ctx->stream);
    drop_graph(b);
    for (cudaEvent_t e : b->ev)
        if (e) cudaEventDestroy(e);
    for (auto &I : b->slots) free_instance(I);
    if (b->d_views) cudaFree(b->d_views);
    if (b->d_tiles) cudaFree(b->d_tiles);
    if (b->d_items) cudaFree(b->d_items);
    if (b->d_words) cudaFree(b->d_words);
    delete b;
    return CFD_OK;
}

}  // extern "C"

// An instance checked and converted on the host (cfd_batch_stage), waiting
// for its device half (cfd_batch_add_staged).
struct cfd_batch_staged {
    cfd_status_t status = CFD_OK;
    std::string error;
    int32_t g_node = 0;
    int ni = 0, nj = 0, nk = 0, N = 0;
    cfd_params_t prm{};
    double dt = 0.0;
    HostDoubles m9, det, fm, fdet, flow;   // lattice geometry (SoA) and FLOW rows 0..N
};

extern "C" {

cfd_status_t cfd_batch_stage(const cfd_geometry_t *geom, const cfd_params_t *params, const cfd_flow_t *flow,
                             double del_t, cfd_batch_staged_t **out)
{
    if (!out) return CFD_EINVAL;
    *out = nullptr;
    cfd_batch_staged *S = new (std::nothrow) cfd_batch_staged;
    if (!S) return CFD_ENOMEM;
    *out = S;
    auto bad = [&](cfd_status_t st, const char *msg) {
        S->status = st;
        S->error = msg;
        return st;
    };
    if (!geom || !flow || !std::isfinite(del_t)) return bad(CFD_EINVAL, "cfd_batch_add: null argument or bad time step");
    if (!geom->grid || !geom->det || !geom->deter || !geom->metric || geom->g_node < 1)
        return bad(CFD_EINVAL, "cfd_batch_add: bad geometry");
    std::atomic<bool> out_of_range{false};
    host_parallel_for((long long)geom->g_node + 1, [&](long long r0, long long r1) {
        for (long long r = r0; r < r1; ++r)
            for (int slot = 0; slot < 6; ++slot) {
                const int v = nb_of(geom->grid[r], slot);
                if (v < 0 || v > geom->g_node) out_of_range = true;
            }
    });
    if (out_of_range) return bad(CFD_EINVAL, "cfd_batch_add: neighbour index out of range");
    LatticeMap map;
    bool natural = false;
    try {
        natural = map_lattice(geom, map) && !map.ghosted() && faces_single_valued(geom, map)
                  && (long long)map.ni * map.nj * map.nk <= kLatticeMaxNodes;
    } catch (const std::bad_alloc &) {
        return bad(CFD_ENOMEM, "cfd_batch_add: out of host memory for the lattice map");
    }
    for (size_t n = 0; natural && n < map.row_of.size(); ++n) natural = map.row_of[n] == (int32_t)n + 1;
    if (!natural)
        return bad(CFD_EUNSUPPORTED, "cfd_batch_add: batched instances must be periodic lattices in row order");
    S->g_node = geom->g_node;
    S->ni = map.ni;
    S->nj = map.nj;
    S->nk = map.nk;
    S->N = map.ni * map.nj * map.nk;
    cfd_params_default(&S->prm);
    if (params) S->prm = *params;
    S->dt = del_t;
    try {
        lattice_geometry_soa(geom, map, S->m9, S->det, S->fm, S->fdet);
        const size_t rows = 9 * ((size_t)S->N + 1);
        S->flow.resize(rows);
        const double *src = reinterpret_cast<const double *>(flow);
        double *dst = host_ptr(S->flow);
        host_parallel_for((long long)rows, [&](long long a, long long e) { std::copy(src + a, src + e, dst + a); });
    } catch (const std::bad_alloc &) {
        S->m9 = S->det = S->fm = S->fdet = S->flow = HostDoubles();
        return bad(CFD_ENOMEM, "cfd_batch_add: out of host memory for the staged geometry");
    }
    return CFD_OK;
}

cfd_status_t cfd_batch_staged_free(cfd_batch_staged_t *staged)
{
    delete staged;
    return CFD_OK;
}

cfd_status_t cfd_batch_add(cfd_batch_t *b, const cfd_geometry_t *geom, const cfd_params_t *params,
                           const cfd_flow_t *flow, double del_t, int32_t *slot_out)
{
    if (!b || !slot_out) return CFD_EINVAL;
    *slot_out = -1;
    cfd_batch_staged *S = nullptr;
    const cfd_status_t st = cfd_batch_stage(geom, params, flow, del_t, &S);
    if (!S) return st;
    return cfd_batch_add_staged(b, S, slot_out);
}

cfd_status_t cfd_batch_add_staged(cfd_batch_t *b, cfd_batch_staged_t *staged, int32_t *slot_out)
{
    std::unique_ptr<cfd_batch_staged> S(staged);
    if (!b || !S || !slot_out) return CFD_EINVAL;
    *slot_out = -1;
    cfd_ctx *ctx = b->ctx;
    if (S->status != CFD_OK) return fail(ctx, S->status, S->error);
    cfd_status_t st = use_device(ctx);
    if (st != CFD_OK) return st;
    const int ni = S->ni, nj = S->nj, nk = S->nk;
    const int N = S->N;
    const uint64_t need = instance_bytes(b->precision, N);
    if (b->used + need > b->capacity) return fail(ctx, CFD_ENOMEM, "cfd_batch_add: device-memory budget exhausted");
    int slot = -1;
    for (size_t s = 0; s < b->slots.size(); ++s)
        if (!b->slots[s].active) {
            slot = (int)s;
            break;
        }
    if (slot < 0) {
        if ((int)b->slots.size() >= kMaxSlots) return fail(ctx, CFD_ENOMEM, "cfd_batch_add: too many instances");
        b->slots.emplace_back();
        slot = (int)b->slots.size() - 1;
    }
    BatchInst &I = b->slots[slot];
    I.g_node = S->g_node;
    I.ni = ni;
    I.nj = nj;
    I.nk = nk;
    I.N = N;
    I.prm = S->prm;
    I.dt = S->dt;
    const double del_t = S->dt;
    const size_t Nz = (size_t)N;
    double *m9, *det, *fm, *fdet, *prim9, *U0, *U1, *U2;
    if ((st = ialloc(b, I, 9 * Nz, &m9)) || (st = ialloc(b, I, Nz, &det)) || (st = ialloc(b, I, 9 * Nz, &fm))
        || (st = ialloc(b, I, 3 * Nz, &fdet)) || (st = ialloc(b, I, 9 * Nz, &prim9)) || (st = ialloc(b, I, 5 * Nz, &U0))
        || (st = ialloc(b, I, 5 * Nz, &U1)) || (st = ialloc(b, I, 5 * Nz, &U2))
        || (st = ialloc(b, I, 9 * (Nz + 1), &I.stage9)) || (st = ialloc(b, I, 5 * (Nz + 1), &I.stage5))) {
        free_instance(I);
        return st;
    }
    LatView &v = I.view;
    v.ni = ni;
    v.nj = nj;
    v.nk = nk;
    v.N = N;
    v.P = make_phys(&I.prm);
    v.per = 7;            // periodic in every direction
    v.loc8 = nullptr;
    v.locdirs = 0;
    v.locflag = nullptr;
    v.row_of = nullptr;
    v.dt = del_t;
    v.dt_hi = (float)del_t;
    v.dt_lo = (float)(del_t - (double)v.dt_hi);
    v.m9 = m9;
    v.det = det;
    v.fm = fm;
    v.fdet = fdet;
    v.prim9 = prim9;
    v.U0 = U0;
    v.U1 = U1;
    v.U2 = U2;
    v.flags = slot_flags(b, slot);
    v.Lout = nullptr;
    if (b->precision == CFD_PREC_MIXED) {
        float *fm32, *fdet32, *node32, *idet32;
        if ((st = ialloc(b, I, 9 * Nz, &fm32)) || (st = ialloc(b, I, 3 * Nz, &fdet32))
            || (st = ialloc(b, I, 11 * Nz, &node32)) || (st = ialloc(b, I, 2 * Nz, &idet32))
            || (st = ialloc(b, I, 9 * Nz, &v.prim32)) || (st = ialloc(b, I, 5 * Nz, &v.Q32))
            || (st = ialloc(b, I, 5 * Nz, &v.R32)) || (st = ialloc(b, I, 15 * Nz, &v.FEG32))
            || (st = ialloc(b, I, 15 * Nz, &v.V32)) || (st = ialloc(b, I, 15 * Nz, &v.Fh32))) {
            free_instance(I);
            return st;
        }
        v.fm32 = fm32;
        v.fdet32 = fdet32;
        v.node32 = node32;
        v.idet32 = idet32;
    } else if (b->precision == CFD_PREC_SPLIT) {
        float *fm32, *node32;
        double *idet64;
        if ((st = ialloc(b, I, 9 * Nz, &fm32)) || (st = ialloc(b, I, 11 * Nz, &node32)) || (st = ialloc(b, I, Nz, &idet64))
            || (st = ialloc(b, I, 9 * Nz, &v.prim32)) || (st = ialloc(b, I, 5 * Nz, &v.Q32))
            || (st = ialloc(b, I, 5 * Nz, &v.R32)) || (st = ialloc(b, I, 15 * Nz, &v.FEG32))
            || (st = ialloc(b, I, 15 * Nz, &v.V32)) || (st = ialloc(b, I, 15 * Nz, &v.Fh))
            || (st = ialloc(b, I, 10 * Nz, &v.Whl))) {
            free_instance(I);
            return st;
        }
        v.fm32 = fm32;
        v.node32 = node32;
        v.idet64 = idet64;
    } else {
        if ((st = ialloc(b, I, 5 * Nz, &v.Q)) || (st = ialloc(b, I, 15 * Nz, &v.FEG)) || (st = ialloc(b, I, 15 * Nz, &v.V))
            || (st = ialloc(b, I, 2 * Nz, &v.sh)) || (st = ialloc(b, I, 15 * Nz, &v.Fh))) {
            free_instance(I);
            return st;
        }
    }
    cudaStream_t sm = ctx->stream;
    cudaError_t e = cudaMemcpyAsync(m9, host_ptr(S->m9), 9 * Nz * 8, cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess) e = cudaMemcpyAsync(det, host_ptr(S->det), Nz * 8, cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fm, host_ptr(S->fm), 9 * Nz * 8, cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fdet, host_ptr(S->fdet), 3 * Nz * 8, cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(I.stage9, host_ptr(S->flow), 9 * (Nz + 1) * 8, cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess) e = cudaMemsetAsync(I.stage5, 0, 5 * (Nz + 1) * 8, sm);
    if (e == cudaSuccess) e = cudaMemsetAsync(v.flags, 0, sizeof(unsigned), sm);
    for (double *u : {U0, U1, U2})
        if (e == cudaSuccess) e = cudaMemsetAsync(u, 0, 5 * Nz * 8, sm);
    if (e == cudaSuccess) e = b->precision != CFD_PREC_FP64 ? cudaMemsetAsync(v.V32, 0, 15 * Nz * 4, sm)
                                                             : cudaMemsetAsync(v.V, 0, 15 * Nz * 8, sm);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(sm);
        free_instance(I);
        return cuda_fail(ctx, e, "cfd_batch_add upload");
    }
    aos_to_soa(sm, I.stage9, 9, 9, N, prim9);
    if (b->precision == CFD_PREC_MIXED) {
        StructuredLaunch S{};
        S.ni = ni;
        S.nj = nj;
        S.nk = nk;
        S.stream = sm;
        S.fm = fm;
        S.fdet = fdet;
        S.m9 = m9;
        S.det = det;
        S.fm32 = const_cast<float *>(v.fm32);
        S.fdet32 = const_cast<float *>(v.fdet32);
        S.node32 = const_cast<float *>(v.node32);
        S.idet32 = const_cast<float *>(v.idet32);
        mixed_geometry(S);
        batch_prep_mixed(v, sm);
    } else if (b->precision == CFD_PREC_SPLIT) {
        StructuredLaunch S{};
        S.ni = ni;
        S.nj = nj;
        S.nk = nk;
        S.stream = sm;
        S.fm = fm;
        S.m9 = m9;
        S.det = det;
        S.fm32 = const_cast<float *>(v.fm32);
        S.node32 = const_cast<float *>(v.node32);
        S.idet64 = const_cast<double *>(v.idet64);
        split_geometry(S);
        batch_prep_split(v, sm);
    } else {
        batch_prep_fp64(v, sm);
    }
    ctx->launches += b->precision == CFD_PREC_MIXED   ? 2 + kMixedGeometryLaunches
                     : b->precision == CFD_PREC_SPLIT ? 2 + kSplitGeometryLaunches
                                                      : 2;
    e = cudaStreamSynchronize(sm);   // host geometry vectors go out of scope
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        free_instance(I);
        return cuda_fail(ctx, e, "cfd_batch_add prep");
    }
    I.active = true;
    b->used += I.bytes;
    b->dirty = true;
    *slot_out = slot;
    return CFD_OK;
}

cfd_status_t cfd_batch_remove(cfd_batch_t *b, int32_t slot)
{
    if (!b || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].active) return CFD_EINVAL;
    use_device(b->ctx);
    cudaStreamSynchronize(b->ctx->stream);
    b->used -= b->slots[slot].bytes;
    free_instance(b->slots[slot]);
    b->dirty = true;
    return CFD_OK;
}

cfd_status_t cfd_batch_set_hold(cfd_batch_t *b, int32_t slot, int32_t hold)
{
    if (!b || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].active) return CFD_EINVAL;
    BatchInst &I = b->slots[slot];
    if (I.held != (hold != 0)) {
        I.held = hold != 0;
        b->dirty = true;    // the tile table of the next step leaves it out / takes it back
    }
    return CFD_OK;
}

namespace {

// Queues nsteps steps of every instance that is not held.
cfd_status_t enqueue_steps(cfd_batch_t *b, int32_t nsteps)
{
    if (!b || nsteps < 0) return CFD_EINVAL;
    cfd_status_t st = use_device(b->ctx);
    if (st != CFD_OK) return st;
    for (size_t s = 0; s < b->slots.size(); ++s) {
        const BatchInst &I = b->slots[s];
        if (I.active && !I.held && I.interrupted)
            return fail(b->ctx, CFD_ETIMEOUT,
                        "cfd_batch_step: slot " + std::to_string(s)
                            + " was interrupted by a barrier timeout; restore it with cfd_batch_set_flow or remove it");
    }
    if (b->dirty && (st = rebuild(b)) != CFD_OK) return st;
    if (b->ntiles == 0 || nsteps == 0) return CFD_OK;
    for (auto &I : b->slots) I.stepped = I.stepped || (I.active && I.in_table);
    if (b->use_graph && !b->graph_ok) try_capture(b);
    cudaStream_t sm = b->ctx->stream;
    for (int s = 0; s < nsteps; ++s) {
        cudaError_t e = b->graph_ok ? cudaGraphLaunch(b->gexec, sm) : launch_step(b);
        if (e != cudaSuccess) return cuda_fail(b->ctx, e, "batch step launch");
        b->ctx->launches += 3;
    }
    return CFD_OK;
}

}  // namespace

cfd_status_t cfd_batch_step(cfd_batch_t *b, int32_t nsteps)
{
    const cfd_status_t st = enqueue_steps(b, nsteps);
    return st != CFD_OK ? st : finish(b);
}

cfd_status_t cfd_batch_step_async(cfd_batch_t *b, int32_t nsteps)
{
    cfd_status_t st = enqueue_steps(b, nsteps);
    if (st != CFD_OK) return st;
    const int k = b->ev_next;
    if (!b->ev[k]) {
        const cudaError_t e = cudaEventCreateWithFlags(&b->ev[k], cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_step_async event");
    }
    cudaError_t e = cudaEventRecord(b->ev[k], b->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_step_async record");
    b->ev_live[k] = true;
    b->ev_next = k ^ 1;
    // the previous call's steps: done before this call returns, so at most
    // the steps of this call are still queued
    if (b->ev_live[k ^ 1]) {
        e = cudaEventSynchronize(b->ev[k ^ 1]);
        b->ev_live[k ^ 1] = false;
        if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_step_async wait");
    }
    return CFD_OK;
}

cfd_status_t cfd_batch_sync(cfd_batch_t *b)
{
    if (!b) return CFD_EINVAL;
    cfd_status_t st = use_device(b->ctx);
    if (st != CFD_OK) return st;
    b->ev_live[0] = b->ev_live[1] = false;
    return finish(b);
}

cfd_status_t cfd_batch_get_flow(cfd_batch_t *b, int32_t slot, cfd_flow_t *host)
{
    if (!b || !host || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].active) return CFD_EINVAL;
    use_device(b->ctx);
    BatchInst &I = b->slots[slot];
    // mixed: FP64 FLOW of the hi/lo state (after whole steps it is in slot 0)
    if (b->precision == CFD_PREC_MIXED) mixed_flow_out(I.view, 0, b->ctx->stream);
    if (b->precision == CFD_PREC_SPLIT) split_flow_out(I.view, 0, b->ctx->stream);
    soa_to_aos(b->ctx->stream, I.view.prim9, 9, 9, I.N, I.stage9);
    cudaError_t e = cudaMemcpyAsync(host, I.stage9, 9 * ((size_t)I.N + 1) * 8, cudaMemcpyDeviceToHost, b->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_get_flow");
    return CFD_OK;
}

cfd_status_t cfd_batch_get_u0(cfd_batch_t *b, int32_t slot, cfd_column_t *host)
{
    if (!b || !host || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].active) return CFD_EINVAL;
    use_device(b->ctx);
    BatchInst &I = b->slots[slot];
    if (b->precision == CFD_PREC_MIXED)
        mixed_u_out(I.view, 0, I.stage5, b->ctx->stream);
    else
        soa_to_aos(b->ctx->stream, I.view.U0, 5, 5, I.N, I.stage5);
    cudaError_t e = cudaMemcpyAsync(host, I.stage5, 5 * ((size_t)I.N + 1) * 8, cudaMemcpyDeviceToHost, b->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_get_u0");
    return CFD_OK;
}

cfd_status_t cfd_batch_slot_status(cfd_batch_t *b, int32_t slot)
{
    if (!b || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].active) return CFD_EINVAL;
    if (b->slots[slot].interrupted) return CFD_ETIMEOUT;
    unsigned w = 0;
    cudaError_t e = cudaMemcpyAsync(&w, slot_flags(b, slot), sizeof w, cudaMemcpyDeviceToHost, b->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_slot_status");
    return (w & CFD_FLAG_NONFINITE) ? CFD_ENONFINITE : CFD_OK;
}

cfd_status_t cfd_batch_set_flow(cfd_batch_t *b, int32_t slot, const cfd_flow_t *flow_host)
{
    if (!b || !flow_host || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].active) return CFD_EINVAL;
    cfd_status_t st = use_device(b->ctx);
    if (st != CFD_OK) return st;
    BatchInst &I = b->slots[slot];
    cudaStream_t sm = b->ctx->stream;
    // queued steps finish first (they may still read this instance)
    cudaError_t e = cudaStreamSynchronize(sm);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(I.stage9, flow_host, 9 * ((size_t)I.N + 1) * 8, cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess) e = cudaMemsetAsync(slot_flags(b, slot), 0, sizeof(unsigned), sm);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_set_flow upload");
    aos_to_soa(sm, I.stage9, 9, 9, I.N, I.view.prim9);
    if (b->precision == CFD_PREC_MIXED)
        batch_prep_mixed(I.view, sm);
    else if (b->precision == CFD_PREC_SPLIT)
        batch_prep_split(I.view, sm);
    else
        batch_prep_fp64(I.view, sm);
    b->ctx->launches += 2;
    e = cudaStreamSynchronize(sm);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_set_flow prep");
    I.interrupted = false;
    return CFD_OK;
}

cfd_status_t cfd_batch_set_wait_limit(cfd_batch_t *b, int64_t limit_ns)
{
    if (!b) return CFD_EINVAL;
    const long long v = limit_ns < 0 ? -1 : (long long)limit_ns;
    if (v != b->wait_limit_ns) {
        b->wait_limit_ns = v;
        b->dirty = true;   // the captured graph holds the old deadline
    }
    return CFD_OK;
}

cfd_status_t cfd_batch_set_tiling(cfd_batch_t *b, int32_t tile_nodes, int32_t max_blocks, int32_t use_graph)
{
    if (!b || max_blocks < 0) return CFD_EINVAL;
    if (tile_nodes != 0 && tile_nodes != 32 && tile_nodes != 64 && tile_nodes != 128 && tile_nodes != 256
        && tile_nodes != CFD_BATCH_FACE_TILES)
        return CFD_EINVAL;
    if (tile_nodes == CFD_BATCH_FACE_TILES && b->precision == CFD_PREC_FP64) return CFD_EINVAL;
    if (tile_nodes == CFD_BATCH_FACE_TILES) {
        b->face_tiles = true;
    } else if (tile_nodes) {
        b->face_tiles = false;
        b->threads = tile_nodes;
    }
    b->blocks_override = max_blocks;
    b->use_graph = use_graph != 0;
    b->dirty = true;
    drop_graph(b);
    return CFD_OK;
}

cfd_status_t cfd_batch_tune(cfd_batch_t *b, int32_t steps_per_trial)
{
    if (!b || steps_per_trial < 1) return CFD_EINVAL;
    cfd_status_t st = use_device(b->ctx);
    if (st != CFD_OK) return st;
    cudaStream_t sm = b->ctx->stream;
    // save the mutable state of every instance
    std::vector<std::pair<void *, size_t>> arrays;
    for (auto &I : b->slots)
        if (I.active)
            for (auto &a : mutable_arrays(I, b->precision)) arrays.push_back(a);
    size_t total = 0;
    for (auto &a : arrays) total += a.second;
    if (total == 0) return CFD_OK;
    char *backup = nullptr;
    cudaError_t e = cudaMalloc(&backup, total);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_tune backup");
    auto copy_all = [&](bool save) {
        size_t off = 0;
        for (auto &a : arrays) {
            if (save) cudaMemcpyAsync(backup + off, a.first, a.second, cudaMemcpyDeviceToDevice, sm);
            else cudaMemcpyAsync(a.first, backup + off, a.second, cudaMemcpyDeviceToDevice, sm);
            off += a.second;
        }
    };
    copy_all(true);
    // 1-D tiles of 32, 64, 128, 256 nodes, and for the reduced forms the
    // shared-memory face tiles
    std::vector<int> candidates = {32, 64, 128, 256};
    if (b->precision != CFD_PREC_FP64) candidates.push_back(CFD_BATCH_FACE_TILES);
    const int threads0 = b->threads;
    const bool faces0 = b->face_tiles;
    int best = faces0 ? CFD_BATCH_FACE_TILES : threads0;
    float best_ms = 1e30f;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    for (int T : candidates) {
        b->face_tiles = T == CFD_BATCH_FACE_TILES;
        if (!b->face_tiles) b->threads = T;
        b->dirty = true;
        if ((st = rebuild(b)) != CFD_OK) continue;
        if (b->use_graph) try_capture(b);
        auto one = [&]() { return b->graph_ok ? cudaGraphLaunch(b->gexec, sm) : launch_step(b); };
        if (one() != cudaSuccess) { cudaGetLastError(); continue; }   // warm-up
        cudaEventRecord(t0, sm);
        bool ok = true;
        for (int s = 0; s < steps_per_trial && ok; ++s) ok = one() == cudaSuccess;
        cudaEventRecord(t1, sm);
        b->ctx->launches += 3 * (steps_per_trial + 1);
        if (!ok || cudaEventSynchronize(t1) != cudaSuccess) { cudaGetLastError(); continue; }
        float ms = 0;
        cudaEventElapsedTime(&ms, t0, t1);
        if (ms < best_ms) {
            best_ms = ms;
            best = T;
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    copy_all(false);
    cudaMemsetAsync(b->d_words, 0, (4 + kMaxSlots) * sizeof(unsigned), sm);
    e = cudaStreamSynchronize(sm);
    cudaFree(backup);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "cfd_batch_tune restore");
    b->face_tiles = best == CFD_BATCH_FACE_TILES;
    b->threads = b->face_tiles ? threads0 : best;
    b->dirty = true;
    return rebuild(b);
}

cfd_status_t cfd_batch_info(const cfd_batch_t *b, cfd_batch_info_t *info)
{
    if (!b || !info) return CFD_EINVAL;
    std::memset(info, 0, sizeof *info);
    int n = 0, held = 0;
    for (auto &I : b->slots) {
        n += I.active ? 1 : 0;
        held += I.active && I.held ? 1 : 0;
    }
    info->n_active = n;
    info->n_held = held;
    info->tile_nodes = b->face_tiles && b->precision != CFD_PREC_FP64 ? kFaceThreads : b->threads;
    info->face_tiles = b->face_tiles && b->precision != CFD_PREC_FP64 ? 1 : 0;
    info->blocks = b->blocks;
    info->graph = b->graph_ok ? 1 : 0;
    info->precision = b->precision;
    uint64_t nodes = 0;
    for (auto &I : b->slots)
        if (I.active) nodes += (uint64_t)I.N;
    info->nodes_total = nodes;
    info->device_bytes = b->used;
    info->capacity_bytes = b->capacity;
    return CFD_OK;
}

}  // extern "C"

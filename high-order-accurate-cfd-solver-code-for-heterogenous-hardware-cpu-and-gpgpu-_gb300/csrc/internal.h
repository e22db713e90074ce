// internal.h -- host-side objects behind the C ABI (context, solver) and the
// launch helpers shared by the .cu translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "cfd_rhs.h"
#include "physics.cuh"

// Device error-flag bits (one 32-bit word per context, or per instance in
// the batched solver).
enum : unsigned {
    CFD_FLAG_BAD_INDEX = 1u,   // a neighbour index outside [0, n_rows)
    CFD_FLAG_NONFINITE = 2u,   // NaN/Inf in an advanced state
    CFD_FLAG_TIMEOUT = 4u      // a bounded wait gave up
};

struct cfd_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool async = false;
    int32_t n_rows = 0;
    unsigned *d_flags = nullptr;   // device error word
    unsigned *h_flags = nullptr;   // pinned mirror
    uint64_t launches = 0;
    std::string last_error;
    // cfd_weno's face scratch (15 doubles per row, allocated by
    // cfd_ctx_set_rows; null: each row evaluates both faces itself)
    double *d_face = nullptr;   // face_scratch_bytes(face_rows)
    long long face_rows = 0;
    unsigned face_gen = 0;
    bool face_reuse = true;
    // device mirrors of host buffers handed to the kernel entry points:
    // host pointer -> (device buffer, bytes)
    std::unordered_map<const void *, std::pair<void *, size_t>> mirrors;
};

namespace cfd {

// Records a CUDA error on the context; returns the status to hand back.
cfd_status_t cuda_fail(cfd_ctx *ctx, cudaError_t e, const char *what);
cfd_status_t fail(cfd_ctx *ctx, cfd_status_t s, const std::string &msg);
// Makes ctx->device current on this host thread.
cfd_status_t use_device(cfd_ctx *ctx);
// After a launch: checks the launch, and in synchronous mode waits and
// converts device flags into a status (clearing them).
cfd_status_t after_launch(cfd_ctx *ctx, const char *what);
// Waits for the stream and converts/clears device flags.
cfd_status_t drain(cfd_ctx *ctx);
cfd_status_t flags_to_status(cfd_ctx *ctx, unsigned flags);
bool is_device_pointer(const void *p);
Phys make_phys(const cfd_params_t *p);

inline unsigned blocks_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// One buffer argument of an entry point.  Device pointers are used as
// given.  A host pointer (the reference host's std::vector data) gets a
// device mirror of n_rows rows owned by the context: stage_in copies the
// host rows in before the launch; stage_out copies buffers the call writes
// back after it (unless the launch failed) and waits -- the whole-array
// copies Solver.cpp:371-541 makes around every launch.
struct BufArg {
    void *user;
    size_t row_bytes;
    bool written;
    long long rows = 0;   // rows of a host buffer (0: the context's n_rows)
    void *dev = nullptr;
    bool host = false;
};
cfd_status_t stage_in(cfd_ctx *ctx, BufArg *a, int n, const char *who);
cfd_status_t stage_out(cfd_ctx *ctx, const BufArg *a, int n, cfd_status_t launch_status);

// Drop-in kernel launchers (dropin.cu).  All pointers are device pointers.
// U_Q; with a scratch of >= n_rows rows (15 doubles each, cfd_weno's face
// scratch) it first computes sqrt(rho) and H once per row.  Returns the
// kernels launched (2 or 1).
int launch_uq(cudaStream_t st, double *U, double *Q, const int *grid, const double *det, const double *flow,
              double *roe, int n_items, int n_rows, unsigned *flags, double *node_scratch, long long scratch_rows);
void launch_viscous(cudaStream_t st, const Phys &P, const double *U, double *F, double *E, double *G, double *Fv,
                    double *Ev, double *Gv, const int *grid, const double *metric, const double *det, double *flow,
                    int n_items, int n_rows, unsigned *flags);
void launch_weno(cudaStream_t st, const Phys &P, int j, double mach, double dt, const double *deter,
                 const double *det, double *U0, double *U1, double *U2, const int *grid, const double *Q,
                 const double *metric, const double *roe, const double *Fv, const double *Ev, const double *Gv,
                 const double *F, const double *E, const double *G, double *flow, int n_items, int n_rows,
                 unsigned *flags, double *L_out, double *face_scratch, long long scratch_rows, unsigned gen);
// Face scratch of launch_weno for `rows` rows: +1/2 faces [3][5][rows] and
// -1/2 faces [3][5][rows] (doubles), then generation stamps [3][rows]
// (unsigned, zero when allocated).  gen: a value new to the scratch on every
// call (next_face_gen).
inline size_t face_scratch_bytes(long long rows) { return (size_t)rows * (30 * sizeof(double) + 3 * sizeof(unsigned)); }
inline unsigned *face_stamps(double *scratch, long long rows) { return reinterpret_cast<unsigned *>(scratch + 30 * rows); }
inline unsigned next_face_gen(unsigned &g)
{
    g = g + 1 == 0 ? 1 : g + 1;
    return g;
}
// Kernels one launch_weno issues: 2 with a face scratch of >= n_items rows,
// else 1.
inline int weno_launches(const double *face_scratch, long long scratch_rows, int n_items)
{
    return face_scratch && scratch_rows >= n_items ? 3 : 1;
}

}  // namespace cfd

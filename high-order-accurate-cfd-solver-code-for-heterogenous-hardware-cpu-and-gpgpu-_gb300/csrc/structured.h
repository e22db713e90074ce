// structured.h -- launch interface of the face-based lattice kernels.
#pragma once

#include <cuda_runtime.h>

#include "lattice.cuh"
#include "physics.cuh"

namespace cfd {

// Device pointers of one lattice (SoA, [component][N]).
struct StructuredLaunch {
    int ni, nj, nk;
    cudaStream_t stream;
    Phys P;
    int mixed;                 // 1: the mixed-precision form (mixed.cu); 2: the split form (split.cu)
    const double *m9;          // [9][N]   node metrics
    const double *det;         // [N]
    const double *fm;          // [3 dir][3 comp][N] metric of face n+1/2
    const double *fdet;        // [3][N]   det of face n+1/2
    double *prim9;             // [9][N]   FLOW fields u,v,w,p,t,rho,mu,a,e (mixed: in/out only)
    double *U[3];              // [5][N]   U0, U1, U2 (mixed: hi/lo FP32 pairs in the same bytes)
    double *Q;                 // [5][N]
    double *FEG;               // [3][5][N] contravariant node fluxes
    double *V;                 // [3][5][N] viscous fluxes
    double *sh;                // [2][N]   sqrt(rho), H
    double *Fh;                // [3][5][N] corrected face fluxes
    unsigned *flags;
    // mixed-precision form (FP32 stage intermediates, mixed.cu)
    float *Q32 = nullptr;      // [5][N]
    float *R32 = nullptr;      // [5][N] u, v, w, sqrt(rho), H
    float *FEG32 = nullptr;    // [3][5][N]
    float *V32 = nullptr;      // [3][5][N]
    float *Fh32 = nullptr;     // [3][5][N]
    float *fm32 = nullptr;     // [3][3][N]
    float *fdet32 = nullptr;   // [3][N]
    float *node32 = nullptr;   // [11][N] node metrics, det, det^(-1/3)
    float *idet32 = nullptr;   // [2][N] 1/det hi, lo
    double *idet64 = nullptr;  // [N] 1/det (split form)
    float *Whl = nullptr;      // [10][N] hi/lo read copy of the stage's state (split form)
    float *prim32 = nullptr;   // [9][N] FP32 pressure (LF_P) and mu (LF_MU) of the stage
    // mixed form: side stream and fork/join events for the viscous pass,
    // and two more for the j and k face passes (null: everything on `stream`)
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaStream_t face_side[2] = {nullptr, nullptr};
    cudaEvent_t face_join[2] = {nullptr, nullptr};
    // lattice shape beyond a plain periodic box (LatView::per, loc8, locdirs,
    // row_of)
    // face-tile widths of the mixed and split face passes: faces along i
    // (32, 64 or 128) and along j and k (8, 16 or 32) per block of 128
    int tile_i = 64, tile_jk = 16;
    // FP64 form: blocks of 128 per SM the face passes along i, j, k request
    // (2, 3 or 4: their register budget; the solver's tuner picks)
    int face_mb[3] = {3, 3, 2};
    int per = 7;
    const unsigned char *loc8 = nullptr;
    int locdirs = 0;
    const unsigned char *locflag = nullptr;   // LatView::locflag
    const int *row_of = nullptr;
};

// Where the mixed stage takes its U_Q (prep) from: nothing (the previous
// stage's update already produced it), the FP64 FLOW (after an upload), or
// the hi/lo state in U slot 0..2.
constexpr int kPrepNone = -2;
constexpr int kPrepFromFlow = -1;

// Mixed-precision stage j (mixed.cu).  prep_from as above; the update always
// produces the next stage's U_Q (its state lands in slot (j+1) mod 3).
// Returns the number of launches; ev (optional) gets one event before and one
// after each launch (launches + 1 events), names[i] the launch names.
int mixed_stage(const StructuredLaunch &S, int j, double dt, double *Lout, cudaEvent_t *ev, int prep_from,
                const char **names);
// FP32 copies of the face and node metrics and 1/det as hi/lo (once, after
// upload; kernels launched: 3).
constexpr int kMixedGeometryLaunches = 3;
void mixed_geometry(const StructuredLaunch &S);
// FP64 FLOW (g.prim9, SoA) from the hi/lo state in slot q; mu from prim32.
void mixed_flow_out(const LatView &g, int q, cudaStream_t st);
// FP64 U of slot q as AoS rows 1..N of 5 doubles.
void mixed_u_out(const LatView &g, int q, double *aos, cudaStream_t st);

// Split-precision stage j (split.cu): the same sequencing and prep sources
// as mixed_stage, the state in FP64 slots.
int split_stage(const StructuredLaunch &S, int j, double dt, double *Lout, cudaEvent_t *ev, int prep_from,
                const char **names);
// FP32 copies of the face and node metrics and the FP64 1/det (once, after
// upload; kernels launched: 2).
constexpr int kSplitGeometryLaunches = 2;
void split_geometry(const StructuredLaunch &S);
// FP64 FLOW (g.prim9, SoA) from the FP64 state in slot q; mu from prim32.
void split_flow_out(const LatView &g, int q, cudaStream_t st);
// U_Q of slot dst from FLOW (src = kPrepFromFlow) or from the state in slot
// src (one launch).
void split_prep(const LatView &g, int src, int dst, cudaStream_t st);

// Device view of a StructuredLaunch for one stage.
inline LatView make_view(const StructuredLaunch &S, double dt, double *Lout)
{
    LatView g{};
    g.ni = S.ni;
    g.nj = S.nj;
    g.nk = S.nk;
    g.N = S.ni * S.nj * S.nk;
    g.P = S.P;
    g.dt = dt;
    g.m9 = S.m9;
    g.det = S.det;
    g.fm = S.fm;
    g.fdet = S.fdet;
    g.dt_hi = (float)dt;
    g.dt_lo = (float)(dt - (double)g.dt_hi);
    g.fm32 = S.fm32;
    g.fdet32 = S.fdet32;
    g.node32 = S.node32;
    g.idet32 = S.idet32;
    g.idet64 = S.idet64;
    g.Whl = S.Whl;
    g.prim9 = S.prim9;
    g.prim32 = S.prim32;
    g.U0 = S.U[0];
    g.U1 = S.U[1];
    g.U2 = S.U[2];
    g.Q = S.Q;
    g.FEG = S.FEG;
    g.V = S.V;
    g.sh = S.sh;
    g.Fh = S.Fh;
    g.Q32 = S.Q32;
    g.R32 = S.R32;
    g.FEG32 = S.FEG32;
    g.V32 = S.V32;
    g.Fh32 = S.Fh32;
    g.flags = S.flags;
    g.Lout = Lout;
    g.per = S.per;
    g.loc8 = S.loc8;
    g.locdirs = S.locdirs;
    g.locflag = S.locflag;
    g.row_of = S.row_of;
    return g;
}

// One RK stage j of the host loop; Lout (device [5][N]) may be null.
// Returns the number of kernel launches; ev (optional, at least
// kMaxStageLaunches+1 entries) receives events bracketing every launch and
// names (optional) the launch names.  prep_from as for mixed_stage (the FP64
// form always runs its own prep from FLOW).
constexpr int kMaxStageLaunches = 6;
int structured_stage(const StructuredLaunch &S, int j, double dt, double *Lout, cudaEvent_t *ev = nullptr,
                     const char **names = nullptr, int prep_from = kPrepFromFlow);

// One face pass along d with face tiles of width `tile` (the tuner's
// candidates, mixed.cu / split.cu), and a uniform state in the FP32 face
// inputs (Q32, R32, FEG32) for timing them before any state exists.
// The FP64 face pass along d at `mb` blocks per SM (face_fp64_mb*.cu), and
// stage jst's prep alone (the face passes' inputs, for the tuner).
void fp64_face_pass_mb2(const LatView &g, int d, cudaStream_t st);
void fp64_face_pass_mb3(const LatView &g, int d, cudaStream_t st);
void fp64_face_pass_mb4(const LatView &g, int d, cudaStream_t st);
void fp64_face_pass(const LatView &g, int d, int mb, cudaStream_t st);
void fp64_face_pass(const StructuredLaunch &S, int d, int mb, cudaStream_t st);
void fp64_prep_pass(const StructuredLaunch &S, int jst);
void mixed_face_pass(const StructuredLaunch &S, int d, int tile, cudaStream_t st);
void split_face_pass(const StructuredLaunch &S, int d, int tile, cudaStream_t st);
void reduced_uniform_inputs(const StructuredLaunch &S, cudaStream_t st);

// AoS reference rows <-> SoA [comp][N]; node n is row row_of[n] (row n + 1
// when row_of is null).
void aos_to_soa(cudaStream_t st, const double *aos, int stride, int ncomp, long long N, double *soa,
                const int *row_of = nullptr);
void soa_to_aos(cudaStream_t st, const double *soa, int stride, int ncomp, long long N, double *aos,
                const int *row_of = nullptr);

}  // namespace cfd

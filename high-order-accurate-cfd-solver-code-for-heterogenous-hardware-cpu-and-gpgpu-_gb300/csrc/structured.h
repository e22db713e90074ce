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
    int mixed;                 // 1: characteristic/WENO/LLF in FP32
    const double *m9;          // [9][N]   node metrics
    const double *det;         // [N]
    const double *fm;          // [3 dir][3 comp][N] metric of face n+1/2
    const double *fdet;        // [3][N]   det of face n+1/2
    double *prim9;             // [9][N]   FLOW fields u,v,w,p,t,rho,mu,a,e
    double *U[3];              // [5][N]   U0, U1, U2
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
    float *m932 = nullptr;     // [9][N] node metrics
    double *idet = nullptr;    // [N] 1/det
};

// The three face-flux launches of the mixed-precision form (mixed.cu).
// Mixed-precision stage (mixed.cu).  With prep = false the stage's U_Q
// outputs are taken as already produced (by the previous stage's fused
// update); with fuse = true the update also produces the next stage's.
// Returns the number of launches; ev (optional) gets one event before and one
// after each launch (launches + 1 events), names[i] the launch names.
int mixed_stage(const StructuredLaunch &S, int j, double dt, double *Lout, cudaEvent_t *ev, bool prep, bool fuse,
                const char **names);
// FP32 copies of the node metrics, face metrics and face dets, and 1/det
// (once, after upload).
// FP32 copies of the face and node metrics and 1/det (kernels launched: 4)
constexpr int kMixedGeometryLaunches = 4;
void mixed_geometry(const StructuredLaunch &S);

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
    g.fm32 = S.fm32;
    g.fdet32 = S.fdet32;
    g.m9_32 = S.m932;
    g.idet = S.idet;
    g.prim9 = S.prim9;
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
    return g;
}

// One RK stage j of the host loop; Lout (device [5][N]) may be null.
// Returns the number of kernel launches; ev (optional, at least
// kMaxStageLaunches+1 entries) receives events bracketing every launch and
// names (optional) the launch names.  prep/fuse as for mixed_stage (the FP64
// form always runs its own prep and no fused update).
constexpr int kMaxStageLaunches = 6;
int structured_stage(const StructuredLaunch &S, int j, double dt, double *Lout, cudaEvent_t *ev = nullptr,
                     const char **names = nullptr, bool prep = true, bool fuse = false);

void aos_to_soa(cudaStream_t st, const double *aos, int stride, int ncomp, long long N, double *soa);
void soa_to_aos(cudaStream_t st, const double *soa, int stride, int ncomp, long long N, double *aos);

}  // namespace cfd

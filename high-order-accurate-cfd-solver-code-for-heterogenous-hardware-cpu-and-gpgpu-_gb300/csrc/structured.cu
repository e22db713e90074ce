// structured.cu -- face-based RHS kernels for a periodic (i,j,k) lattice.
//
// When the reference's neighbour table is a periodic lattice (detected by the
// solver at create time), the same arithmetic runs on a structure-of-arrays
// layout with index arithmetic instead of neighbour chains, and every face is
// computed once.  The reference computes each face twice: as i+1/2 of node i
// and as i-1/2 of node i+1, from identical inputs (the face metric and face
// det of Main.cpp:2369-2440 are single-valued, the Roe average is symmetric
// in its two nodes), so one evaluation per face gives the same fluxes.
//
// Per RK stage j:
//   k_prep    pointwise: Q, U_j = det*Q (U_Q.cl), contravariant node fluxes
//             F,E,G (Viscous.cl:560-631), sqrt(rho) and H for the Roe average
//   k_visc    radius-2 star: viscous + MTS SGS fluxes Fv,Ev,Gv and mu
//   k_face<d> one thread per face i+1/2 along d: Roe eigenvectors, WENO5,
//             LLF, 6th-order correction -> corrected face flux
//   k_update  pointwise + radius-2: L = -(flux differences + viscous
//             divergence), SSP-RK3 stage j, primitive recovery
// Layout: every field is [component][N] with n = i + ni*(j + nj*k).
//
// The FP64 kernels use the exact arithmetic layer (physics_exact.cuh) and
// this file is compiled with --fmad=false: the face flux of face i+1/2 is
// bit-identical to what the reference computes for it (twice).  The FP32
// face kernel of the mixed-precision form lives in mixed.cu.
#include "internal.h"
#include "physics_exact.cuh"
#include "structured.h"

namespace cfd {

__device__ __forceinline__ int wrap(int x, int n)
{
    x %= n;
    return x < 0 ? x + n : x;
}

struct Lat {
    int ni, nj, nk;
    long long N;
    __device__ __forceinline__ void ijk(long long n, int &i, int &j, int &k) const
    {
        i = (int)(n % ni);
        long long r = n / ni;
        j = (int)(r % nj);
        k = (int)(r / nj);
    }
    __device__ __forceinline__ long long at(int i, int j, int k) const
    {
        return (long long)wrap(i, ni) + (long long)ni * ((long long)wrap(j, nj) + (long long)nj * wrap(k, nk));
    }
    // node at offset o along direction d from (i,j,k)
    __device__ __forceinline__ long long step(int i, int j, int k, int d, int o) const
    {
        return d == 0 ? at(i + o, j, k) : (d == 1 ? at(i, j + o, k) : at(i, j, k + o));
    }
};

enum { FU = 0, FV = 1, FW = 2, FP = 3, FT = 4, FRHO = 5, FMU = 6, FA = 7, FE = 8 };

// ------------------------------------------------------------------ prep --
__global__ void __launch_bounds__(128) k_prep(Lat g, const double *__restrict__ m9, const double *__restrict__ det,
                                              const double *__restrict__ prim9, double *__restrict__ Uj,
                                              double *__restrict__ Q, double *__restrict__ FEG,
                                              double *__restrict__ sh)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    const double rho = prim9[FRHO * N + n], u = prim9[FU * N + n], v = prim9[FV * N + n], w = prim9[FW * N + n],
                 p = prim9[FP * N + n];
    const double D = det[n];
    const double ke = 0.5 * rho * (u * u + v * v + w * w);
    const double E = (p / 0.4) + ke;
    Q[0 * N + n] = rho;
    Q[1 * N + n] = rho * u;
    Q[2 * N + n] = rho * v;
    Q[3 * N + n] = rho * w;
    Q[4 * N + n] = E;
    Uj[0 * N + n] = D * rho;
    Uj[1 * N + n] = D * rho * u;
    Uj[2 * N + n] = D * rho * v;
    Uj[3 * N + n] = D * rho * w;
    Uj[4 * N + n] = D * E;
    double m[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) m[k] = m9[k * N + n];
    const double prim[5] = {rho, u, v, w, p};
    double F[5], Ec[5], G[5];
    ex::node_flux(prim, m, D, F, Ec, G);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        FEG[(0 * 5 + c) * N + n] = F[c];
        FEG[(1 * 5 + c) * N + n] = Ec[c];
        FEG[(2 * 5 + c) * N + n] = G[c];
    }
    sh[n] = sqrt(rho);
    sh[N + n] = ex::enthalpy(rho, u, v, w, p);
}

// ------------------------------------------------------------- viscous --
__global__ void __launch_bounds__(128) k_visc(Lat g, Phys P, const double *__restrict__ m9,
                                              const double *__restrict__ det, const double *__restrict__ Uj,
                                              double *__restrict__ prim9, double *__restrict__ V)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    int i, j, k;
    g.ijk(n, i, j, k);
    double dU[3][5], KS[3];
    double Ui[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) Ui[c] = Uj[c * N + n];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long m2 = g.step(i, j, k, d, -2), m1 = g.step(i, j, k, d, -1), p1 = g.step(i, j, k, d, 1),
                        p2 = g.step(i, j, k, d, 2);
#pragma unroll
        for (int c = 0; c < 5; ++c)
            dU[d][c] = ex::central4(Uj[c * N + m2], Uj[c * N + m1], Uj[c * N + p1], Uj[c * N + p2]);
        const int c = d + 1;
        KS[d] = ex::ks(Ui[c], Ui[0], Uj[c * N + m1], Uj[m1], Uj[c * N + p1], Uj[p1]);
    }
    double m[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) m[q] = m9[q * N + n];
    const double prim[5] = {prim9[FRHO * N + n], prim9[FU * N + n], prim9[FV * N + n], prim9[FW * N + n],
                            prim9[FP * N + n]};
    double Fv[5], Ev[5], Gv[5], mu;
    const ex::Visc Vp{P.mach, P.reynolds, P.prandtl, P.t_inf, P.les};
    ex::viscous_node(dU, Ui, m, det[n], prim, KS, Vp, Fv, Ev, Gv, mu);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        V[(0 * 5 + c) * N + n] = Fv[c];
        V[(1 * 5 + c) * N + n] = Ev[c];
        V[(2 * 5 + c) * N + n] = Gv[c];
    }
    prim9[FMU * N + n] = mu;
}

// Sutherland viscosity only (inviscid runs still report mu, Viscous.cl:458).
__global__ void __launch_bounds__(128) k_mu_only(Lat g, Phys P, const double *__restrict__ Uj, double *__restrict__ prim9)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    const double Ui[5] = {Uj[n], Uj[N + n], Uj[2 * N + n], Uj[3 * N + n], Uj[4 * N + n]};
    prim9[FMU * N + n] = ex::mu_of(Ui, P.mach, P.t_inf);
}

// ---------------------------------------------------------------- faces --
// One thread per face n+1/2 along D (FP64, exact arithmetic): Roe average of
// the two adjacent nodes, LLF face flux and the 6th-order correction.
template <int D>
__global__ void __launch_bounds__(128) k_face(Lat g, double eps, const double *__restrict__ Q,
                                              const double *__restrict__ prim9, const double *__restrict__ sh,
                                              const double *__restrict__ fm, const double *__restrict__ fdet,
                                              const double *__restrict__ FEG, double *__restrict__ Fh)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    int i, j, k;
    g.ijk(n, i, j, k);
    long long s[6];
#pragma unroll
    for (int o = 0; o < 6; ++o) s[o] = g.step(i, j, k, D, o - 2);
    double pts[6][5];
#pragma unroll
    for (int o = 0; o < 6; ++o)
#pragma unroll
        for (int c = 0; c < 5; ++c) pts[o][c] = Q[c * N + s[o]];
    double roe[5];
    {
        const long long l = s[2], r = s[3];   // node (left) and its +D neighbour
        ex::roe(sh[r], prim9[FU * N + r], prim9[FV * N + r], prim9[FW * N + r], sh[N + r], sh[l], prim9[FU * N + l],
                prim9[FV * N + l], prim9[FW * N + l], sh[N + l], roe);
    }
    double Fhat[5];
    ex::face_flux(pts, fm[(D * 3 + 0) * N + n], fm[(D * 3 + 1) * N + n], fm[(D * 3 + 2) * N + n], fdet[D * N + n], roe,
                  eps, Fhat);
    const double *NF = FEG + (size_t)D * 5 * N;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        double f[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) f[o] = NF[c * N + s[o]];
        Fh[(D * 5 + c) * N + n] = ex::corrected(Fhat[c], f);
    }
}

// --------------------------------------------------------------- update --
__global__ void __launch_bounds__(128) k_update(Lat g, int viscous, int jst, double mach, double dt,
                                                const double *__restrict__ det, const double *__restrict__ Fh,
                                                const double *__restrict__ V, double *__restrict__ U0,
                                                double *__restrict__ U1, double *__restrict__ U2,
                                                double *__restrict__ prim9, unsigned *flags, double *__restrict__ Lout)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const long long N = g.N;
    int i, j, k;
    g.ijk(n, i, j, k);
    double dflux[3][5], dvis[3][5];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long m1 = g.step(i, j, k, d, -1);
#pragma unroll
        for (int c = 0; c < 5; ++c) dflux[d][c] = Fh[(d * 5 + c) * N + n] - Fh[(d * 5 + c) * N + m1];
        if (viscous) {
            const long long m2 = g.step(i, j, k, d, -2), p1 = g.step(i, j, k, d, 1), p2 = g.step(i, j, k, d, 2);
            const double *Vd = V + (size_t)d * 5 * N;
#pragma unroll
            for (int c = 0; c < 5; ++c) dvis[d][c] = ex::central4(Vd[c * N + m2], Vd[c * N + m1], Vd[c * N + p1], Vd[c * N + p2]);
        } else {
#pragma unroll
            for (int c = 0; c < 5; ++c) dvis[d][c] = 0.0;
        }
    }
    double L[5];
#pragma unroll
    for (int c = 0; c < 5; ++c)
        L[c] = (-1.0) * (dflux[0][c] + dflux[1][c] + dflux[2][c] + dvis[0][c] + dvis[1][c] + dvis[2][c]);
    if (Lout) {
#pragma unroll
        for (int c = 0; c < 5; ++c) Lout[c * N + n] = L[c];
    }
    double u0[5], u1[5], u2[5], Un[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) { u0[c] = U0[c * N + n]; u1[c] = U1[c * N + n]; u2[c] = U2[c * N + n]; }
    double rho, u, v, w, e, p, t, a;
    ex::rk_and_primitives(jst, dt, mach, det[n], u0, u1, u2, L, Un, rho, u, v, w, e, p, t, a);
    double *Uo = jst == 0 ? U1 : (jst == 1 ? U2 : U0);
#pragma unroll
    for (int c = 0; c < 5; ++c) Uo[c * N + n] = Un[c];
    prim9[FRHO * N + n] = rho;
    prim9[FU * N + n] = u;
    prim9[FV * N + n] = v;
    prim9[FW * N + n] = w;
    prim9[FE * N + n] = e;
    prim9[FP * N + n] = p;
    prim9[FT * N + n] = t;
    prim9[FA * N + n] = a;
    if (!(isfinite(rho) && isfinite(u) && isfinite(v) && isfinite(w) && isfinite(p))) atomicOr(flags, CFD_FLAG_NONFINITE);
}

// ----------------------------------------------------- layout transforms --
// AoS rows 1..N (row stride `stride` doubles) <-> SoA [comp][N].
__global__ void k_aos_to_soa(const double *__restrict__ aos, int stride, int ncomp, long long N, double *__restrict__ soa)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * ncomp) return;
    const long long n = t / ncomp;
    const int c = (int)(t % ncomp);
    soa[c * N + n] = aos[(n + 1) * stride + c];
}

__global__ void k_soa_to_aos(const double *__restrict__ soa, int stride, int ncomp, long long N, double *__restrict__ aos)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * ncomp) return;
    const long long n = t / ncomp;
    const int c = (int)(t % ncomp);
    aos[(n + 1) * stride + c] = soa[c * N + n];
}

// ------------------------------------------------------------- launchers --
static Lat lat(const StructuredLaunch &S) { return Lat{S.ni, S.nj, S.nk, (long long)S.ni * S.nj * S.nk}; }

void structured_stage(const StructuredLaunch &S, int jst, double dt, double *Lout, cudaEvent_t *ev)
{
    if (S.mixed) {
        mixed_stage(S, jst, dt, Lout, ev);
        return;
    }
    const Lat g = lat(S);
    const unsigned nb = blocks_for(g.N, 128);
    cudaStream_t st = S.stream;
    double *Uj = S.U[jst];
    int e = 0;
    auto mark = [&]() {
        if (ev) cudaEventRecord(ev[e++], st);
    };
    mark();
    k_prep<<<nb, 128, 0, st>>>(g, S.m9, S.det, S.prim9, Uj, S.Q, S.FEG, S.sh);
    mark();
    if (S.P.viscous)
        k_visc<<<nb, 128, 0, st>>>(g, S.P, S.m9, S.det, Uj, S.prim9, S.V);
    else
        k_mu_only<<<nb, 128, 0, st>>>(g, S.P, Uj, S.prim9);
    mark();
    k_face<0><<<nb, 128, 0, st>>>(g, S.P.eps, S.Q, S.prim9, S.sh, S.fm, S.fdet, S.FEG, S.Fh);
    mark();
    k_face<1><<<nb, 128, 0, st>>>(g, S.P.eps, S.Q, S.prim9, S.sh, S.fm, S.fdet, S.FEG, S.Fh);
    mark();
    k_face<2><<<nb, 128, 0, st>>>(g, S.P.eps, S.Q, S.prim9, S.sh, S.fm, S.fdet, S.FEG, S.Fh);
    mark();
    k_update<<<nb, 128, 0, st>>>(g, S.P.viscous, jst, S.P.mach, dt, S.det, S.Fh, S.V, S.U[0], S.U[1], S.U[2], S.prim9,
                                 S.flags, Lout);
    mark();
}

const char *structured_kernel_name(int i, bool viscous)
{
    static const char *names[6] = {"prep", "viscous", "face_i", "face_j", "face_k", "update"};
    if (i == 1 && !viscous) return "mu_only";
    return (i >= 0 && i < 6) ? names[i] : "?";
}

int structured_launches_per_stage() { return 6; }

void aos_to_soa(cudaStream_t st, const double *aos, int stride, int ncomp, long long N, double *soa)
{
    const long long t = N * ncomp;
    k_aos_to_soa<<<blocks_for(t, 256), 256, 0, st>>>(aos, stride, ncomp, N, soa);
}

void soa_to_aos(cudaStream_t st, const double *soa, int stride, int ncomp, long long N, double *aos)
{
    const long long t = N * ncomp;
    k_soa_to_aos<<<blocks_for(t, 256), 256, 0, st>>>(soa, stride, ncomp, N, aos);
}

}  // namespace cfd

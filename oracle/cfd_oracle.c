/*
 * cfd_oracle.c -- CPU restatement of the reference RHS path (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library, never part of
 * the product path.  Each function names the reference lines it restates.
 * Arithmetic is written in the same evaluation order as the reference kernels
 * so that, built with -ffp-contract=off, it agrees with the reference sources
 * compiled as host code (oracle/_ref) to the last bit on most inputs.
 *
 * Index conventions of the reference ABI (functions.h:57-113, U_Q.cl:51-56):
 *   direction d = 0 (i, zeta), 1 (j, eta), 2 (k, xi)
 *   +d neighbour: N1 / N0 / N4;   -d neighbour: N3 / N2 / N5
 *   TRANSFORMED blocks of 9: node, ip, im, jp, jm, kp, km; inside a block
 *       zeta_{x,y,z}, eta_{x,y,z}, xi_{x,y,z}
 *   ROE_AVERAGING blocks of 6 (u,v,w,p,h,rho): ip, jp, kp, im, jm, km
 *   DETERM: ip, im, jp, jm, kp, km
 */
#include "cfd_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;
static int g_poison = 0;

/* With poison on, the derivative branches the reference leaves undefined
 * yield NaN, so a checker can mask exactly the outputs that depend on them. */
void oracle_set_poison(int on) { g_poison = on; }

void oracle_set_threads(int n) { g_threads = n; }
int oracle_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

static inline double sq(double x) { return x * x; }

static inline int nb_plus(const or_grid *g, int d)
{
    return d == 0 ? g->N1 : (d == 1 ? g->N0 : g->N4);
}
static inline int nb_minus(const or_grid *g, int d)
{
    return d == 0 ? g->N3 : (d == 1 ? g->N2 : g->N5);
}

/* idx[d][o+3] for o = -3..3, following the chained neighbour reads of
 * Weno.cl:159-226 and Viscous.cl:99-163. */
static void gather_star(const or_grid *grid, int gid, int idx[3][7], int loc[3][7])
{
    for (int d = 0; d < 3; ++d) {
        idx[d][3] = gid;
        int p = gid, m = gid;
        for (int o = 1; o <= 3; ++o) {
            p = nb_plus(&grid[p], d);
            m = nb_minus(&grid[m], d);
            idx[d][3 + o] = p;
            idx[d][3 - o] = m;
        }
        for (int o = 0; o < 7; ++o) loc[d][o] = grid[idx[d][o]].loc;
    }
}

/* ---------------------------------------------------------------- U_Q ---- */

/* Total enthalpy per unit mass as written in U_Q.cl:64-65. */
static inline double enthalpy(const or_flow *f)
{
    return ((f->p / 0.4) + 0.5 * f->rho * (f->u * f->u + f->v * f->v + f->w * f->w) + f->p) / f->rho;
}

/* U_Q.cl:36-125.  ROE block order ip, jp, kp, im, jm, km; the loop walks the
 * reference's face order ip, im, jp, jm, kp, km. */
void oracle_uq(int n_items, or_col5 *U_C, or_col5 *Q_C, const or_grid *grid,
               const double *det, const or_flow *flow, or_roe *roe)
{
#pragma omp parallel for schedule(static) num_threads(oracle_get_threads())
    for (int gid = 0; gid < n_items; ++gid) {
        const or_flow *fi = &flow[gid];
        const double DET_I = det[gid];
        const double sqr_i = sqrt(fi->rho);
        const double h_i = enthalpy(fi);
        for (int d = 0; d < 3; ++d) {
            for (int s = 0; s < 2; ++s) {
                int nb = s == 0 ? nb_plus(&grid[gid], d) : nb_minus(&grid[gid], d);
                const or_flow *fn = &flow[nb];
                double sqr_b = sqrt(fn->rho);
                double *r = &roe[gid].v[6 * (d + 3 * s)];
                r[5] = sqr_b * sqr_i;
                r[0] = (sqr_b * fn->u + sqr_i * fi->u) / (sqr_b + sqr_i);
                r[1] = (sqr_b * fn->v + sqr_i * fi->v) / (sqr_b + sqr_i);
                r[2] = (sqr_b * fn->w + sqr_i * fi->w) / (sqr_b + sqr_i);
                r[4] = (sqr_b * enthalpy(fn) + sqr_i * h_i) / (sqr_b + sqr_i);
                /* roe_p_* is declared but never written by the reference. */
            }
        }
        const double ke = 0.5 * fi->rho * (fi->u * fi->u + fi->v * fi->v + fi->w * fi->w);
        U_C[gid].N[0] = DET_I * fi->rho;
        U_C[gid].N[1] = DET_I * fi->rho * fi->u;
        U_C[gid].N[2] = DET_I * fi->rho * fi->v;
        U_C[gid].N[3] = DET_I * fi->rho * fi->w;
        U_C[gid].N[4] = DET_I * ((fi->p / 0.4) + ke);
        Q_C[gid].N[0] = fi->rho;
        Q_C[gid].N[1] = fi->rho * fi->u;
        Q_C[gid].N[2] = fi->rho * fi->v;
        Q_C[gid].N[3] = fi->rho * fi->w;
        Q_C[gid].N[4] = ((fi->p / 0.4) + ke);
    }
}

/* ------------------------------------------------------------ Viscous ---- */

/* One-sided / biased / central first derivative along one direction, with the
 * branch order of Viscous.cl:285-332 (later branches override earlier ones).
 * f[o+3], o=-3..3.  Cases the reference leaves undefined (no branch taken)
 * return 0 here. */
static double visc_deriv(const double f[7], const int L[7])
{
    const int L0 = L[3];
    double D = g_poison ? NAN : 0.0;
    if (L0 > 0 && L0 <= 52 && L[4] == 100)
        D = (1.0 / 6.0) * (11.0 * f[3] - 18.0 * f[2] + 9.0 * f[1] - 2.0 * f[0]);
    if (L0 > 0 && L0 <= 52 && L[2] == 100)
        D = (1.0 / 6.0) * (-11.0 * f[3] + 18.0 * f[4] - 9.0 * f[5] + 2.0 * f[6]);
    if (L0 == 0 && L[4] > 0 && L[4] <= 52 && L[5] == 100)
        D = (1.0 / 6.0) * (2.0 * f[4] + 3.0 * f[3] - 6.0 * f[2] + f[1]);
    if (L0 == 0 && L[2] > 0 && L[2] && L[1] == 100)
        D = (1.0 / 6.0) * ((-2.0) * f[2] - 3.0 * f[3] + 6.0 * f[4] - f[5]);
    if (L0 == 0 && L[1] != 100 && L[2] != 100 && L[5] != 100 && L[4] != 100)
        D = (1.0 / 12.0) * (8.0 * (f[4] - f[2]) - (f[5] - f[1]));
    if (L0 > 0 && L[1] != 100 && L[2] != 100 && L[5] != 100 && L[4] != 100)
        D = (1.0 / 12.0) * (8.0 * (f[4] - f[2]) - (f[5] - f[1]));
    return D;
}

/* Viscous.cl:23-643. */
void oracle_viscous(int n_items, const or_params *prm, const or_col5 *U_C,
                    or_col5 *F, or_col5 *E, or_col5 *G, or_col5 *Fv, or_col5 *Ev, or_col5 *Gv,
                    const or_grid *grid, const or_metric *metric, const double *det, or_flow *flow)
{
    const double Mach = prm->mach, Reyl = prm->reynolds, Pr = prm->prandtl, Free_t = prm->t_inf;
#pragma omp parallel for schedule(static) num_threads(oracle_get_threads())
    for (int gid = 0; gid < n_items; ++gid) {
        int idx[3][7], loc[3][7];
        gather_star(grid, gid, idx, loc);
        const double *m = metric[gid].m;
        const double DET_I = det[gid];
        const double zeta_x = m[0], zeta_y = m[1], zeta_z = m[2];
        const double eta_x = m[3], eta_y = m[4], eta_z = m[5];
        const double xi_x = m[6], xi_y = m[7], xi_z = m[8];
        const or_flow fl = flow[gid];

        /* dU[d][c]: derivative of component c along direction d. */
        double dU[3][5];
        for (int d = 0; d < 3; ++d)
            for (int c = 0; c < 5; ++c) {
                double f[7];
                for (int o = 0; o < 7; ++o) f[o] = U_C[idx[d][o]].N[c];
                dU[d][c] = visc_deriv(f, loc[d]);
            }
        const double U0_I = U_C[gid].N[0], U1_I = U_C[gid].N[1], U2_I = U_C[gid].N[2];
        const double U3_I = U_C[gid].N[3], U4_I = U_C[gid].N[4];

        /* Viscous.cl:439-453: quotient-rule velocity and internal-energy
         * gradients in computational space. */
        double uc[3], vc[3], wc[3], tc[3];
        for (int d = 0; d < 3; ++d) {
            uc[d] = (1.0 / U0_I) * (dU[d][1]) - (U1_I / ((U0_I * U0_I))) * (dU[d][0]);
            vc[d] = (1.0 / U0_I) * (dU[d][2]) - (U2_I / ((U0_I * U0_I))) * (dU[d][0]);
            wc[d] = (1.0 / U0_I) * (dU[d][3]) - (U3_I / ((U0_I * U0_I))) * (dU[d][0]);
        }
        for (int d = 0; d < 3; ++d)
            tc[d] = (1.0 / U0_I) * (dU[d][4]) - (U4_I / ((U0_I * U0_I))) * (dU[d][0]) - (U1_I / U0_I) * uc[d]
                    - (U2_I / U0_I) * vc[d] - (U3_I / U0_I) * wc[d];

        /* Viscous.cl:455-458: Sutherland's law. */
        const double d_temp = (1.4 * Mach * Mach * 0.4 * ((U4_I / U0_I) - 0.5 * (((U1_I * U1_I) / (U0_I * U0_I)) + ((U2_I * U2_I) / (U0_I * U0_I)) + ((U3_I * U3_I) / (U0_I * U0_I)))));
        const double d_temp1 = sqrt(d_temp) * sqrt(d_temp) * sqrt(d_temp);
        const double mu = (d_temp1) * ((1.0 + (110.4 / Free_t)) / (d_temp + (110.4 / Free_t)));

        /* Cartesian gradients: f_x = f_zeta*zeta_x + f_eta*eta_x + f_xi*xi_x. */
#define GX(a) ((a)[0] * zeta_x + (a)[1] * eta_x + (a)[2] * xi_x)
#define GY(a) ((a)[0] * zeta_y + (a)[1] * eta_y + (a)[2] * xi_y)
#define GZ(a) ((a)[0] * zeta_z + (a)[1] * eta_z + (a)[2] * xi_z)
        /* Viscous.cl:461-463 heat flux. */
        const double qz = (-1.0) * (mu * 1.4 / (Pr * Reyl)) * GX(tc);
        const double qe = (-1.0) * (mu * 1.4 / (Pr * Reyl)) * GY(tc);
        const double qx = (-1.0) * (mu * 1.4 / (Pr * Reyl)) * GZ(tc);
        /* Viscous.cl:466-476 Stokes stresses. */
        const double tauzz = (mu / Reyl) * ((4.0 / 3.0) * GX(uc) - (2.0 / 3.0) * GY(vc) - (2.0 / 3.0) * GZ(wc));
        const double tauee = (mu / Reyl) * ((4.0 / 3.0) * GY(vc) - (2.0 / 3.0) * GX(uc) - (2.0 / 3.0) * GZ(wc));
        const double tauxx = (mu / Reyl) * ((4.0 / 3.0) * GZ(wc) - (2.0 / 3.0) * GX(uc) - (2.0 / 3.0) * GY(vc));
        const double s_xy = uc[0] * zeta_y + uc[1] * eta_y + uc[2] * xi_y + vc[0] * zeta_x + vc[1] * eta_x + vc[2] * xi_x;
        const double s_xz = uc[0] * zeta_z + uc[1] * eta_z + uc[2] * xi_z + wc[0] * zeta_x + wc[1] * eta_x + wc[2] * xi_x;
        const double s_yz = vc[0] * zeta_z + vc[1] * eta_z + vc[2] * xi_z + wc[0] * zeta_y + wc[1] * eta_y + wc[2] * xi_y;
        const double tauze = (mu / Reyl) * s_xy;
        const double tauzx = (mu / Reyl) * s_xz;
        const double tauex = (mu / Reyl) * s_yz;

        /* Viscous.cl:490-558: mixed-time-scale SGS model (C=0.03, C_T=10),
         * filter width 1/cbrt(det), test filter (1/4,1/2,1/4) per direction. */
        double TAU_XY = 0, TAU_YZ = 0, TAU_XZ = 0, TAU_XX = 0, TAU_YY = 0, TAU_ZZ = 0;
        double H_X = 0, H_Y = 0, H_Z = 0, D_X = 0, D_Y = 0, D_Z = 0;
        if (prm->les) {
            const double C_MTS = 0.03, C_T = 10.0;
            const or_col5 *Ui = &U_C[gid];
            const double KS_x = sq(((U1_I / U0_I) - ((0.25 * U_C[idx[0][2]].N[1] + 0.5 * Ui->N[1] + 0.25 * U_C[idx[0][4]].N[1]) / (0.25 * U_C[idx[0][2]].N[0] + 0.5 * U0_I + 0.25 * U_C[idx[0][4]].N[0]))));
            const double KS_y = sq(((U2_I / U0_I) - ((0.25 * U_C[idx[1][2]].N[2] + 0.5 * Ui->N[2] + 0.25 * U_C[idx[1][4]].N[2]) / (0.25 * U_C[idx[1][2]].N[0] + 0.5 * U0_I + 0.25 * U_C[idx[1][4]].N[0]))));
            const double KS_z = sq(((U3_I / U0_I) - ((0.25 * U_C[idx[2][2]].N[3] + 0.5 * Ui->N[3] + 0.25 * U_C[idx[2][4]].N[3]) / (0.25 * U_C[idx[2][2]].N[0] + 0.5 * U0_I + 0.25 * U_C[idx[2][4]].N[0]))));
            const double stress_xy = (0.5 * s_xy);
            const double stress_yz = (0.5 * (vc[0] * zeta_z + vc[1] * eta_z + vc[2] * xi_z + wc[0] * zeta_y + wc[1] * eta_y + wc[2] * xi_y));
            const double stress_xz = (0.5 * (wc[0] * zeta_x + wc[1] * eta_x + wc[2] * xi_x + uc[0] * zeta_z + uc[1] * eta_z + uc[2] * xi_z));
            const double stress_xx = GX(uc), stress_yy = GY(vc), stress_zz = GZ(wc);
            const double mod_stress = sqrt(2.0 * ((stress_xy * stress_xy + stress_yz * stress_yz + stress_xz * stress_xz) + (2.0 / 3.0) * (stress_xx * stress_xx + stress_yy * stress_yy + stress_zz * stress_zz)));
            const double DEL = (1.0 / cbrt(DET_I));
            double EDDY_x, EDDY_y, EDDY_z;
            if (prm->les == 2) {
                /* Smagorinsky, a builder addition (the reference implements only
                 * MTS): (C_s Delta)^2 |S|, |S| = sqrt(2 S_ij S_ij), isotropic,
                 * Delta = det^(1/3) (det is the cell volume). */
                const double S = sqrt(2.0 * (stress_xx * stress_xx + stress_yy * stress_yy + stress_zz * stress_zz)
                                      + 4.0 * (stress_xy * stress_xy + stress_yz * stress_yz + stress_xz * stress_xz));
                const double ls = prm->smagorinsky_cs * cbrt(DET_I);
                EDDY_x = EDDY_y = EDDY_z = (ls * ls) * S;
            } else if (mod_stress != 0.0) {
                const double Rx = (DEL * (mod_stress)) / sqrt(KS_x);
                const double Ry = (DEL * (mod_stress)) / sqrt(KS_y);
                const double Rz = (DEL * (mod_stress)) / sqrt(KS_z);
                EDDY_x = (C_MTS / (1.0 + (1.0 * Rx / (C_T)))) * DEL * sqrt(KS_x);
                EDDY_y = (C_MTS / (1.0 + (1.0 * Ry / (C_T)))) * DEL * sqrt(KS_y);
                EDDY_z = (C_MTS / (1.0 + (1.0 * Rz / (C_T)))) * DEL * sqrt(KS_z);
            } else {
                EDDY_x = (C_MTS) * DEL * sqrt(KS_x);
                EDDY_y = (C_MTS) * DEL * sqrt(KS_y);
                EDDY_z = (C_MTS) * DEL * sqrt(KS_z);
            }
            TAU_XY = -2.0 * U0_I * EDDY_x * (0.5 * s_xy);
            TAU_YZ = -2.0 * U0_I * EDDY_y * (stress_yz);
            TAU_XZ = -2.0 * U0_I * EDDY_z * (stress_xz);
            TAU_XX = -2.0 * U0_I * EDDY_x * stress_xx;
            TAU_YY = -2.0 * U0_I * EDDY_y * stress_yy;
            TAU_ZZ = -2.0 * U0_I * EDDY_z * stress_zz;
            const double Q_x = (1.0 / (1.4 * 0.4 * Mach * Mach)) * (-1.0) * (EDDY_x) * GX(tc);
            const double Q_y = (1.0 / (1.4 * 0.4 * Mach * Mach)) * (-1.0) * (EDDY_y) * GY(tc);
            const double Q_z = (1.0 / (1.4 * 0.4 * Mach * Mach)) * (-1.0) * (EDDY_z) * GZ(tc);
            const double DEL_X = TAU_XX * fl.u + TAU_XY * fl.u + TAU_XZ * fl.u;
            const double DEL_Y = TAU_XY * fl.v + TAU_YY * fl.v + TAU_YZ * fl.v;
            const double DEL_Z = TAU_XZ * fl.w + TAU_YZ * fl.w + TAU_ZZ * fl.w;
            H_X = Q_x + DEL_X;
            H_Y = Q_y + DEL_Y;
            H_Z = Q_z + DEL_Z;
            D_X = 0.4 * Q_x;
            D_Y = 0.4 * Q_y;
            D_Z = 0.4 * Q_z;
        }
#undef GX
#undef GY
#undef GZ

        /* Viscous.cl:560-613: Cartesian node fluxes from the primitives. */
        const double rho = fl.rho, u = fl.u, v = fl.v, w = fl.w, p = fl.p;
        const double Et = (((p / 0.4) + 0.5 * rho * (u * u + v * v + w * w)) + p);
        double tF[5] = {rho * u, rho * u * u + p, rho * v * u, rho * u * w, Et * u};
        double tE[5] = {rho * v, rho * v * u, rho * v * v + p, rho * v * w, Et * v};
        double tG[5] = {rho * w, rho * u * w, rho * v * w, rho * w * w + p, Et * w};
        double tFv[5] = {0.0, (-1.0) * tauzz + TAU_XX, (-1.0) * tauze + TAU_XY, (-1.0) * tauzx + TAU_XZ,
                         (((-1.0) * u * tauzz - v * tauze - w * tauzx) + qz + H_X + D_X)};
        double tEv[5] = {0.0, (-1.0) * tauze + TAU_XY, (-1.0) * tauee + TAU_YY, (-1.0) * tauex + TAU_YZ,
                         (((-1.0) * u * tauze - v * tauee - w * tauex) + qe + H_Y + D_Y)};
        double tGv[5] = {0.0, (-1.0) * tauzx + TAU_XZ, (-1.0) * tauex + TAU_YZ, (-1.0) * tauxx + TAU_ZZ,
                         (((-1.0) * u * tauzx - v * tauex - w * tauxx) + qx + H_Z + D_Z)};
        /* Viscous.cl:615-631: contravariant projection with the node metric. */
        for (int c = 0; c < 5; ++c) {
            F[gid].N[c] = DET_I * (zeta_x * tF[c] + zeta_y * tE[c] + zeta_z * tG[c]);
            E[gid].N[c] = DET_I * (eta_x * tF[c] + eta_y * tE[c] + eta_z * tG[c]);
            G[gid].N[c] = DET_I * (xi_x * tF[c] + xi_y * tE[c] + xi_z * tG[c]);
            if (prm->viscous) {
                Fv[gid].N[c] = DET_I * (zeta_x * tFv[c] + zeta_y * tEv[c] + zeta_z * tGv[c]);
                Ev[gid].N[c] = DET_I * (eta_x * tFv[c] + eta_y * tEv[c] + eta_z * tGv[c]);
                Gv[gid].N[c] = DET_I * (xi_x * tFv[c] + xi_y * tEv[c] + xi_z * tGv[c]);
            } else {
                Fv[gid].N[c] = 0.0;
                Ev[gid].N[c] = 0.0;
                Gv[gid].N[c] = 0.0;
            }
        }
        /* Viscous.cl:633-641: only mu changes in FLOW. */
        flow[gid].mu = mu;
    }
}

/* --------------------------------------------------------------- Weno ---- */

/* Viscous-flux derivative branches of Weno.cl:2732-2856.  Weno.cl has no
 * branch for a boundary node (0 < loc <= 52) away from ghosts in this
 * direction (the reference leaves the value uninitialised there); this
 * restatement uses the 4th-order central form of Viscous.cl:325-332 for it. */
static double weno_visc_deriv(const double f[7], const int L[7], int *defined)
{
    const int L0 = L[3];
    double D = 0.0;
    int set = 0;
    if (L0 > 0 && L0 <= 52 && L[4] == 100) {
        D = (1.0 / 6.0) * (11.0 * f[3] - 18.0 * f[2] + 9.0 * f[1] - 2.0 * f[0]);
        set = 1;
    }
    if (L0 > 0 && L0 <= 52 && L[2] == 100) {
        D = (1.0 / 6.0) * (-11.0 * f[3] + 18.0 * f[4] - 9.0 * f[5] + 2.0 * f[6]);
        set = 1;
    }
    if (L0 == 0 && L[4] > 0 && L[4] <= 52 && L[5] == 100) {
        D = (1.0 / 6.0) * ((2.0) * f[4] + 3.0 * f[3] - 6.0 * f[2] + f[1]);
        set = 1;
    }
    if (L0 == 0 && L[2] > 0 && L[2] <= 52 && L[1] == 100) {
        D = (1.0 / 6.0) * ((-2.0) * f[2] - 3.0 * f[3] + 6.0 * f[4] - f[5]);
        set = 1;
    }
    if (L0 == 0 && L[1] != 100 && L[2] != 100 && L[5] != 100 && L[4] != 100) {
        D = (1.0 / 12.0) * (8.0 * (f[4] - f[2]) - (f[5] - f[1]));
        set = 1;
    }
    if (!set) D = g_poison ? NAN : (1.0 / 12.0) * (8.0 * (f[4] - f[2]) - (f[5] - f[1]));
    if (defined) *defined = set;
    return D;
}

/* Cartesian Euler fluxes of a face state, Weno.cl:2291-2507. */
static void cart_flux(const double q[5], double F[5], double E[5], double G[5])
{
    const double k1 = (q[1] * q[1] / q[0]), k2 = (q[2] * q[2] / q[0]), k3 = (q[3] * q[3] / q[0]);
    const double pr = 0.4 * (q[4] - 0.5 * (k1 + k2 + k3));
    const double hq = (1.4 * q[4] - 0.2 * (k1 + k2 + k3));
    F[0] = q[1];
    F[1] = k1 + pr;
    F[2] = (q[1] * q[2]) / q[0];
    F[3] = (q[1] * q[3]) / q[0];
    F[4] = hq * (q[1] / q[0]);
    E[0] = q[2];
    E[1] = (q[1] * q[2]) / q[0];
    E[2] = k2 + pr;
    E[3] = (q[2] * q[3]) / q[0];
    E[4] = hq * (q[2] / q[0]);
    G[0] = q[3];
    G[1] = (q[1] * q[3]) / q[0];
    G[2] = (q[2] * q[3]) / q[0];
    G[3] = k3 + pr;
    G[4] = hq * (q[3] / q[0]);
}

/* Largest eigenvalue U.grad(zeta) + c|grad(zeta)| of a face state, with the
 * un-normalised face metric (Weno.cl:2511-2583, element [4]). */
static double lambda5(const double q[5], double mx, double my, double mz)
{
    return (mx * (q[1] / q[0]) + my * (q[2] / q[0]) + mz * (q[3] / q[0]))
           + sqrt(1.4 * 0.4 * ((q[4] / q[0]) - ((q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) / (2.0 * (q[0] * q[0])))) * (mx * mx + my * my + mz * mz));
}

/* WENO5 nonlinear interpolation of one characteristic variable to a
 * half point (Weno.cl:1056-1280).  c[o+3] for o=-3..3; off = 0 for the
 * i+1/2 face, -1 for the i-1/2 face.  Returns the right-biased ("pos")
 * and left-biased ("neg") values. */
static void weno_pair(const double *cc, int off, double eps, double *pos, double *neg)
{
    const double *c = cc + 3 + off;  /* c[0] is the left node of the face */
    double p0 = (15.0 / 8.0) * c[1] - (5.0 / 4.0) * c[2] + (3.0 / 8.0) * c[3];
    double p1 = (3.0 / 8.0) * c[0] + (3.0 / 4.0) * c[1] - (1.0 / 8.0) * c[2];
    double p2 = (-1.0 / 8.0) * c[-1] + (3.0 / 4.0) * c[0] + (3.0 / 8.0) * c[1];
    double m0 = (3.0 / 8.0) * c[0] + (3.0 / 4.0) * c[1] - (1.0 / 8.0) * c[2];
    double m1 = (-1.0 / 8.0) * c[-1] + (3.0 / 4.0) * c[0] + (3.0 / 8.0) * c[1];
    double m2 = (3.0 / 8.0) * c[-2] - (5.0 / 4.0) * c[-1] + (15.0 / 8.0) * c[0];

    double ISm2 = (13.0 / 12.0) * (sq(c[-2] - 2.0 * c[-1] + c[0])) + (1.0 / 4.0) * (sq(c[-2] - 4.0 * c[-1] + 3.0 * c[0]));
    double ISm1 = (13.0 / 12.0) * (sq(c[-1] - 2.0 * c[0] + c[1])) + (1.0 / 4.0) * (sq(c[-1] - c[1]));
    double ISm0 = (13.0 / 12.0) * (sq(c[0] - 2.0 * c[1] + c[2])) + (1.0 / 4.0) * (sq(3.0 * c[0] - 4.0 * c[1] + c[2]));
    double ISp2 = (13.0 / 12.0) * (sq(c[-1] - 2.0 * c[0] + c[1])) + (1.0 / 4.0) * (sq(c[-1] - 4.0 * c[0] + 3.0 * c[1]));
    double ISp1 = (13.0 / 12.0) * (sq(c[0] - 2.0 * c[1] + c[2])) + (1.0 / 4.0) * (sq(c[0] - c[2]));
    double ISp0 = (13.0 / 12.0) * (sq(c[1] - 2.0 * c[2] + c[3])) + (1.0 / 4.0) * (sq(3.0 * c[1] - 4.0 * c[2] + c[3]));

    double wp0 = (1.0 / 16.0) / (sq(eps + (ISp0)));
    double wp1 = (5.0 / 8.0) / (sq(eps + (ISp1)));
    double wp2 = (5.0 / 16.0) / (sq(eps + (ISp2)));
    double wm0 = (5.0 / 16.0) / (sq(eps + (ISm0)));
    double wm1 = (5.0 / 8.0) / (sq(eps + (ISm1)));
    double wm2 = (1.0 / 16.0) / (sq(eps + (ISm2)));

    double Wp0 = wp0 / (wp0 + wp1 + wp2), Wp1 = wp1 / (wp0 + wp1 + wp2), Wp2 = wp2 / (wp0 + wp1 + wp2);
    double Wm0 = wm0 / (wm0 + wm1 + wm2), Wm1 = wm1 / (wm0 + wm1 + wm2), Wm2 = wm2 / (wm0 + wm1 + wm2);
    *pos = Wp0 * p0 + Wp1 * p1 + Wp2 * p2;
    *neg = Wm0 * m0 + Wm1 * m1 + Wm2 * m2;
}

/* One face (direction d, side s: 0 = +1/2, 1 = -1/2) of node gid: Roe
 * eigenvectors from the face metric (Weno.cl:336-1051), characteristic
 * projection of the 7-point stencil, WENO5 (1056-2186), back-projection
 * (2188-2289), Cartesian fluxes (2291-2507), lambda_5 (2509-2583),
 * contravariant projection x face det (2585-2728) and the LLF flux
 * (2859-2947).  Writes the LLF face flux into Fhat[5]. */
static void weno_face(int gid, int d, int s, const int *stencil, double eps,
                      const or_determ *deter, const or_col5 *Q_C, const or_metric *metric,
                      const or_roe *roe, double Fhat[5])
{
    const double *fm = &metric[gid].m[9 * (1 + 2 * d + s) + 3 * d];
    const double mx = fm[0], my = fm[1], mz = fm[2];
    const double *ra = &roe[gid].v[6 * (d + 3 * s)];
    const double ru = ra[0], rv = ra[1], rw = ra[2], rh = ra[4], rrho = ra[5];
    const double *dd = &deter[gid].ip;
    const double DET_F = dd[2 * d + s];

    const double kk = sqrt(mx * mx + my * my + mz * mz);
    const double a = sqrt(0.4 * (rh - 0.5 * (ru * ru + rv * rv + rw * rw)));
    const double kx = mx / kk, ky = my / kk, kz = mz / kk;
    const double theta = kx * ru + ky * rv + kz * rw;
    const double phi_sq = 0.5 * 0.4 * (ru * ru + rv * rv + rw * rw);
    const double alpha = rrho / (sqrt(2.0) * a);
    const double beta = 1.0 / (sqrt(2.0) * rrho * a);

    double R[5][5] = {
        {kx, ky, kz, alpha, alpha},
        {kx * ru, ky * ru - kz * rrho, kz * ru + ky * rrho, alpha * (ru + kx * a), alpha * (ru - kx * a)},
        {kx * rv + kz * rrho, ky * rv, kz * rv - kx * rrho, alpha * (rv + ky * a), alpha * (rv - ky * a)},
        {kx * rw - ky * rrho, ky * rw + kx * rrho, kz * rw, alpha * (rw + kz * a), alpha * (rw - kz * a)},
        {((kx * phi_sq) / 0.4) + rrho * (kz * rv - ky * rw), ((ky * phi_sq) / 0.4) + rrho * (kx * rw - kz * ru),
         ((kz * phi_sq) / 0.4) + rrho * (ky * ru - kx * rv), alpha * (((phi_sq + a * a) / (0.4)) + theta * a),
         alpha * (((phi_sq + a * a) / (0.4)) - theta * a)}};
    double Lm[5][5] = {
        {kx * (1.0 - (phi_sq / (a * a))) - ((kz * rv - ky * rw) / rrho), kx * 0.4 * ru / (a * a),
         (kx * 0.4 * rv / (a * a)) + (kz / rrho), (kx * 0.4 * rw / (a * a)) - (ky / rrho), -kx * 0.4 / (a * a)},
        {ky * (1.0 - (phi_sq / (a * a))) - ((kx * rw - kz * ru) / rrho), (ky * 0.4 * ru / (a * a)) - kz / rrho,
         ky * 0.4 * rv / (a * a), (ky * 0.4 * rw / (a * a)) + (kx / rrho), -ky * 0.4 / (a * a)},
        {kz * (1.0 - (phi_sq / (a * a))) - ((ky * ru - kx * rv) / rrho), kz * 0.4 * ru / (a * a) + (ky / rrho),
         kz * 0.4 * rv / (a * a) - (kx / rrho), kz * 0.4 * rw / (a * a), -kz * 0.4 / (a * a)},
        {beta * (phi_sq - theta * a), -beta * (0.4 * ru - kx * a), -beta * (0.4 * rv - ky * a),
         -beta * (0.4 * rw - kz * a), beta * 0.4},
        {beta * (phi_sq + theta * a), -beta * (0.4 * ru + kx * a), -beta * (0.4 * rv + ky * a),
         -beta * (0.4 * rw + kz * a), beta * 0.4}};

    /* characteristic values cv[r][o+3] of the 7 stencil points */
    double cv[5][7];
    for (int o = 0; o < 7; ++o) {
        const double *q = Q_C[stencil[o]].N;
        for (int r = 0; r < 5; ++r)
            cv[r][o] = Lm[r][0] * q[0] + Lm[r][1] * q[1] + Lm[r][2] * q[2] + Lm[r][3] * q[3] + Lm[r][4] * q[4];
    }
    double cpos[5], cneg[5];
    for (int r = 0; r < 5; ++r) weno_pair(cv[r], s == 0 ? 0 : -1, eps, &cpos[r], &cneg[r]);

    double qp[5], qn[5];
    for (int r = 0; r < 5; ++r) {
        qp[r] = R[r][0] * (cpos[0]) + R[r][1] * (cpos[1]) + R[r][2] * (cpos[2]) + R[r][3] * (cpos[3]) + R[r][4] * (cpos[4]);
        qn[r] = R[r][0] * (cneg[0]) + R[r][1] * (cneg[1]) + R[r][2] * (cneg[2]) + R[r][3] * (cneg[3]) + R[r][4] * (cneg[4]);
    }
    double Fp[5], Ep[5], Gp[5], Fn[5], En[5], Gn[5];
    cart_flux(qp, Fp, Ep, Gp);
    cart_flux(qn, Fn, En, Gn);
    const double lp = lambda5(qp, mx, my, mz);
    const double ln = lambda5(qn, mx, my, mz);
    double alpha_llf = NAN;
    if (fabs(lp) >= fabs(ln)) alpha_llf = fabs(lp);
    else if (fabs(ln) >= fabs(lp)) alpha_llf = fabs(ln);
    for (int c = 0; c < 5; ++c) {
        const double fcp = DET_F * (mx * Fp[c] + my * Ep[c] + mz * Gp[c]);
        const double fcn = DET_F * (mx * Fn[c] + my * En[c] + mz * Gn[c]);
        const double qpd = DET_F * qp[c], qnd = DET_F * qn[c];
        Fhat[c] = 0.5 * (fcp + fcn - alpha_llf * (qpd - qnd));
    }
}

/* Weno.cl:36-3137 for every Gid in [0, n_items). */
void oracle_weno(int n_items, int j, double mach, double del_t, const or_params *prm,
                 const or_determ *deter, const double *det,
                 or_col5 *U0, or_col5 *U1, or_col5 *U2, const or_grid *grid,
                 const or_col5 *Q_C, const or_metric *metric, const or_roe *roe,
                 const or_col5 *Fv, const or_col5 *Ev, const or_col5 *Gv,
                 const or_col5 *F, const or_col5 *E, const or_col5 *G,
                 or_flow *flow, or_col5 *L_out)
{
    const double eps = prm->weno_eps;
#pragma omp parallel for schedule(static) num_threads(oracle_get_threads())
    for (int gid = 0; gid < n_items; ++gid) {
        int idx[3][7], loc[3][7];
        gather_star(grid, gid, idx, loc);
        double dflux[3][5], dvis[3][5];
        for (int d = 0; d < 3; ++d) {
            double Fp[5], Fm[5];
            weno_face(gid, d, 0, idx[d], eps, deter, Q_C, metric, roe, Fp);
            weno_face(gid, d, 1, idx[d], eps, deter, Q_C, metric, roe, Fm);
            const or_col5 *NF = d == 0 ? F : (d == 1 ? E : G);
            const or_col5 *VF = d == 0 ? Fv : (d == 1 ? Ev : Gv);
            const int *ix = idx[d];
            for (int c = 0; c < 5; ++c) {
                /* Weno.cl:2950-3058 midpoint-and-node correction */
                const double f_3 = NF[ix[0]].N[c], f_2 = NF[ix[1]].N[c], f_1 = NF[ix[2]].N[c], f0 = NF[ix[3]].N[c];
                const double f1 = NF[ix[4]].N[c], f2 = NF[ix[5]].N[c], f3 = NF[ix[6]].N[c];
                const double d2p = (1.0 / 48.0) * (-5.0 * f_2 + 39.0 * f_1 - 34.0 * f0 - 34.0 * f1 + 39.0 * f2 - 5.0 * f3);
                const double d2m = (1.0 / 48.0) * (-5.0 * f_3 + 39.0 * f_2 - 34.0 * f_1 - 34.0 * f0 + 39.0 * f1 - 5.0 * f2);
                const double d4p = (1.0 / 2.0) * (f_2 - 3.0 * f_1 + 2.0 * f0 + 2.0 * f1 - 3.0 * f2 + f3);
                const double d4m = (1.0 / 2.0) * (f_3 - 3.0 * f_2 + 2.0 * f_1 + 2.0 * f0 - 3.0 * f1 + f2);
                const double hp = Fp[c] - (1.0 / 24.0) * d2p + (7.0 / 5760.0) * d4p;
                const double hm = Fm[c] - (1.0 / 24.0) * d2m + (7.0 / 5760.0) * d4m;
                dflux[d][c] = hp - hm;
                double fv[7];
                for (int o = 0; o < 7; ++o) fv[o] = VF[ix[o]].N[c];
                dvis[d][c] = weno_visc_deriv(fv, loc[d], NULL);
            }
        }
        double L[5];
        for (int c = 0; c < 5; ++c)
            L[c] = (-1.0) * (dflux[0][c] + dflux[1][c] + dflux[2][c] + dvis[0][c] + dvis[1][c] + dvis[2][c]);
        if (L_out) memcpy(L_out[gid].N, L, sizeof L);

        /* Weno.cl:3084-3126: Shu-Osher SSP-RK3 stage j. */
        double fu[5];
        if (j == 0) {
            for (int c = 0; c < 5; ++c) U1[gid].N[c] = U0[gid].N[c] + del_t * L[c];
            for (int c = 0; c < 5; ++c) fu[c] = (1.0 / det[gid]) * U1[gid].N[c];
        } else if (j == 1) {
            for (int c = 0; c < 5; ++c)
                U2[gid].N[c] = (3.0 / 4.0) * U0[gid].N[c] + (1.0 / 4.0) * U1[gid].N[c] + 0.25 * del_t * L[c];
            for (int c = 0; c < 5; ++c) fu[c] = (1.0 / det[gid]) * U2[gid].N[c];
        } else {
            for (int c = 0; c < 5; ++c)
                U0[gid].N[c] = (U0[gid].N[c] / 3.0) + ((2.0 / 3.0) * U2[gid].N[c]) + (2.0 / 3.0) * (del_t * L[c]);
            for (int c = 0; c < 5; ++c) fu[c] = (1.0 / det[gid]) * U0[gid].N[c];
        }
        /* Weno.cl:3128-3135: primitive recovery. */
        or_flow *fo = &flow[gid];
        fo->rho = fu[0];
        fo->u = fu[1] / fu[0];
        fo->v = fu[2] / fu[0];
        fo->w = fu[3] / fu[0];
        fo->e = (fu[4] / fu[0]) - 0.5 * (fo->u * fo->u + fo->v * fo->v + fo->w * fo->w);
        fo->p = fo->e * fo->rho * 0.4;
        fo->t = (1.4 * mach * mach) * (fo->p / fo->rho);
        fo->a = sqrt(1.4 * fo->p / fo->rho);
    }
}

/* -------------------------------------------------------- host loop ---- */

/* Solver.cpp:365-541 with the stage index passed per stage. */
void oracle_stage(or_case *c, const or_params *prm, int j, double del_t, or_col5 *L_out)
{
    or_col5 *Uj = j == 0 ? c->U0 : (j == 1 ? c->U1 : c->U2);
    const int n_all = c->g_node + 1, n_owned = c->sd_node + 1;
    oracle_uq(n_all, Uj, c->Q, c->grid, c->det, c->flow, c->roe);
    oracle_viscous(n_all, prm, Uj, c->F, c->E, c->G, c->Fv, c->Ev, c->Gv, c->grid, c->metric, c->det, c->flow);
    oracle_weno(n_owned, j, prm->mach, del_t, prm, c->deter, c->det, c->U0, c->U1, c->U2, c->grid, c->Q,
                c->metric, c->roe, c->Fv, c->Ev, c->Gv, c->F, c->E, c->G, c->flow, L_out);
}

void oracle_rk3_steps(or_case *c, const or_params *prm, double del_t, int nsteps)
{
    for (int n = 0; n < nsteps; ++n)
        for (int j = 0; j < 3; ++j) oracle_stage(c, prm, j, del_t, NULL);
}

/* ------------------------------------------------- boundary routine ---- */

/* Missing-neighbour slot l (towards the ghosts) and inward slot k of the
 * face boundary codes 1..6 (Flow_Initialisation.cpp:55-89): 1 no element
 * north (+j), 2 east (+i), 3 south (-j), 4 west (-i), 5 (-k), 6 (+k). */
static const int bc_face_l[7] = {-1, 0, 1, 2, 3, 5, 4};
static const int bc_face_k[7] = {-1, 2, 3, 0, 1, 4, 5};

/* Neighbour-slot chains from an edge or corner node (codes 7..26) to the
 * node it copies (Flow_Initialisation.cpp:139-340 and the same chains in the
 * inlet, boundary and wall sections); -1 ends a chain. */
static const int bc_edge_chain[20][3] = {
    {1, 5, 2}, {1, 4, 2}, {3, 4, 2}, {3, 5, 2}, {1, 5, 0}, {1, 4, 0}, {3, 4, 0}, {3, 5, 0},
    {5, 0, -1}, {1, 0, -1}, {4, 0, -1}, {3, 0, -1}, {5, 2, -1}, {1, 2, -1}, {4, 2, -1}, {3, 2, -1},
    {1, 5, -1}, {1, 4, -1}, {3, 4, -1}, {3, 5, -1}};

static inline int bc_nb(const or_grid *g, int r, int slot)
{
    const int32_t *N = &g[r].N0;
    return N[slot];
}

static inline void bc_derive_rho_e(or_flow *f, double mach)
{
    f->rho = (1.4 * mach * mach) * (f->p / f->t);
    f->e = f->p / (0.4 * f->rho);
}

/* the eight fields the routine copies between nodes (mu is never touched) */
static inline void bc_copy8(or_flow *dst, const or_flow *src)
{
    dst->u = src->u;
    dst->v = src->v;
    dst->w = src->w;
    dst->p = src->p;
    dst->rho = src->rho;
    dst->t = src->t;
    dst->a = src->a;
    dst->e = src->e;
}

enum { BC_OUTLET = 0, BC_INLET = 1, BC_BOUNDARY = 2, BC_WALL = 3 };

static int bc_wall_singular(const or_grid *g, int r)
{
    const int loc = g[r].loc;
    return loc == 29 || loc == 30 || (loc >= 33 && loc <= 56) || g[r].ID == 10;
}

/* neighbour slot s of row r in the singular table */
static inline int bc_sing(const int32_t *sing, int r, int s) { return sing[(size_t)r * 6 + s]; }

/* The wall rule of one node from source row s: zero velocity, p and t of s,
 * rho and e derived; a untouched (Flow_Initialisation.cpp:1194-1222). */
static void bc_wall_from(or_flow *F, int b, int s, double mach)
{
    or_flow *fb = &F[b];
    fb->u = 0.0;
    fb->v = 0.0;
    fb->w = 0.0;
    fb->p = F[s].p;
    fb->t = F[s].t;
    bc_derive_rho_e(fb, mach);
}

/* One mirror pass of the singular branches (:1242-1270, :1354-1382): the
 * three ghosts along slot l of wall node b take the three nodes along slot
 * k from the singular neighbour singular[b][k], velocity negated, and the
 * wall node's a. */
static void bc_singular_mirror(const or_grid *g, or_flow *F, const int32_t *sing, int b, int l, int k)
{
    int gr = b, sr = -1;
    for (int m = 0; m < 3; ++m) {
        gr = bc_nb(g, gr, l);
        sr = m == 0 ? bc_sing(sing, b, k) : bc_nb(g, sr, k);
        or_flow *fg = &F[gr];
        const or_flow *fs = &F[sr];
        fg->u = (-1.0) * fs->u;
        fg->v = (-1.0) * fs->v;
        fg->w = (-1.0) * fs->w;
        fg->p = fs->p;
        fg->rho = fs->rho;
        fg->t = fs->t;
        fg->a = F[b].a;
        fg->e = fs->e;
    }
}

/* The passes (l = ghost slot, k = singular slot) of the codes 33..52
 * (:1285-1342): 33..36 and 41..44 and 49..52 take two, 37..40 and 45..48
 * three.  Returns the number of passes written to lk. */
static int bc_multi_pass(int loc, int lk[3][2])
{
    int n = 0;
    if ((loc >= 33 && loc <= 40)) { lk[n][0] = 2; lk[n][1] = 0; ++n; }
    else if (loc >= 41 && loc <= 48) { lk[n][0] = 0; lk[n][1] = 2; ++n; }
    else if (loc == 49 || loc == 52) { lk[n][0] = 5; lk[n][1] = 4; ++n; }
    else { lk[n][0] = 4; lk[n][1] = 5; ++n; }   /* 50, 51 */
    if (loc == 33 || loc == 43 || loc == 51 || loc == 52 || loc == 39 || loc == 40 || loc == 47 || loc == 48) {
        lk[n][0] = 3; lk[n][1] = 1;
    } else if (loc == 35 || loc == 41 || loc == 49 || loc == 50 || loc == 37 || loc == 38 || loc == 45 || loc == 46) {
        lk[n][0] = 1; lk[n][1] = 3;
    } else if (loc == 34 || loc == 44) {
        lk[n][0] = 5; lk[n][1] = 4;
    } else {   /* 36, 42 */
        lk[n][0] = 4; lk[n][1] = 5;
    }
    ++n;
    if ((loc >= 37 && loc <= 40) || (loc >= 45 && loc <= 48)) {
        if (loc == 37 || loc == 40 || loc == 48 || loc == 45) { lk[n][0] = 5; lk[n][1] = 4; }
        else { lk[n][0] = 4; lk[n][1] = 5; }
        ++n;
    }
    return n;
}

/* The singular-node branches of one wall node, after its face or edge rule
 * (Flow_Initialisation.cpp:1194-1392): codes 29 and 30 (in the routine's
 * chain of codes) from the node beyond singular[b][3]; ID 10 (other codes)
 * the node from singular[b][3] and three mirror passes; codes 33..52 the
 * node from singular[b][0], then per pass the node from singular[b][k] and
 * a mirror pass. */
static void bc_wall_singular_branches(const or_grid *g, or_flow *F, const int32_t *sing, int b, double mach)
{
    const int loc = g[b].loc;
    if (loc == 29 || loc == 30) bc_wall_from(F, b, bc_nb(g, bc_sing(sing, b, 3), loc == 29 ? 4 : 5), mach);
    if (g[b].ID == 10 && loc != 29 && loc != 30) {
        static const int lk10[3][2] = {{2, 0}, {0, 2}, {1, 3}};
        bc_wall_from(F, b, bc_sing(sing, b, 3), mach);
        for (int h = 0; h < 3; ++h) bc_singular_mirror(g, F, sing, b, lk10[h][0], lk10[h][1]);
    }
    if (loc >= 33 && loc <= 52) {
        int lk[3][2];
        const int n = bc_multi_pass(loc, lk);
        bc_wall_from(F, b, bc_sing(sing, b, 0), mach);
        for (int h = 0; h < n; ++h) {
            bc_wall_from(F, b, bc_sing(sing, b, lk[h][1]), mach);
            bc_singular_mirror(g, F, sing, b, lk[h][0], lk[h][1]);
        }
    }
}

/* One list of the routine, visited in order (Flow_Initialisation.cpp:50-342
 * outlet, 343-624 inlet, 625-909 boundary, 910-1394 wall). */
static void bc_list(int type, const or_grid *g, or_flow *F, const int32_t *rows, int n, double mach,
                    const int32_t *sing)
{
    for (int q = 0; q < n; ++q) {
        const int b = rows[q];
        const int loc = g[b].loc;
        if (loc >= 1 && loc <= 6) {
            const int l = bc_face_l[loc], k = bc_face_k[loc];
            const int g1 = bc_nb(g, b, l), g2 = bc_nb(g, g1, l), g3 = bc_nb(g, g2, l);
            const int s1 = bc_nb(g, b, k), s2 = bc_nb(g, s1, k), s3 = bc_nb(g, s2, k);
            or_flow *fb = &F[b];
            if (type == BC_OUTLET) {          /* :92-137 */
                fb->u = F[s1].u;
                fb->v = F[s1].v;
                fb->w = F[s1].w;
                fb->p = F[s1].p;
                fb->t = F[s1].t;
                bc_derive_rho_e(fb, mach);
                fb->a = sqrt(1.4 * fb->p / fb->rho);
                bc_copy8(&F[g1], fb);
                bc_copy8(&F[g2], fb);
                bc_copy8(&F[g3], fb);
            } else if (type == BC_INLET) {    /* :385-419 */
                fb->u = 1.0;
                fb->v = 0.0;
                fb->w = 0.0;
                fb->p = 1.0 / (1.4 * mach * mach);
                fb->t = 1.0;
                bc_derive_rho_e(fb, mach);
                fb->a = sqrt(1.4 * fb->p / fb->rho);
                bc_copy8(&F[g1], fb);
                bc_copy8(&F[g2], fb);
                bc_copy8(&F[g3], fb);
            } else if (type == BC_BOUNDARY) { /* :667-704 */
                bc_copy8(fb, &F[s1]);
                bc_copy8(&F[g1], &F[s1]);
                bc_copy8(&F[g2], &F[s2]);
                bc_copy8(&F[g3], &F[s3]);
            } else {                          /* :953-990 */
                fb->u = 0.0;
                fb->v = 0.0;
                fb->w = 0.0;
                fb->p = F[s1].p;
                fb->t = F[s1].t;
                bc_derive_rho_e(fb, mach);
                fb->a = sqrt(1.4 * fb->p / fb->rho);
                const int gs[3] = {g1, g2, g3}, ss[3] = {s1, s2, s3};
                for (int m = 0; m < 3; ++m) {
                    or_flow *fg = &F[gs[m]];
                    const or_flow *fs = &F[ss[m]];
                    fg->u = (-1.0) * fs->u;
                    fg->v = (-1.0) * fs->v;
                    fg->w = (-1.0) * fs->w;
                    fg->p = fs->p;
                    fg->rho = fs->rho;
                    fg->t = fs->t;
                    fg->a = fs->a;
                    fg->e = fs->e;
                }
            }
        } else if (loc >= 7 && loc <= 26) {
            const int *ch = bc_edge_chain[loc - 7];
            int s = b;
            for (int m = 0; m < 3 && ch[m] >= 0; ++m) s = bc_nb(g, s, ch[m]);
            or_flow *fb = &F[b];
            if (type == BC_WALL) {
                fb->u = 0.0;
                fb->v = 0.0;
                fb->w = 0.0;
            } else {
                fb->u = F[s].u;
                fb->v = F[s].v;
                fb->w = F[s].w;
            }
            fb->p = F[s].p;
            fb->t = F[s].t;
            bc_derive_rho_e(fb, mach);
        }
        /* other codes: the routine has no branch for them */
        if (type == BC_WALL && sing && bc_wall_singular(g, b)) bc_wall_singular_branches(g, F, sing, b, mach);
    }
}

int oracle_boundary_fill(const or_grid *grid, or_flow *flow, const or_bc_lists *bc, double mach, int initial,
                         int sd_node)
{
    for (int q = 0; q < bc->n_wall; ++q) {
        const int r = bc->wall[q], loc = grid[r].loc;
        if (bc_wall_singular(grid, r) && (!bc->singular || (loc >= 53 && loc <= 56))) return -1;
    }
    if (initial == 0) {   /* Flow_Initialisation.cpp:35-48 */
        for (int r = 1; r <= sd_node; ++r) {
            or_flow *f = &flow[r];
            f->u = 1.0;
            f->v = 0.0;
            f->w = 0.0;
            f->p = 1.0 / (1.4 * mach * mach);
            f->t = 1.0;
            f->rho = (1.4 * mach * mach) * (f->p / f->t);
            f->e = f->p / (0.4 * f->rho);
            f->a = sqrt(1.4 * f->p / f->rho);
        }
    }
    bc_list(BC_OUTLET, grid, flow, bc->outlet, bc->n_outlet, mach, NULL);
    bc_list(BC_INLET, grid, flow, bc->inlet, bc->n_inlet, mach, NULL);
    bc_list(BC_BOUNDARY, grid, flow, bc->boundary, bc->n_boundary, mach, NULL);
    bc_list(BC_WALL, grid, flow, bc->wall, bc->n_wall, mach, bc->singular);
    /* Solver.cpp:660-683: the tips after the routine, from their slot-3 node */
    for (int q = 0; q < bc->n_tips; ++q) bc_wall_from(flow, bc->tips[q], bc_nb(grid, bc->tips[q], 3), mach);
    return 0;
}

/* Solver.cpp:364-658: the boundary routine after every stage. */
int oracle_rk3_steps_bc(or_case *c, const or_params *prm, double del_t, int nsteps, const or_bc_lists *bc)
{
    for (int n = 0; n < nsteps; ++n)
        for (int j = 0; j < 3; ++j) {
            oracle_stage(c, prm, j, del_t, NULL);
            if (bc && oracle_boundary_fill(c->grid, c->flow, bc, prm->mach, 1, c->sd_node) != 0) return -1;
        }
    return 0;
}

/* ------------------------------------------------------ geometry producer */

/* neighbour slot s of row r (0 = none) */
static int nb(const or_grid *g, int r, int s)
{
    switch (s) {
    case 0: return g[r].N0;
    case 1: return g[r].N1;
    case 2: return g[r].N2;
    case 3: return g[r].N3;
    case 4: return g[r].N4;
    default: return g[r].N5;
    }
}

/* coordinate c (0 x, 1 y, 2 z) of row r */
static double crd(const or_grid *g, int r, int c) { return c == 0 ? g[r].x : (c == 1 ? g[r].y : g[r].z); }

/* One line of Grid_Transformation.cpp:29-204 (zeta; the eta and xi blocks
 * are the same with other slots): tridiagonal rows a/d/b and right-hand
 * sides c[3] along the line from `start` (no + neighbour, slot P) through the
 * - neighbours (slot Mn), then the reference's elimination from the far end
 * and substitution from `start`.  J[row*3 + c] receives d x_c / d dir. */
static int compact_line(const or_grid *g, int start, int P, int Mn, double dz, int n_rows, double *J,
                        double *a, double *b, double *dd, double *cc, double *dp, double *cp)
{
    int i = start, step = 0;
    while (i != 0) {
        if (step >= n_rows) return -1;   /* a closed chain: not a line */
        const int p1 = nb(g, i, P), p2 = nb(g, p1, P), p3 = nb(g, p2, P), p4 = nb(g, p3, P), p5 = nb(g, p4, P);
        const int m1 = nb(g, i, Mn), m2 = nb(g, m1, Mn), m3 = nb(g, m2, Mn), m4 = nb(g, m3, Mn), m5 = nb(g, m4, Mn);
        for (int c = 0; c < 3; ++c) {
            double *rhs = cc + 3 * step + c;
            if (step > 1) {   /* interior: alpha = 1/3, 7/9 and 1/36 (:46-52) */
                b[step] = 1.0 / 3.0;
                dd[step] = 1.0;
                a[step] = 1.0 / 3.0;
                *rhs = (1.0 / dz) * ((-1.0 / 36.0) * crd(g, m2, c) - (7.0 / 9.0) * crd(g, m1, c)
                                     + (7.0 / 9.0) * crd(g, p1, c) + (1.0 / 36.0) * crd(g, p2, c));
            }
            if (step == 0 && p1 == 0) {   /* the + end (:55-62) */
                b[step] = 5.0;
                dd[step] = 1.0;
                a[step] = 0.0;
                *rhs = (1.0 / dz) * ((197.0 / 60.0) * crd(g, i, c) + (5.0 / 12.0) * crd(g, m1, c) - (5.0) * crd(g, m2, c)
                                     + (5.0 / 3.0) * crd(g, m3, c) - (5.0 / 12.0) * crd(g, m4, c)
                                     + (1.0 / 20.0) * crd(g, m5, c));
            }
            if (step == 1) {   /* next to the + end (:63-70) */
                b[step] = 2.0 / 11.0;
                dd[step] = 1.0;
                a[step] = 2.0 / 11.0;
                *rhs = (1.0 / dz) * ((20.0 / 33.0) * crd(g, p1, c) + (35.0 / 132.0) * crd(g, i, c)
                                     - (34.0 / 33.0) * crd(g, m1, c) + (7.0 / 33.0) * crd(g, m2, c)
                                     - (2.0 / 33.0) * crd(g, m3, c) + (1.0 / 132.0) * crd(g, m4, c));
            }
            if (step > 1 && m2 == 0 && m1 != 0) {   /* next to the - end (:72-79) */
                b[step] = 2.0 / 11.0;
                dd[step] = 1.0;
                a[step] = 2.0 / 11.0;
                *rhs = (1.0 / dz) * (-1.0) * ((20.0 / 33.0) * crd(g, m1, c) + (35.0 / 132.0) * crd(g, i, c)
                                              - (34.0 / 33.0) * crd(g, p1, c) + (7.0 / 33.0) * crd(g, p2, c)
                                              - (2.0 / 33.0) * crd(g, p3, c) + (1.0 / 132.0) * crd(g, p4, c));
            }
            if (step != 0 && m1 == 0) {   /* the - end (:80-87) */
                b[step] = 0.0;
                dd[step] = 1.0;
                a[step] = 5.0;
                *rhs = (1.0 / dz) * (-1.0) * ((197.0 / 60.0) * crd(g, i, c) + (5.0 / 12.0) * crd(g, p1, c)
                                              - (5.0) * crd(g, p2, c) + (5.0 / 3.0) * crd(g, p3, c)
                                              - (5.0 / 12.0) * crd(g, p4, c) + (1.0 / 20.0) * crd(g, p5, c));
            }
        }
        i = m1;
        ++step;
    }
    const int M = step - 1;
    if (M < 2) return -1;
    /* elimination from the far end (:133-152) */
    dp[M - 1] = dd[M - 1] - ((b[M - 1] * a[M]) / dd[M]);
    for (int c = 0; c < 3; ++c) cp[3 * (M - 1) + c] = cc[3 * (M - 1) + c] - ((cc[3 * M + c] * b[M - 1]) / dd[M]);
    for (int s = M - 2; s >= 0; --s) {
        dp[s] = dd[s] - ((b[s] * a[s + 1]) / dp[s + 1]);
        for (int c = 0; c < 3; ++c) cp[3 * s + c] = cc[3 * s + c] - ((cp[3 * (s + 1) + c] * b[s]) / dp[s + 1]);
    }
    /* substitution from the + end (:154-204) */
    i = start;
    step = 0;
    while (i != 0) {
        const int prev = nb(g, i, P);
        for (int c = 0; c < 3; ++c) {
            double *Jc = J + 3 * (size_t)i + c;
            if (step > 0 && step < M) *Jc = (cp[3 * step + c] - a[step] * J[3 * (size_t)prev + c]) / dp[step];
            if (step == 0) *Jc = cp[c] / dp[0];
            if (step == M) *Jc = (cc[3 * step + c] - a[M] * J[3 * (size_t)prev + c]) / dd[M];
        }
        i = nb(g, i, Mn);
        ++step;
    }
    return 0;
}

int oracle_compact_metrics(const or_grid *g, int n_rows, double dz, double *det, or_metric *metric)
{
    for (int r = 1; r < n_rows; ++r)
        if (g[r].ID == 10) return -1;
    /* J[d][row][c] = d x_c / d dir_d, zero where no line passes */
    double *J = (double *)calloc((size_t)3 * 3 * n_rows, sizeof(double));
    double *w = (double *)malloc((size_t)14 * n_rows * sizeof(double));
    if (!J || !w) {
        free(J);
        free(w);
        return -1;
    }
    double *a = w, *b = w + n_rows, *dd = w + 2 * n_rows, *dp = w + 3 * n_rows, *cc = w + 4 * n_rows,
           *cp = w + 7 * n_rows;
    /* zeta: + is N1, - is N3 (:29-36); eta: N0 / N2 (:213-218); xi: N4 / N5
     * with the reference's loc condition (:328-334) */
    static const int P[3] = {1, 0, 4}, Mn[3] = {3, 2, 5};
    int rc = 0;
    for (int r = 1; r < n_rows && rc == 0; ++r)
        for (int d = 0; d < 3 && rc == 0; ++d) {
            if (nb(g, r, P[d]) != 0) continue;
            const int loc = g[r].loc;
            if (d == 2 && !(loc == 30 || loc == 31 || loc <= 27 || loc == 28)) continue;
            rc = compact_line(g, r, P[d], Mn[d], dz, n_rows, J + (size_t)3 * n_rows * d, a, b, dd, cc, dp, cp);
        }
    if (rc == 0) {
        const double *Jz = J, *Je = J + 3 * (size_t)n_rows, *Jx = J + 6 * (size_t)n_rows;
        for (int r = 1; r < n_rows; ++r) {
            const double x_zeta = Jz[3 * r], y_zeta = Jz[3 * r + 1], z_zeta = Jz[3 * r + 2];
            const double x_eta = Je[3 * r], y_eta = Je[3 * r + 1], z_eta = Je[3 * r + 2];
            const double x_xi = Jx[3 * r], y_xi = Jx[3 * r + 1], z_xi = Jx[3 * r + 2];
            /* :447 and :1029-1037 */
            const double D = (((x_zeta) * ((y_eta * z_xi) - (y_xi * z_eta))) + ((x_eta) * ((y_xi * z_zeta) - (y_zeta * z_xi)))
                              + ((x_xi) * ((y_zeta * z_eta) - (y_eta * z_zeta))));
            double *m = metric[r].m;
            det[r] = D;
            m[0] = (1.0 / D) * (y_eta * z_xi - y_xi * z_eta);
            m[1] = (1.0 / D) * (z_eta * x_xi - z_xi * x_eta);
            m[2] = (1.0 / D) * (x_eta * y_xi - x_xi * y_eta);
            m[3] = (1.0 / D) * (y_xi * z_zeta - y_zeta * z_xi);
            m[4] = (1.0 / D) * (z_xi * x_zeta - z_zeta * x_xi);
            m[5] = (1.0 / D) * (x_xi * y_zeta - x_zeta * y_xi);
            m[6] = (1.0 / D) * (y_zeta * z_eta - y_eta * z_zeta);
            m[7] = (1.0 / D) * (z_zeta * x_eta - z_eta * x_zeta);
            m[8] = (1.0 / D) * (x_zeta * y_eta - x_eta * y_zeta);
        }
    }
    free(J);
    free(w);
    return rc;
}

/* (3 f0 - 25 f1 + 150 f2 + 150 f3 - 25 f4 + 3 f5) / 256 in the reference's order */
static double six_point(double f0, double f1, double f2, double f3, double f4, double f5)
{
    return (1.0 / 256.0) * (3.0 * (f0) - 25.0 * (f1) + 150.0 * (f2) + 150.0 * (f3) - 25.0 * (f4) + 3.0 * (f5));
}

void oracle_half_point_metrics(const or_grid *g, int n_owned, const double *det, or_metric *metric,
                               or_determ *deter)
{
    /* direction d: + slot, - slot; the + face block 1 + 2d, the - face 2 + 2d */
    static const int P[3] = {1, 0, 4}, Mn[3] = {3, 2, 5};
    for (int r = 1; r <= n_owned; ++r) {
        double *fd = &deter[r].ip;
        for (int d = 0; d < 3; ++d) {
            const int m1 = nb(g, r, Mn[d]), m2 = nb(g, m1, Mn[d]), m3 = nb(g, m2, Mn[d]);
            const int p1 = nb(g, r, P[d]), p2 = nb(g, p1, P[d]), p3 = nb(g, p2, P[d]);
            double *plus = metric[r].m + 9 * (1 + 2 * d), *minus = metric[r].m + 9 * (2 + 2 * d);
            for (int c = 0; c < 9; ++c) {
                plus[c] = six_point(metric[m2].m[c], metric[m1].m[c], metric[r].m[c], metric[p1].m[c],
                                    metric[p2].m[c], metric[p3].m[c]);
                minus[c] = six_point(metric[m3].m[c], metric[m2].m[c], metric[m1].m[c], metric[r].m[c],
                                     metric[p1].m[c], metric[p2].m[c]);
            }
            fd[2 * d] = six_point(det[m2], det[m1], det[r], det[p1], det[p2], det[p3]);
            fd[2 * d + 1] = six_point(det[m3], det[m2], det[m1], det[r], det[p1], det[p2]);
        }
    }
}

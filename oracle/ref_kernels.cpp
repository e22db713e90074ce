/*
 * ref_kernels.cpp -- host-callable wrappers around the reference kernels,
 * compiled from the reference's unmodified U_Q.cl, Viscous.cl and Weno.cl
 * (include path = the reference checkout) plus one generated copy of
 * Viscous.cl whose four hard-coded constants (Viscous.cl:30-33) read globals.
 * TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh into oracle/_ref/.
 * Each entry point runs the kernel body for Gid in [0, n_items) under OpenMP,
 * as the reference's OpenCL CPU device does with local size 1.
 */
#include "ref_shim.h"

thread_local unsigned shim_gid = 0;
double ref_visc_mach = 1.5, ref_visc_reyl = 500.0, ref_visc_pr = 0.72, ref_visc_tinf = 273.0;

namespace kr_uq {
#include "U_Q.cl"
}
namespace kr_visc {
#include "Viscous.cl"
}
namespace kr_visc_param {
#include "Viscous_param.cl"
}
namespace kr_weno {
#include "Weno.cl"
}

extern "C" {

void ref_uq(int n_items, void *U_C, void *Q_C, const void *grid, const double *det, void *flow, void *roe)
{
#pragma omp parallel for schedule(static)
    for (int g = 0; g < n_items; ++g) {
        shim_gid = (unsigned)g;
        kr_uq::U_Q((kr_uq::Solver_Column_matrix *)U_C, (kr_uq::Solver_Column_matrix *)Q_C,
                    (const kr_uq::GRID *)grid, det, (kr_uq::FLOW_VARIABLES *)flow,
                    (kr_uq::ROE_AVERAGING *)roe);
    }
}

void ref_viscous(int n_items, const void *U_C, void *F, void *E, void *G, void *Fv, void *Ev, void *Gv,
                 const void *grid, const void *metric, const double *det, void *flow)
{
    typedef kr_visc::Solver_Column_matrix C5;
#pragma omp parallel for schedule(static)
    for (int g = 0; g < n_items; ++g) {
        shim_gid = (unsigned)g;
        kr_visc::Viscous((C5 *)U_C, (C5 *)F, (C5 *)E, (C5 *)G, (C5 *)Fv, (C5 *)Ev, (C5 *)Gv,
                          (const kr_visc::GRID *)grid, (const kr_visc::TRANSFORMED *)metric, det,
                          (kr_visc::FLOW_VARIABLES *)flow);
    }
}

void ref_viscous_param(int n_items, double mach, double reyl, double pr, double tinf,
                       const void *U_C, void *F, void *E, void *G, void *Fv, void *Ev, void *Gv,
                       const void *grid, const void *metric, const double *det, void *flow)
{
    ref_visc_mach = mach;
    ref_visc_reyl = reyl;
    ref_visc_pr = pr;
    ref_visc_tinf = tinf;
    typedef kr_visc_param::Solver_Column_matrix C5;
#pragma omp parallel for schedule(static)
    for (int g = 0; g < n_items; ++g) {
        shim_gid = (unsigned)g;
        kr_visc_param::Viscous((C5 *)U_C, (C5 *)F, (C5 *)E, (C5 *)G, (C5 *)Fv, (C5 *)Ev, (C5 *)Gv,
                                (const kr_visc_param::GRID *)grid, (const kr_visc_param::TRANSFORMED *)metric,
                                det, (kr_visc_param::FLOW_VARIABLES *)flow);
    }
}

void ref_weno(int n_items, int j, double mach, double del_t, const void *deter, const double *det,
              void *U0, void *U1, void *U2, const void *grid, void *Q_C, const void *metric, void *roe,
              void *Fv, void *Ev, void *Gv, void *F, void *E, void *G, void *flow)
{
    typedef kr_weno::Solver_Column_matrix C5;
#pragma omp parallel for schedule(static)
    for (int g = 0; g < n_items; ++g) {
        shim_gid = (unsigned)g;
        kr_weno::Weno(j, mach, del_t, (const kr_weno::DETERM *)deter, det, (C5 *)U0, (C5 *)U1, (C5 *)U2,
                       (const kr_weno::GRID *)grid, (C5 *)Q_C, (const kr_weno::TRANSFORMED *)metric,
                       (kr_weno::ROE_AVERAGING *)roe, (C5 *)Fv, (C5 *)Ev, (C5 *)Gv, (C5 *)F, (C5 *)E,
                       (C5 *)G, (kr_weno::FLOW_VARIABLES *)flow);
    }
}

}  // extern "C"

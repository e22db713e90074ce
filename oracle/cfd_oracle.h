/*
 * cfd_oracle.h -- CPU restatement of the reference right-hand-side path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA
 * library: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  Nothing in the product path calls it.
 *
 * It restates, in plain C with loops, the arithmetic of the three OpenCL
 * kernels of the reference solver and the stage sequencing of its host loop:
 *   U_Q.cl       -> oracle_uq        (Roe averages, U = det*Q, Q)
 *   Viscous.cl   -> oracle_viscous   (node fluxes F,E,G and viscous/SGS fluxes)
 *   Weno.cl      -> oracle_weno      (characteristic WENO5 + LLF + RK stage)
 *   Solver.cpp:365-658 -> oracle_rk3_step (U_Q, Viscous, Weno per stage)
 *   Flow_Initialisation.cpp:23-1394 -> oracle_boundary_fill (ghost fill)
 *   Grid_Transformation.cpp:22-1045 -> oracle_compact_metrics (node metrics)
 *   Main.cpp:2369-2440 -> oracle_half_point_metrics (face metrics, face dets)
 * The structs below are the reference's packed ABI (functions.h:49-113).
 *
 * Parity pin: the restatement is checked against the reference's own kernel
 * sources compiled as host C++ (oracle/build_ref.sh -> oracle/_ref/), and the
 * committed golden vectors under tests/golden/ were produced by that build.
 */
#ifndef CFD_ORACLE_H
#define CFD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#pragma pack(push, 1)
typedef struct { double x, y, z; int32_t N0, N1, N2, N3, N4, N5; int32_t ID, loc; } or_grid;   /* 56 B */
typedef struct { double u, v, w, p, t, rho, mu, a, e; } or_flow;                                 /* 72 B */
typedef struct { double N[5]; } or_col5;                                                          /* 40 B */
typedef struct { double m[63]; } or_metric;  /* node, ip, im, jp, jm, kp, km blocks of 9 */      /* 504 B */
typedef struct { double ip, im, jp, jm, kp, km; } or_determ;                                      /* 48 B */
typedef struct { double v[36]; } or_roe;     /* (u,v,w,p,h,rho) for ip, jp, kp, im, jm, km */     /* 288 B */
#pragma pack(pop)

/* Constants that the reference hard-codes in Viscous.cl:30-33 and Weno.cl:59,
 * made explicit.  The reference values are mach=1.5, reynolds=500,
 * prandtl=0.72, t_inf=273, weno_eps=1e-7 (10e-8 as written). */
typedef struct {
    double mach;
    double reynolds;
    double prandtl;
    double t_inf;
    double weno_eps;
    int viscous;   /* 0: zero Fv/Ev/Gv after the Viscous pass (inviscid runs) */
    int les;       /* SGS model: 0 none, 1 mixed time scale (the reference), 2 Smagorinsky */
    double smagorinsky_cs; /* C_s of les = 2 (a builder addition: no reference to pin it) */
} or_params;

/* A whole case in the reference layout.  Index 0 is the reference's dummy row;
 * owned nodes are 1..sd_node, ghosts sd_node+1..g_node. */
typedef struct {
    int g_node, sd_node;
    or_grid *grid;
    double *det;
    or_determ *deter;
    or_metric *metric;
    or_flow *flow;
    or_col5 *U0, *U1, *U2, *Q, *F, *E, *G, *Fv, *Ev, *Gv;
    or_roe *roe;
} or_case;

void oracle_uq(int n_items, or_col5 *U_C, or_col5 *Q_C, const or_grid *grid,
               const double *det, const or_flow *flow, or_roe *roe);

void oracle_viscous(int n_items, const or_params *prm, const or_col5 *U_C,
                    or_col5 *F, or_col5 *E, or_col5 *G, or_col5 *Fv, or_col5 *Ev, or_col5 *Gv,
                    const or_grid *grid, const or_metric *metric, const double *det, or_flow *flow);

/* Writes the RHS L of every processed node into L_out when it is non-NULL. */
void oracle_weno(int n_items, int j, double mach, double del_t, const or_params *prm,
                 const or_determ *deter, const double *det,
                 or_col5 *U0, or_col5 *U1, or_col5 *U2, const or_grid *grid,
                 const or_col5 *Q_C, const or_metric *metric, const or_roe *roe,
                 const or_col5 *Fv, const or_col5 *Ev, const or_col5 *Gv,
                 const or_col5 *F, const or_col5 *E, const or_col5 *G,
                 or_flow *flow, or_col5 *L_out);

/* One RK stage j of the host loop (Solver.cpp:365-541) with j passed per
 * stage: U_Q writes U_j, Viscous reads U_j, Weno(j).  L_out may be NULL. */
void oracle_stage(or_case *c, const or_params *prm, int j, double del_t, or_col5 *L_out);

/* nsteps full SSP-RK3 steps (three stages each). */
void oracle_rk3_steps(or_case *c, const or_params *prm, double del_t, int nsteps);

/* Boundary node lists of the reference's boundary routine intialise()
 * (Flow_Initialisation.cpp:23-1394): row indices in visiting order.  The
 * routine's second half (:1395-2742) applies the same rules to the
 * subdomain lists sd_*_node; pass those as a second set. */
typedef struct {
    const int32_t *outlet, *inlet, *boundary, *wall;
    int n_outlet, n_inlet, n_boundary, n_wall;
    /* singular-node table of the wake cut (functions.h singul; the
     * reference fills it in Main.cpp:1640-1700): six neighbour slots per
     * row, row-major [rows][6]; NULL when no wall node needs it. */
    const int32_t *singular;
    /* trailing-edge tip rows fixed after the routine (Solver.cpp:660-683) */
    const int32_t *tips;
    int n_tips;
} or_bc_lists;

/* intialise(RK) restated: with initial == 0 rows 1..sd_node first get the
 * free stream; then outlet, inlet, boundary and wall nodes in that order --
 * face codes 1..6 with their three ghost layers, edge and corner codes 7..26
 * from a diagonal node, and on walls the singular-node branches (codes
 * 29/30, ID 10, codes 33..52) from the singular table; then the tip rows.
 * Returns -1 (and changes nothing) when a wall node needs the singular
 * table and none is given, or has a code 53..56 (the routine leaves the
 * mirror slots of those codes unset). */
int oracle_boundary_fill(const or_grid *grid, or_flow *flow, const or_bc_lists *bc, double mach, int initial,
                         int sd_node);

/* oracle_rk3_steps with the boundary routine after every stage
 * (Solver.cpp:364-658).  bc may be NULL.  Returns -1 as above. */
int oracle_rk3_steps_bc(or_case *c, const or_params *prm, double del_t, int nsteps, const or_bc_lists *bc);

/* Node Jacobians by the sixth-order compact scheme along every line of
 * the node table, det and the node metrics as cofactors / det
 * (Grid_Transformation.cpp:22-1045, metric_term()).  A line starts at a row
 * with no neighbour in the + direction (zeta: N1, eta: N0, xi: N4, subject
 * to the reference's start conditions) and walks the - neighbours to the
 * row that has none; rows 1..n_rows-1.  Writes det[] and the node block
 * (columns 0..8) of metric[].  Returns -1 (writing nothing) when a row has
 * ID 10 (the reference's C-grid wake-cut branches) or a line is shorter
 * than three rows. */
int oracle_compact_metrics(const or_grid *grid, int n_rows, double del_zeta, double *det, or_metric *metric);

/* Face metrics and face dets of rows 1..n_owned by the six-point midpoint
 * rule (3, -25, 150, 150, -25, 3)/256 of node values (Main.cpp:2369-2440). */
void oracle_half_point_metrics(const or_grid *grid, int n_owned, const double *det, or_metric *metric,
                               or_determ *deter);

/* Undefined-branch poisoning (NaN) for masking checks; off by default. */
void oracle_set_poison(int on);

/* OpenMP thread count used by the loops (0 = runtime default). */
void oracle_set_threads(int n);
int oracle_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif

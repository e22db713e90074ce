/*
 * cfd_rhs.h -- C ABI of the GB300 right-hand-side path (libcfd_gb300.so).
 *
 * Drop-in replacement for the three OpenCL kernel launches of the reference
 * solver's host loop (Solver.cpp:365-541):
 *
 *   reference launch                                   replacement
 *   -------------------------------------------------  -----------------
 *   queue.enqueueNDRangeKernel(kernel_U_Q, ...)        cfd_uq
 *        Solver.cpp:377, kernel args Solver.cpp:277-282, U_Q.cl:36-38
 *   queue_viscous.enqueueNDRangeKernel(kernel_viscous) cfd_viscous
 *        Solver.cpp:440, args Solver.cpp:284-294, Viscous.cl:23-26
 *   queue_weno.enqueueNDRangeKernel(kernel_weno, ...)  cfd_weno
 *        Solver.cpp:521, args Solver.cpp:296-314, Weno.cl:36-40
 *   cl::Buffer(...) / cl::copy(...)                    cfd_buffer_*
 *        Solver.cpp:232-273 and the copies around each launch
 *
 * The buffers use the reference's packed array-of-structs layout
 * (functions.h:49-113), reproduced below with the same field names and
 * sizes.  Row 0 is the reference's dummy row; the NDRange of U_Q and Viscous
 * is g_node+1 rows, that of Weno sd_node+1 rows (Solver.cpp:31-38).
 *
 * Beyond the drop-in, the library offers whole SSP-RK3 steps on the same
 * buffers (cfd_rk3_step), the reference's boundary routine on the device
 * (cfd_bc_*, cfd_boundary_fill), a resident solver object (cfd_solver_*)
 * that selects a face-based lattice path when the neighbour table is a
 * lattice (periodic, or with ghost layers in non-periodic directions) and
 * runs FP64 or mixed precision, and a batched solver for many grids in one
 * launch per stage with scheduling hooks for a request loop (cfd_batch_*).
 *
 * Error handling: every entry point returns a cfd_status_t; none exits the
 * process (the reference prints and calls exit(1), Solver.cpp:378-381).
 * Threading: a context is used by one host thread at a time; separate
 * contexts may be used concurrently.
 */
#ifndef CFD_RHS_H
#define CFD_RHS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CFD_ABI_VERSION 1

typedef enum {
    CFD_OK = 0,
    CFD_EINVAL = 1,        /* bad argument, pointer kind, neighbour index or size */
    CFD_ENONFINITE = 2,    /* a NaN/Inf appeared in the advanced state            */
    CFD_ETIMEOUT = 3,      /* a bounded device wait gave up                       */
    CFD_ECUDA = 4,         /* a CUDA runtime call failed (see cfd_last_error)     */
    CFD_ENOMEM = 5,        /* device allocation failed                            */
    CFD_EUNSUPPORTED = 6   /* request outside what the library supports           */
} cfd_status_t;

/* ------------------------------------------------ reference data layout -- */
#pragma pack(push, 1)
/* GRID (functions.h:57-61): coordinates, neighbours N0=+j N1=+i N2=-j N3=-i
 * N4=+k N5=-k (U_Q.cl:51-56), node ID and location code (0 interior,
 * 1..56 boundary, 100 ghost). */
typedef struct {
    double x, y, z;
    int32_t N0, N1, N2, N3, N4, N5;
    int32_t ID, loc;
} cfd_grid_t;

/* FLOW_VARIABLES (functions.h:49-51). */
typedef struct {
    double u, v, w, p, t, rho, mu, a, e;
} cfd_flow_t;

/* Solver_Column_matrix (functions.h:53-55): rho, rho u, rho v, rho w, E. */
typedef struct {
    double N0, N1, N2, N3, N4;
} cfd_column_t;

/* TRANSFORMED (functions.h:93-98): node metrics, then the half-point metrics
 * of the six faces. */
typedef struct {
    double zeta_x, zeta_y, zeta_z, eta_x, eta_y, eta_z, xi_x, xi_y, xi_z;
    double zeta_xip, zeta_yip, zeta_zip, eta_xip, eta_yip, eta_zip, xi_xip, xi_yip, xi_zip;
    double zeta_xim, zeta_yim, zeta_zim, eta_xim, eta_yim, eta_zim, xi_xim, xi_yim, xi_zim;
    double zeta_xjp, zeta_yjp, zeta_zjp, eta_xjp, eta_yjp, eta_zjp, xi_xjp, xi_yjp, xi_zjp;
    double zeta_xjm, zeta_yjm, zeta_zjm, eta_xjm, eta_yjm, eta_zjm, xi_xjm, xi_yjm, xi_zjm;
    double zeta_xkp, zeta_ykp, zeta_zkp, eta_xkp, eta_ykp, eta_zkp, xi_xkp, xi_ykp, xi_zkp;
    double zeta_xkm, zeta_ykm, zeta_zkm, eta_xkm, eta_ykm, eta_zkm, xi_xkm, xi_ykm, xi_zkm;
} cfd_metric_t;

/* DETERM (functions.h:110-112): face Jacobian determinants. */
typedef struct {
    double ip, im, jp, jm, kp, km;
} cfd_determ_t;

/* ROE_AVERAGING (functions.h:63-70): Roe states of the six faces. */
typedef struct {
    double roe_u_ip, roe_v_ip, roe_w_ip, roe_p_ip, roe_h_ip, roe_rho_ip;
    double roe_u_jp, roe_v_jp, roe_w_jp, roe_p_jp, roe_h_jp, roe_rho_jp;
    double roe_u_kp, roe_v_kp, roe_w_kp, roe_p_kp, roe_h_kp, roe_rho_kp;
    double roe_u_im, roe_v_im, roe_w_im, roe_p_im, roe_h_im, roe_rho_im;
    double roe_u_jm, roe_v_jm, roe_w_jm, roe_p_jm, roe_h_jm, roe_rho_jm;
    double roe_u_km, roe_v_km, roe_w_km, roe_p_km, roe_h_km, roe_rho_km;
} cfd_roe_t;
#pragma pack(pop)

/* The packed sizes of functions.h:49-113, which the host's vectors have. */
#ifdef __cplusplus
#define CFD_SIZE_CHECK(T, n) static_assert(sizeof(T) == (n), #T " must match the reference layout")
#else
#define CFD_SIZE_CHECK(T, n) _Static_assert(sizeof(T) == (n), #T " must match the reference layout")
#endif
CFD_SIZE_CHECK(cfd_grid_t, 56);
CFD_SIZE_CHECK(cfd_flow_t, 72);
CFD_SIZE_CHECK(cfd_column_t, 40);
CFD_SIZE_CHECK(cfd_metric_t, 504);
CFD_SIZE_CHECK(cfd_determ_t, 48);
CFD_SIZE_CHECK(cfd_roe_t, 288);
#undef CFD_SIZE_CHECK

/* -------------------------------------------------------- parameters ---- */
/* Arithmetic of a solver or batch (no counterpart in the reference, whose
 * kernels are FP64 throughout):
 *   CFD_PREC_FP64   the reference's FP64 arithmetic in its evaluation order
 *                   (relative L2 <= 1e-12 against it);
 *   CFD_PREC_MIXED  everything in FP32 on the FP32 pipe: the conserved state
 *                   and the RK3 accumulation as hi + lo pairs of FP32 numbers
 *                   (double-float, about 48 bits), the geometry as FP32
 *                   copies -- no FP64 instruction in a stage;
 *   CFD_PREC_SPLIT  FP64 for the conserved state, the RK3 accumulation,
 *                   Q = U/det, the metric/Jacobian products of the face flux
 *                   (DET_f (m_f . F), Weno.cl:2585-2728) with its LLF
 *                   average and the flux difference L; FP32 for the
 *                   characteristic projection, WENO5, the LLF speed and
 *                   dissipation, the viscous and SGS fluxes and the node
 *                   fluxes of the sixth-order correction.
 * The mixed and split forms run on lattices only (structured path). */
typedef enum { CFD_PREC_FP64 = 0, CFD_PREC_MIXED = 1, CFD_PREC_SPLIT = 2 } cfd_precision_t;

/* The constants the reference hard-codes (Viscous.cl:30-33 Mach 1.5,
 * Reyl 500, Pr 0.72, Free_t 273; Weno.cl:59 Epsilon 10e-8).  A NULL params
 * pointer anywhere below means exactly these values with viscous and LES on
 * and FP64 arithmetic.  gamma is 1.4 throughout, as in the reference. */
typedef struct {
    double mach;
    double reynolds;
    double prandtl;
    double t_inf;
    double weno_eps;
    int32_t viscous;     /* 0: Fv = Ev = Gv = 0 (inviscid)                    */
    int32_t les;         /* SGS model: 0 none, 1 mixed time scale (the
                          * reference, Viscous.cl:490-558), 2 Smagorinsky   */
    int32_t precision;   /* cfd_precision_t (solver objects only)             */
    int32_t reserved;
    double smagorinsky_cs; /* C_s of les = 2 (default 0.1): eddy viscosity
                            * (C_s det^(1/3))^2 |S|, |S| = sqrt(2 S_ij S_ij),
                            * in the reference's SGS stress and heat-flux
                            * terms; no counterpart in the reference */
} cfd_params_t;

void cfd_params_default(cfd_params_t *p);

/* ----------------------------------------------------------- context ---- */
typedef struct cfd_ctx cfd_ctx_t;

/* Creates a context on CUDA device `device` with its own stream. */
cfd_status_t cfd_ctx_create(cfd_ctx_t **ctx, int device);
cfd_status_t cfd_ctx_destroy(cfd_ctx_t *ctx);
/* Use a caller-owned cudaStream_t (as void*) instead of the context's. */
cfd_status_t cfd_ctx_set_stream(cfd_ctx_t *ctx, void *cuda_stream);
/* async = 0 (default): each kernel entry point waits for its launch and
 * reports device-side errors, like the reference's event.wait(); finish().
 * async = 1: entry points only enqueue; errors surface at synchronize. */
cfd_status_t cfd_ctx_set_async(cfd_ctx_t *ctx, int async);
cfd_status_t cfd_ctx_synchronize(cfd_ctx_t *ctx);
/* Number of rows of every buffer (g_node + 1).  Neighbour indices outside
 * [0, n_rows) make a kernel skip the row and report CFD_EINVAL. */
cfd_status_t cfd_ctx_set_rows(cfd_ctx_t *ctx, int32_t n_rows);
/* Sharing of intermediates between rows (default on): cfd_weno computes each
 * row's +1/2 faces once and takes a row's -1/2 face from its minus
 * neighbour's +1/2 face wherever the two evaluations have bit-identical
 * inputs (Weno.cl:336-3058 evaluates both at every row), and cfd_uq computes
 * sqrt(rho) and H once per row instead of once per row and neighbour
 * (U_Q.cl:60-109); the results are the same bits.  on = 0 evaluates
 * everything per row, as the reference does.  Needs 252 bytes per row,
 * allocated by cfd_ctx_set_rows. */
cfd_status_t cfd_ctx_set_face_reuse(cfd_ctx_t *ctx, int on);
/* Kernels this context launched since creation (for accounting). */
uint64_t cfd_ctx_launch_count(const cfd_ctx_t *ctx);
const char *cfd_status_string(cfd_status_t s);
const char *cfd_last_error(const cfd_ctx_t *ctx);

/* ------------------------------------------- buffers (cl::Buffer/copy) -- */
cfd_status_t cfd_buffer_alloc(cfd_ctx_t *ctx, size_t bytes, void **device_ptr);
cfd_status_t cfd_buffer_free(cfd_ctx_t *ctx, void *device_ptr);
cfd_status_t cfd_buffer_write(cfd_ctx_t *ctx, void *device_dst, const void *host_src, size_t bytes);
cfd_status_t cfd_buffer_read(cfd_ctx_t *ctx, void *host_dst, const void *device_src, size_t bytes);

/* ------------------------------------------- drop-in kernel entry points -- */
/* Buffer arguments are device pointers (cfd_buffer_alloc or any cudaMalloc'd
 * memory; the resident mode: nothing is copied) or host pointers to arrays of
 * n_rows rows (the reference host's std::vector data): a host buffer gets a
 * device mirror owned by the context (one per host address, kept until
 * cfd_ctx_destroy), its rows are copied in before the launch and, if the
 * call writes it, back before the call returns -- the cl::copy of
 * Solver.cpp:371-541 around each launch.  Argument order follows
 * the reference kernels; the trailing params pointer (NULL = reference
 * constants) carries the constants the reference hard-codes. */

/* U_Q.cl:36-125: Roe averages of the six faces, U_C = det*Q, Q_C. */
cfd_status_t cfd_uq(cfd_ctx_t *ctx, cfd_column_t *U_C, cfd_column_t *Q_C, const cfd_grid_t *Grid_P,
                    const double *det, cfd_flow_t *FLOW, cfd_roe_t *ROE_AVER, int32_t n_items);

/* Viscous.cl:23-643: node fluxes F,E,G and viscous + SGS fluxes Fv,Ev,Gv
 * (contravariant, times det); writes FLOW.mu. */
cfd_status_t cfd_viscous(cfd_ctx_t *ctx, cfd_column_t *U_C, cfd_column_t *F_C, cfd_column_t *E_C,
                         cfd_column_t *G_C, cfd_column_t *Fv_C, cfd_column_t *Ev_C, cfd_column_t *Gv_C,
                         const cfd_grid_t *Grid_P, const cfd_metric_t *metric, const double *det,
                         cfd_flow_t *FLOW, int32_t n_items, const cfd_params_t *params);

/* Weno.cl:36-3137: characteristic WENO5 + LLF + 6th-order flux correction +
 * viscous divergence, RHS L, SSP-RK3 stage j (0,1,2) and primitive update.
 * L_out (may be NULL) receives L per row. */
cfd_status_t cfd_weno(cfd_ctx_t *ctx, int32_t j, double Mach, double del_t, const cfd_determ_t *deter,
                      const double *det, cfd_column_t *U0, cfd_column_t *U1, cfd_column_t *U2,
                      const cfd_grid_t *Grid_P, cfd_column_t *Q_C, const cfd_metric_t *metric,
                      cfd_roe_t *ROE_AVER, cfd_column_t *Fv, cfd_column_t *Ev, cfd_column_t *Gv,
                      cfd_column_t *F, cfd_column_t *E, cfd_column_t *G, cfd_flow_t *FLOW, int32_t n_items,
                      const cfd_params_t *params, cfd_column_t *L_out);

/* ---------------------------------------------- resident solver object -- */
/* Host-side description of one grid in the reference layout (all host
 * pointers, rows 0..g_node).  Copied at create time. */
typedef struct {
    int32_t g_node;     /* rows 1..g_node hold owned + ghost nodes   */
    int32_t sd_node;    /* rows 1..sd_node are owned (advanced) rows  */
    const cfd_grid_t *grid;
    const double *det;
    const cfd_determ_t *deter;
    const cfd_metric_t *metric;
} cfd_geometry_t;

typedef enum {
    CFD_PATH_GATHER = 0,       /* drop-in kernels on the reference layout       */
    CFD_PATH_STRUCTURED = 1    /* face-based kernels on a periodic lattice (SoA) */
} cfd_path_t;

typedef struct {
    int32_t path;              /* cfd_path_t chosen at create time           */
    int32_t ni, nj, nk;        /* lattice shape for the structured path      */
    int32_t precision;         /* cfd_precision_t                            */
    int32_t reserved;
    uint64_t device_bytes;     /* device memory held by the solver           */
    int32_t face_tile_i;       /* mixed/split lattice: faces per tile along i */
    int32_t face_tile_jk;      /*   and along j and k (0 otherwise)          */
    int32_t face_blocks[3];    /* FP64 lattice: blocks of 128 per SM the i, j,
                                  k face passes request (0 otherwise)        */
    int32_t reserved2;
} cfd_solver_info_t;

typedef struct cfd_solver cfd_solver_t;

/* `force_path` = -1 chooses automatically; 0/1 forces a path (forcing the
 * structured path on a table that is not a lattice -> CFD_EINVAL).  A
 * lattice here is periodic in every direction, or has non-periodic
 * directions whose outermost ghost rows point at themselves, at least three
 * ghost layers beyond the owned rows (1..sd_node, loc != 100) and ghosts
 * carrying loc 100 -- the face-based kernels then follow the reference's
 * loc-code derivative branches. */
cfd_status_t cfd_solver_create(cfd_ctx_t *ctx, const cfd_geometry_t *geom, const cfd_params_t *params,
                               int32_t force_path, cfd_solver_t **solver);
cfd_status_t cfd_solver_destroy(cfd_solver_t *s);
cfd_status_t cfd_solver_info(const cfd_solver_t *s, cfd_solver_info_t *info);
/* Face-tile widths of the mixed and split face passes (blocks of 128
 * threads staging their stencil lines in shared memory): tile_i faces along
 * i (32, 64 or 128) and tile_jk along j and k (8, 16 or 32); 0 keeps a
 * width.  cfd_solver_create times every width once per form and lattice
 * shape in the process and keeps the fastest; the widths change no result
 * bit.  CFD_EUNSUPPORTED for FP64 or gather-path solvers. */
cfd_status_t cfd_solver_set_face_tiles(cfd_solver_t *s, int32_t tile_i, int32_t tile_jk);
/* Register budgets of the FP64 face passes along i, j and k: the blocks of
 * 128 threads per SM their launch bounds request (2, 3 or 4; 0 keeps one).
 * The solver's second stage times the three per direction on its real
 * inputs, once per lattice shape in the process, and keeps the fastest
 * (cfd_solver_info reports 3, 3, 2 before that); every budget gives the same
 * bits.
 * CFD_EUNSUPPORTED for the reduced forms and gather-path solvers. */
cfd_status_t cfd_solver_set_face_blocks(cfd_solver_t *s, int32_t blocks_i, int32_t blocks_j, int32_t blocks_k);
/* State in/out as FLOW rows 0..g_node (host pointers). */
cfd_status_t cfd_solver_set_flow(cfd_solver_t *s, const cfd_flow_t *flow_host);
cfd_status_t cfd_solver_get_flow(cfd_solver_t *s, cfd_flow_t *flow_host);
/* Conserved state U0 (= det*Q at the last step boundary), rows 0..g_node. */
cfd_status_t cfd_solver_get_u0(cfd_solver_t *s, cfd_column_t *u0_host);
/* nsteps SSP-RK3 steps of size del_t, entirely on the device. */
cfd_status_t cfd_solver_step(cfd_solver_t *s, double del_t, int32_t nsteps);
/* One stage j of the host loop; copies L (rows 0..g_node, owned rows set)
 * to L_host when non-NULL. */
cfd_status_t cfd_solver_stage(cfd_solver_t *s, int32_t j, double del_t, cfd_column_t *L_host);

/* ------------------------------------------------- boundary routine ---- */
/* The reference's boundary routine intialise() (Flow_Initialisation.cpp:
 * 23-1394, called after every RK stage at Solver.cpp:658) on the device.
 * The four lists are the routine's wall_node, inlet_node, outlet_node and
 * boundary_node arrays (row indices; the routine's second half,
 * :1395-2742, applies the same rules to the subdomain lists sd_*_node --
 * pass those to a second cfd_bc_t).  Face codes 1..6 fill the node and its
 * three ghost layers, edge and corner codes 7..26 copy a diagonal node;
 * wall nodes that need the reference's singular-node table (ID 10, loc
 * 29/30/33..56) give CFD_EUNSUPPORTED here (see cfd_bc_create_singular).
 * `grid` is host memory, read once. */
typedef struct cfd_bc cfd_bc_t;
cfd_status_t cfd_bc_create(cfd_ctx_t *ctx, const cfd_grid_t *grid, int32_t n_rows, const int32_t *outlet,
                           int32_t n_outlet, const int32_t *inlet, int32_t n_inlet, const int32_t *boundary,
                           int32_t n_boundary, const int32_t *wall, int32_t n_wall, cfd_bc_t **bc);
/* cfd_bc_create for grids with a wake cut (C-grids): `singular` (host, may
 * be NULL) is the reference's singular-node table -- six neighbour slots per
 * row, row-major [n_rows][6], the `singular[].n_n[0..5]` array that
 * Main.cpp:1612-1700 fills with the neighbours across the cut.  Wall nodes
 * with ID 10 or loc 29/30/33..52 then get the routine's singular branches
 * (Flow_Initialisation.cpp:1194-1392) after the rule of their code: codes
 * 29/30 the node rule from the node beyond singular[b][3]; ID 10 the node
 * rule from singular[b][3] and three mirror passes of three ghosts each;
 * codes 33..52 the node rule from singular[b][0] and two or three (node
 * rule, mirror pass) pairs.  Wall codes 53..56 give CFD_EUNSUPPORTED (the
 * routine runs their mirror pass with slots it never sets).  `tips`
 * (n_tips rows) are the trailing-edge rows the solver loop fixes after the
 * routine (Solver.cpp:660-683: zero velocity, p and t of the slot-3
 * neighbour, rho and e derived); they run after every list of this object,
 * so with a second cfd_bc_t for the subdomain lists pass them to the one
 * applied last. */
cfd_status_t cfd_bc_create_singular(cfd_ctx_t *ctx, const cfd_grid_t *grid, int32_t n_rows, const int32_t *outlet,
                                    int32_t n_outlet, const int32_t *inlet, int32_t n_inlet, const int32_t *boundary,
                                    int32_t n_boundary, const int32_t *wall, int32_t n_wall, const int32_t *singular,
                                    const int32_t *tips, int32_t n_tips, cfd_bc_t **bc);
cfd_status_t cfd_bc_destroy(cfd_bc_t *bc);
/* intialise() on a FLOW buffer of the reference layout (device, or the host
 * rows of the table the lists were made for, copied as for the kernel entry
 * points); with
 * initial == 0 rows 1..sd_node first get the free stream
 * (Flow_Initialisation.cpp:35-48). */
cfd_status_t cfd_boundary_fill(cfd_ctx_t *ctx, const cfd_bc_t *bc, cfd_flow_t *FLOW, double Mach, int32_t initial,
                               int32_t sd_node);

/* nsteps whole SSP-RK3 steps of the host loop (Solver.cpp:356-658) in one
 * call on the reference buffers: per stage j, U_Q (rows 0..g_node, writes
 * U_j), Viscous (rows 0..g_node), Weno stage j (rows 0..sd_node) and, if bc
 * is not NULL, the boundary routine (initial = 1).  Buffers as for the
 * kernel entry points (host buffers are copied in once and out once per
 * call); argument order that of cfd_weno without j. */
cfd_status_t cfd_rk3_step(cfd_ctx_t *ctx, double Mach, double del_t, const cfd_determ_t *deter, const double *det,
                          cfd_column_t *U0, cfd_column_t *U1, cfd_column_t *U2, const cfd_grid_t *Grid_P,
                          cfd_column_t *Q_C, const cfd_metric_t *metric, cfd_roe_t *ROE_AVER, cfd_column_t *Fv,
                          cfd_column_t *Ev, cfd_column_t *Gv, cfd_column_t *F, cfd_column_t *E, cfd_column_t *G,
                          cfd_flow_t *FLOW, int32_t g_node, int32_t sd_node, const cfd_params_t *params,
                          const cfd_bc_t *bc, int32_t nsteps);
/* The solver runs the routine after every stage (with its Mach number);
 * NULL switches it off.  The solver keeps its own copy of the plan. */
cfd_status_t cfd_solver_set_boundary(cfd_solver_t *s, const cfd_bc_t *bc);

/* One stage j of the host loop with a CUDA event around every kernel
 * launch; out[i] receives each launch's name and device time.  The stage
 * advances the state like cfd_solver_stage. */
typedef struct {
    char name[24];
    double ms;
} cfd_kernel_time_t;
cfd_status_t cfd_solver_profile_stage(cfd_solver_t *s, int32_t j, double del_t, cfd_kernel_time_t *out,
                                      int32_t max_out, int32_t *n_out);

/* ------------------------------------------------ batched lattices ---- */
/* Many independent periodic lattices of different sizes advanced together:
 * one persistent cooperative kernel launch per RK stage covers every
 * instance through a tile table, and one RK step is captured as a CUDA
 * graph.  Instances are admitted against a device-memory budget, stay
 * resident, and may be added or removed between steps (the serving loop's
 * engine).  Each instance has its own parameters and time step. */
typedef struct cfd_batch cfd_batch_t;

typedef struct {
    int32_t n_active;          /* instances in the batch                      */
    int32_t tile_nodes;        /* nodes per tile = threads per block          */
    int32_t blocks;            /* persistent grid size                        */
    int32_t graph;             /* 1 when steps replay a captured CUDA graph   */
    int32_t precision;         /* cfd_precision_t of the whole batch          */
    int32_t n_held;            /* instances held out of cfd_batch_step        */
    uint64_t nodes_total;
    uint64_t device_bytes;     /* admitted instance memory                    */
    uint64_t capacity_bytes;   /* admission budget                            */
    int32_t face_tiles;        /* 1: phase A in shared-memory face tiles      */
    int32_t reserved;
} cfd_batch_info_t;

/* capacity_bytes = 0: 85 % of the device memory free at creation. */
cfd_status_t cfd_batch_create(cfd_ctx_t *ctx, int32_t precision, uint64_t capacity_bytes, cfd_batch_t **batch);
cfd_status_t cfd_batch_destroy(cfd_batch_t *b);
/* Device bytes one instance of `nodes` lattice nodes takes (admission). */
uint64_t cfd_batch_instance_bytes(int32_t precision, int64_t nodes);
/* Adds a periodic-lattice instance (CFD_EUNSUPPORTED otherwise) with its
 * initial FLOW rows 0..g_node and time step; CFD_ENOMEM beyond the budget. */
cfd_status_t cfd_batch_add(cfd_batch_t *b, const cfd_geometry_t *geom, const cfd_params_t *params,
                           const cfd_flow_t *flow, double del_t, int32_t *slot);
/* cfd_batch_add in two halves.  cfd_batch_stage checks the table and
 * converts the geometry and FLOW into host memory of its own; it touches no
 * device, context or batch, so it may run on another host thread while the
 * batch steps (the caller's arrays may be released once it returns).  It
 * returns the check's status and, unless out of host memory, always sets
 * *staged.  cfd_batch_add_staged allocates, uploads and prepares the staged
 * instance (reporting a failed check with its message, as cfd_batch_add
 * does) and frees *staged in every case; cfd_batch_staged_free discards one
 * unused. */
typedef struct cfd_batch_staged cfd_batch_staged_t;
cfd_status_t cfd_batch_stage(const cfd_geometry_t *geom, const cfd_params_t *params, const cfd_flow_t *flow,
                             double del_t, cfd_batch_staged_t **staged);
cfd_status_t cfd_batch_add_staged(cfd_batch_t *b, cfd_batch_staged_t *staged, int32_t *slot);
cfd_status_t cfd_batch_staged_free(cfd_batch_staged_t *staged);
cfd_status_t cfd_batch_remove(cfd_batch_t *b, int32_t slot);
/* nsteps SSP-RK3 steps of every instance that is not held.  CFD_ENONFINITE
 * names the first failing slot in cfd_last_error; the other instances
 * advance normally. */
cfd_status_t cfd_batch_step(cfd_batch_t *b, int32_t nsteps);
/* The same steps, queued: returns once the steps of the previous
 * cfd_batch_step_async call have finished, with this call's steps still
 * running, so the host can prepare the next step (admission, scheduling)
 * while the device works.  Errors of queued steps (CFD_ENONFINITE,
 * CFD_ETIMEOUT) are reported by the next cfd_batch_sync or cfd_batch_step. */
cfd_status_t cfd_batch_step_async(cfd_batch_t *b, int32_t nsteps);
/* Waits for every queued step and reports their status. */
cfd_status_t cfd_batch_sync(cfd_batch_t *b);
/* hold != 0: the instance stays resident (state, slot and memory) but
 * cfd_batch_step leaves it out until it is released (hold = 0); a
 * scheduler uses this to run a subset of the batch.  Takes effect at the
 * next step (the tile table and graph are rebuilt once per change). */
cfd_status_t cfd_batch_set_hold(cfd_batch_t *b, int32_t slot, int32_t hold);
cfd_status_t cfd_batch_get_flow(cfd_batch_t *b, int32_t slot, cfd_flow_t *flow_host);
/* U0 = det*Q of the current FLOW (the next stage's U_Q output). */
cfd_status_t cfd_batch_get_u0(cfd_batch_t *b, int32_t slot, cfd_column_t *u0_host);
/* CFD_ENONFINITE after a non-finite state; CFD_ETIMEOUT while the slot is
 * interrupted (below). */
cfd_status_t cfd_batch_slot_status(cfd_batch_t *b, int32_t slot);
/* Replaces the state of an instance with FLOW rows 0..g_node (host memory)
 * and prepares its next step, as cfd_batch_add does; clears the slot's
 * error flags.  Waits for queued steps first.  This is the recovery path
 * after a barrier timeout and the restore path of a checkpoint. */
cfd_status_t cfd_batch_set_flow(cfd_batch_t *b, int32_t slot, const cfd_flow_t *flow_host);
/* Deadline of the persistent kernel's grid barrier in nanoseconds (< 0: the
 * default, 5 s + 50 ns per batched node).  A block that waits longer gives up
 * and skips the rest of that stage; the step reports CFD_ETIMEOUT once (the
 * reference exits the process on any kernel failure, Solver.cpp:378-381)
 * and every instance it was advancing is marked interrupted: its state is
 * part old, part new, so cfd_batch_step refuses to advance it
 * (CFD_ETIMEOUT) until cfd_batch_set_flow restores it or it is removed.
 * Instances that were held are not affected. */
cfd_status_t cfd_batch_set_wait_limit(cfd_batch_t *b, int64_t limit_ns);
/* tile_nodes in {32, 64, 128, 256}: phase A of a stage works on 1-D tiles of
 * that many nodes, each face evaluated from its own stencil gathers;
 * CFD_BATCH_FACE_TILES (mixed and split batches): phase A works on the
 * viscous ranges and on 2-D face tiles whose stencil lines a block of 128
 * threads stages in shared memory (32 faces along i x 4, or 16 along j or k
 * x 8); 0 keeps the current choice.  max_blocks (0 = occupancy limit),
 * use_graph 0/1. */
#define CFD_BATCH_FACE_TILES 1
cfd_status_t cfd_batch_set_tiling(cfd_batch_t *b, int32_t tile_nodes, int32_t max_blocks, int32_t use_graph);
/* Times each tiling (1-D tiles of 32, 64, 128, 256 nodes and, for the mixed and
 * split batches, the face tiles) on the live batch (state saved and
 * restored) and keeps the fastest. */
cfd_status_t cfd_batch_tune(cfd_batch_t *b, int32_t steps_per_trial);
cfd_status_t cfd_batch_info(const cfd_batch_t *b, cfd_batch_info_t *info);

/* ------------------------------------------------- geometry producer ---- */
/* The inputs the kernels read, computed from a node table as the reference
 * computes them once before its time loop.  Host functions (all pointers
 * host memory, rows 0..n_rows-1, row 0 the dummy row); the results equal
 * the reference's bit for bit.
 *
 * cfd_compact_metrics (Grid_Transformation.cpp:22-1045, metric_term()):
 * x, y, z differentiated along every grid line by the sixth-order compact
 * scheme (alpha = 1/3, coefficients 7/9 and 1/36; one-sided 197/60 closures
 * and 2/11 rows next to the ends) with computational spacing del_zeta; det
 * of the Jacobian and the node metrics (cofactors / det) into det[] and the
 * node block of metric[] (zeta_x .. xi_z).  A line starts at a row with no
 * neighbour (index 0) in the + direction (zeta: N1, eta: N0, xi: N4 with
 * loc <= 28, 30 or 31) and follows the - neighbours to a row that has none.
 * Rows with ID 10 (the reference's C-grid wake-cut branches) ->
 * CFD_EUNSUPPORTED; a line of fewer than three rows -> CFD_EINVAL. */
cfd_status_t cfd_compact_metrics(const cfd_grid_t *grid, int32_t n_rows, double del_zeta, double *det,
                                 cfd_metric_t *metric);
/* cfd_half_point_metrics (Main.cpp:2369-2440): the six face blocks of
 * metric[] and deter[] for rows 1..n_owned by the six-point midpoint rule
 * (3, -25, 150, 150, -25, 3)/256 of the node blocks and det along each
 * direction. */
cfd_status_t cfd_half_point_metrics(const cfd_grid_t *grid, int32_t n_rows, int32_t n_owned, const double *det,
                                    cfd_metric_t *metric, cfd_determ_t *deter);

/* ------------------------------------------------------------ probes ---- */
/* A public diagnostic with no counterpart in the reference: the measured
 * FMA throughput of this device (FLOP/s, FMA = 2 FLOP; fp64 != 0 for
 * double, 0 for float), from eight independent FMA chains per thread on
 * every SM.  A
 * caller divides its own FLOP rate by it to express a kernel as a fraction
 * of the device's FP64 or FP32 peak (the FP64 roofline of the RHS path). */
cfd_status_t cfd_probe_flops(cfd_ctx_t *ctx, int32_t fp64, double *flops_per_s);
/* A public diagnostic with no counterpart in the reference: the library's
 * integer-pipe binary64 routines -- the exact FP32 -> FP64 conversion, the
 * round-to-nearest FP64 -> FP32 conversion and the double-float split
 * hi = (float)x, lo = (float)(x - hi), FP64 add, subtract and multiply
 * (the split precision form keeps its conversions off the FP64 pipe with
 * them), and the division x / b from a reciprocal shared between
 * numerators (the FP64 form) -- against the device's own instructions on
 * about n_per_class seeded operand pairs in each of six classes (everyday
 * magnitudes, the full exponent range, sparse significands that produce
 * rounding ties, zeros / subnormals / infinities / NaN / range ends, values
 * around the binary32 range, near cancellation).  mismatches[0..4] receive
 * the counts of results whose bits differ, for f2d, d2f (with the split),
 * add/sub, mul and the shared-reciprocal division (NaN matches NaN); all
 * five are 0 on a correct build. */
cfd_status_t cfd_probe_emu64(cfd_ctx_t *ctx, int64_t n_per_class, uint64_t seed, int64_t mismatches[5]);

/* ------------------------------------------- allocation-free RK3 stage -- */
/* No counterpart in the reference.  For callers that must not allocate
 * device memory while they advance a solution (a host framework that owns a
 * fixed memory pool, a real-time loop that forbids the allocation and the
 * device synchronisation cudaMalloc/cudaFree can cause, a plugin that is
 * only handed buffers): one SSP-RK3 stage j on a periodic ni x nj x nk
 * lattice, the same kernels as the resident solver's structured path, with
 * every intermediate kept in a library-owned device array sized for
 * CFD_STATIC_MAX_NODES nodes (about 27 MB per GPU that loads the library,
 * held until the process exits).  The caller passes the reference-layout
 * device buffers, rows 1..ni*nj*nk in lattice order (i fastest); det, deter
 * and metric are read; FLOW, U_j, the U the stage advances and L_out (may be
 * NULL) are written; FP64 form only (another precision -> CFD_EUNSUPPORTED).
 * Larger lattices are rejected with CFD_EINVAL.  The
 * first call on each device looks up the array's device address; make it
 * before any stream capture.  The address is kept for the process: do not
 * call the entry point after cudaDeviceReset.  A CUDA error already pending
 * on the calling thread is left in place and reported as CFD_ECUDA.  All calls share the array: calls that overlap
 * on the GPU race and must be serialised by the caller.  The call waits for
 * the stage to finish on `cuda_stream` and returns its status. */
#define CFD_STATIC_MAX_NODES 32768
cfd_status_t cfd_lattice_stage_static(void *cuda_stream, int32_t ni, int32_t nj, int32_t nk, int32_t j,
                                      double del_t, const cfd_params_t *params, const double *det,
                                      const cfd_determ_t *deter, const cfd_metric_t *metric, cfd_column_t *U0,
                                      cfd_column_t *U1, cfd_column_t *U2, cfd_flow_t *FLOW, cfd_column_t *L_out);

#ifdef __cplusplus
}
#endif
#endif /* CFD_RHS_H */

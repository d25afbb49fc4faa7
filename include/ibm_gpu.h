/*
 * ibm_gpu.h — per-timestep solver of the immersed-boundary channel flow on
 * one GB300 (hand-written sm_103a CUDA kernels behind a plain C ABI).
 *
 * This is the drop-in for the reference's hot path (main.cu:249-376): the
 * convection / momentum right-hand side, the three momentum solves, the
 * divergence / pressure right-hand side, the pressure Poisson solve, the
 * projection and the per-step diagnostics. It replaces the reference's HYPRE
 * Struct interface (hypre_struct_utils.hpp:1-26) and the HYPRE Struct GMRES /
 * Jacobi / PFMG solvers it configures (main.cu:151-221), plus the dense
 * kernels of gpu_dense_ops.hpp. Each entry point cites the call it replaces.
 *
 * Conventions (all entry points):
 *  - return IBM_OK (0) on success; IBM_NOT_CONVERGED (1) is a non-fatal
 *    warning mirroring HYPRE's error 256, which the reference accepts
 *    (common.hpp:36-43); negative values are errors. Nothing aborts.
 *  - a context owns every device buffer and one CUDA stream; all work is
 *    issued on that stream. A context is not thread-safe; distinct contexts
 *    are independent.
 *  - array arguments may be host or device pointers (detected per call);
 *    the context copies what it keeps. Field arrays use the reference's MAC
 *    layouts, x fastest (common.hpp:230-238): u (nx+1)*ny*nz, v nx*(ny+1)*nz,
 *    w nx*ny*(nz+1), p nx*ny*nz. Solve-box vectors use the Struct boxes of
 *    main.cu:151: u (nx-1)*ny*nz, v nx*(ny-1)*nz, w nx*ny*(nz-1), p nx*ny*nz.
 *  - ids are 1-based with 0 = inactive, as the reference builds them
 *    (main.cu:73-81); id-indexed vectors have length count+1, index 0 unused.
 */
#ifndef IBM_GPU_H
#define IBM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  IBM_OK = 0,
  IBM_NOT_CONVERGED = 1,      /* solve stopped above tolerance (HYPRE 256) */
  IBM_ERR_ARG = -1,
  IBM_ERR_CUDA = -2,
  IBM_ERR_NONFINITE = -3,     /* non-finite solve output (main.cu:302-305, 333-336) */
  IBM_ERR_STATE = -4,         /* a required set_* call is missing */
  IBM_ERR_NOMEM = -5,
  IBM_ERR_UNSUPPORTED = -6,   /* input not representable (e.g. off-stencil CSR entry) */
  IBM_ERR_TOO_LARGE = -7      /* problem larger than a fixed-size buffer allows */
};

enum { IBM_FIELD_U = 0, IBM_FIELD_V = 1, IBM_FIELD_W = 2, IBM_FIELD_P = 3 };

/* Grid and physics, from the reference's Params (common.hpp:45-66). */
typedef struct ibm_grid_desc {
  int nx, ny, nz;
  double Lx, Ly, Lz;
  double rho, nu, dt;
  int device;
} ibm_grid_desc;

/* Solver options (the reference's solver flags, common.hpp:68-80, plus the
 * choices this implementation adds). */
typedef struct ibm_solver_params {
  double vel_tol;        /* -vel-tol: relative residual of the momentum solves */
  int vel_maxit;         /* -vel-maxit */
  int vel_kdim;          /* -vel-kdim: GMRES restart length (<= 63) */
  int vel_jacobi_iters;  /* -vel-jacobi-iters: Jacobi sweeps per preconditioner application */
  double p_tol;          /* -p-tol */
  int p_maxit;           /* -p-maxit */
  int p_kdim;            /* -p-kdim (<= 63) */
  int p_pc;              /* pressure preconditioner: 0 Jacobi, 1 semicoarsening multigrid */
  int p_pc_maxit;        /* -p-pc-maxit: V-cycles per preconditioner application */
  int p_pc_relax_type;   /* -p-pc-relax-type: 1 weighted Jacobi, 2 red-black Gauss-Seidel */
  int p_pc_rap_type;     /* -p-pc-rap-type: 0 Galerkin (27-point coarse stencils), 1 collapsed 7-point */
  int mg_nu1, mg_nu2;    /* pre/post relaxation sweeps per level */
  double mg_omega;       /* weighted-Jacobi weight */
  int mg_coarse_max;     /* coarsen until a level has at most this many points (dense solve there) */
  int mg_max_levels;
  int use_zero_initial_guess; /* -use-zero-initial-guess (momentum) */
  int precision;         /* 0: FP64 throughout; 1: FP32 preconditioners inside FP64 flexible GMRES;
                            2: as 1 with the Arnoldi cycles in FP32 (FP32 basis and operator copy,
                            FP64 scalars), each cycle stopping after a cycle_rtol32 reduction and the
                            FP64 restart measuring the true residual (mixed-precision iterative
                            refinement): same FP64 tolerance, far fewer FP64 operations */
  int use_graph;         /* 1: replay the step as a CUDA graph */
  int vel_inner_sweeps;  /* precision 1, 2: FP32 Jacobi sweeps per momentum preconditioner application */
  double mg_group_ratio; /* between relaxed levels, coarsen every direction whose spacing is within
                            this factor of the smallest (0: one direction per relaxed level) */
  int mg_options;        /* bit 0: points with no coupling along the coarsening direction
                            interpolate constants from their coupled coarse neighbours, and the
                            7-point collapse moves no coupling onto an uncoupled (solid) point;
                            bit 1: when Ap = W S with W diagonal and S symmetric (the cut-cell
                            divergence scales rows by 1 / open fraction), build the hierarchy on
                            S and apply it to W^-1 r. 0 = PFMG's plain rules. Default 3. */
  int mg_nu_coarse;      /* sweeps each way on the relaxed levels below the finest (0: mg_nu1 / mg_nu2) */
  double cycle_rtol32;   /* precision 2: an FP32 Arnoldi cycle stops once its residual estimate fell by
                            this factor (default 1e-5, about what an FP32 basis resolves); the FP64
                            restart then measures the true residual */
  int compute_forces;    /* fill ibm_step_stats.force each step (one extra kernel): 1 staircase force,
                            2 cut-surface force (needs ibm_set_body); default 0 */
  int row_classes;       /* 1 (default): where an operator repeats few distinct rows (every fluid cell
                            away from walls and bodies has the same ones), kernels read a 2-byte class
                            per row and the row from a table of the distinct rows; results are bitwise
                            those of the plain layout. 0: plain layout */
  int mg_quads;          /* 1 (default): FP32 levels with nx % 4 == 0 relax (two-colour phases), form
                            residuals and transfer along x four points per thread (same arithmetic,
                            bitwise equal results) */
  int df_residual;       /* precision 2 with row classes, 1 (default): the true residual at each restart
                            is computed in double-float on the FP32 pipe (about 48 significant bits;
                            GB300's FP64 rate makes the FP64 stencil the bound there). 0: FP64 */
  int mg_fused_coarse;   /* FP32 multigrid with two-colour relaxation on 27-point coarse levels: the
                            coarse end of the V-cycle, from the first level below the finest with at
                            most this many points, runs as one persistent cooperative kernel per
                            V-cycle (one phase per former launch, grid-wide barriers between them;
                            bitwise the same results). 0 (default): one launch per phase; 1: from
                            the first level of at most 262144 points. Measured on the 640x128x128
                            channel: no faster (each fused phase stays bound by the latency of its
                            dependent loads plus the grid barrier, about 5 us) */
  int mg_fused_sweep;    /* 1: an FP32 7-point level's two-colour sweep (both phases) runs as one kernel
                            on shared-memory tiles with a halo, out of place (bitwise the two in-place
                            phases); 0 (default): one launch per phase. Measured on the 640x128x128
                            channel: about 96 us a sweep against 62 us for the two phases */
  int vel_precision;     /* precision of the three momentum solves (0, 1, 2 as `precision`); -1
                            (default): `precision` */
  int df_spmv;           /* precision 1 with row classes, 1 (default): the Arnoldi product A z_j of the
                            FP32 flexible basis is formed in double-float on the FP32 pipe (about 46
                            significant bits of the row's magnitude) and widened to FP64 once per row;
                            the Arnoldi dot products and everything after them stay FP64. 0: FP64 */
  int df_rhs;            /* momentum solves in precision 1 or 2, 1 (default): the convection / momentum
                            right-hand side (ibm_step, ibm_assemble_momentum) is evaluated in
                            double-float on the FP32 and integer pipes, inputs split from their FP64
                            bits, and widened to FP64 once per row (about 2^-44 of the row's largest
                            term). 0, or FP64 momentum solves: the FP64 kernel, bitwise the reference's */
  int arnoldi_passes;    /* precision 1 (FP64 flexible GMRES): classical Gram-Schmidt passes per Arnoldi
                            step, 2 (default: one re-orthogonalisation, as the FP64 form) or 1 (one
                            pass and one fewer sweep over the basis; the FP64 true residual at each
                            restart still decides convergence) */
} ibm_solver_params;

typedef struct ibm_solve_stats {
  int iters;       /* HYPRE_StructGMRESGetNumIterations */
  double rel_res;  /* HYPRE_StructGMRESGetFinalRelativeResidualNorm */
  int status;      /* IBM_OK or IBM_NOT_CONVERGED */
} ibm_solve_stats;

/* One row of the reference's per-step table (main.cu:365-368) plus timings. */
typedef struct ibm_step_stats {
  double ramp;
  ibm_solve_stats u, v, w, p;
  double div_l2, umax, vmax, wmax;
  double t_rhs_ms, t_mom_ms, t_p_ms, t_proj_ms, t_total_ms;
  int status;
  /* Force of the fluid on the body (x, y, z) from the end-of-step fields when
   * ibm_solver_params.compute_forces is set (the reference computes none):
   * pressure on the faces shared by fluid and non-fluid cells, and wall shear
   * 2 rho nu u / h on face velocities whose neighbours across a direction are
   * non-fluid (a staircase of the body, first order in h). Else 0. */
  double force[3];
} ibm_step_stats;

typedef struct ibm_ctx ibm_ctx;

/* Create a context on grid->device (replaces HYPRE_Initialize + grid/stencil
 * creation, main.cu:16-18, hypre_struct_utils.hpp:1-11). */
int ibm_create(const ibm_grid_desc *grid, ibm_ctx **out);
void ibm_destroy(ibm_ctx *ctx);
/* Text of the last error on this context (or of the last failed create). */
const char *ibm_last_error(ibm_ctx *ctx);

/* Operator of one field as the row-major 7-point Struct values the
 * reference embeds (solver_helpers.hpp:51-84, 227-329): vals[7*row + s],
 * s = C,-x,+x,-y,+y,-z,+z, on the field's solve box nbx*nby*nbz.
 * Replaces HYPRE_StructMatrixSetBoxValues (hypre_struct_utils.hpp:12-18). */
int ibm_set_operator(ibm_ctx *ctx, int field, const double *vals7, int nbx, int nby, int nbz);

/* Masks and 1-based ids (main.cu:128-139 uploads). */
int ibm_set_masks(ibm_ctx *ctx, const uint8_t *active_u, const uint8_t *active_v, const uint8_t *active_w,
                  const uint8_t *fluid_p, const uint8_t *active_qu, const uint8_t *active_qv,
                  const uint8_t *active_qw, const int32_t *id_u, const int32_t *id_v, const int32_t *id_w,
                  const int32_t *id_p, const int32_t *id_qu, const int32_t *id_qv, const int32_t *id_qw);

/* Row scales, boundary vectors (id-indexed, main.cu:140) and the inlet
 * profile uin (ny*nz, at Um; main.cu:119). Requires ibm_set_masks first. */
int ibm_set_aux(ibm_ctx *ctx, const double *scale_u, const double *scale_v, const double *scale_w,
                const double *rhs_u_bc, const double *rhs_v_bc, const double *rhs_w_bc,
                const double *div_bc_unit, const double *uin);

/* Projection operators as 1-based CSR (build_managed_csr_1based,
 * gpu_dense_ops.hpp:32-48): D is np x nq, G is nq x np, columns ascending.
 * They are converted to structured per-cell / per-face coefficients; an entry
 * that is not a face-neighbour coupling gives IBM_ERR_UNSUPPORTED. Requires
 * ibm_set_masks first. */
int ibm_set_projection_csr(ibm_ctx *ctx, const int32_t *D_rowptr, const int32_t *D_col, const double *D_val,
                           int D_nrows, const int32_t *G_rowptr, const int32_t *G_col, const double *G_val,
                           int G_nrows);

/* GPU assembly of the three momentum operators (immersed_operators.hpp:1-177,
 * row-scaled as main.cu:98-100) from the active masks and 1-based ids of the
 * u, v, w faces (full MAC layouts, as ibm_set_masks takes them; host or
 * device pointers) and the cylinder (centre, radius), with the context's
 * grid, rho, nu and dt. Every row and row scale is bitwise the CPU setup's.
 * The operators are set on the context as ibm_set_operator sets them;
 * vals_out[f] (the row-major [box rows][7] values) and scale_out[f] (the
 * id-indexed row scales, max id + 1 values, index 0 = 1) are written when
 * the arrays and their entries are not NULL (host or device pointers).
 * When ibm_set_aux has been called and the ids match the context's, the
 * new row scales also replace the context's right-hand-side scales, so the
 * next step scales its right-hand sides as the new rows are scaled; with
 * other ids, call ibm_set_aux with scale_out before the next step. */
int ibm_assemble_momentum(ibm_ctx *ctx, double xcirc, double ycirc, double Rcirc, const uint8_t *const *active,
                          const int32_t *const *id, double *const *vals_out, double *const *scale_out);

/* GPU assembly of the sign-flipped pressure operator -D G
 * (immersed_operators.hpp:179-250, main.cu:101-103) from the cells' fluid
 * mask, ids and open fractions beta_p (nx*ny*nz) and the faces' open
 * fractions alpha[3], q-face masks active_q[3] and q ids id_q[3] (full MAC
 * layouts; host or device pointers), with the context's grid. Bitwise the
 * CPU setup's rows; set on the context as ibm_set_operator sets them and
 * written to vals_out (row-major [nx*ny*nz][7]) when it is not NULL. */
int ibm_assemble_pressure(ibm_ctx *ctx, const uint8_t *fluid_p, const int32_t *id_p, const double *beta_p,
                          const double *const *alpha, const uint8_t *const *active_q, const int32_t *const *id_q,
                          double *vals_out);

/* The body for the cut-surface force (compute_forces = 2); the reference
 * computes no force. Cylinder centre and radius as the geometry code takes
 * them (common.hpp:64-66) and the open fractions of the u and v faces
 * (alpha_u, alpha_v: full MAC layouts, host or device pointers; the
 * fractions immersed_geometry.hpp:29-73 computes, extruded in z). The shear
 * is the wall flux the momentum operators apply where a row meets the body
 * (rho nu u_P / d_P over the control-volume face, d_P from
 * segmentCircleDistance, immersed_operators.hpp:1-177); the pressure acts
 * on each fluid cell's cut surface, -sum_f alpha_f A_f n_f, with faces
 * towards non-fluid cells closed. Requires ibm_set_masks; a later
 * ibm_set_masks drops the body. */
int ibm_set_body(ibm_ctx *ctx, double xcirc, double ycirc, double Rcirc, const double *alpha_u,
                 const double *alpha_v);

/* Solver configuration (main.cu:173-221). */
void ibm_solver_params_default(ibm_solver_params *p);
int ibm_set_solver_params(ibm_ctx *ctx, const ibm_solver_params *p);
int ibm_get_solver_params(ibm_ctx *ctx, ibm_solver_params *p);

/* State fields (full MAC layouts). Either pointer may be NULL to skip it. */
int ibm_set_fields(ibm_ctx *ctx, const double *u, const double *v, const double *w, const double *p);
int ibm_get_fields(ibm_ctx *ctx, double *u, double *v, double *w, double *p);

/* One timestep with inlet ramp factor `ramp` (main.cu:249-368). Returns the
 * worst status of the four solves, or an error. */
int ibm_step(ibm_ctx *ctx, double ramp, ibm_step_stats *stats);

/* One solve on a field's solve box: x is the initial guess in, the solution
 * out (HYPRE_StructGMRESSolve, main.cu:284-286, 327). */
int ibm_solve(ibm_ctx *ctx, int field, const double *b, double *x, ibm_solve_stats *stats);

/* y = A x with the field's operator on its solve box (HYPRE StructMatvec). */
int ibm_apply_operator(ibm_ctx *ctx, int field, const double *x, double *y);

/* z = M r: one application of the field's preconditioner from a zero guess,
 * as the solver applies it (HYPRE_StructPFMGSolve / HYPRE_StructJacobiSolve
 * with maxit 1, main.cu:182, 212-218). precision 1 or 2 applies the FP32 form. */
int ibm_apply_preconditioner(ibm_ctx *ctx, int field, const double *r, double *z);

/* The last right-hand side (which = 0) or solution (which = 1) of a field's
 * solve box, as HYPRE_StructVectorGetBoxValues returns the reference's
 * b/x vectors (hypre_struct_utils.hpp:23-24, main.cu:298-300, 332). */
int ibm_get_solver_vector(ibm_ctx *ctx, int field, int which, double *out);

/* Launch accounting (replaces the reference's MPI_Wtime buckets,
 * main.cu:247-389, with per-kernel-class counts, algorithmic bytes — every
 * element a kernel must read or write once — and CUDA-event time of one
 * selected class). Phases: right-hand sides, momentum solves, pressure
 * solve, projection, other. */
#define IBM_PROFILE_MAX_KERNELS 32
typedef struct ibm_profile {
  int nkernels;
  long long launches[IBM_PROFILE_MAX_KERNELS];
  double bytes[IBM_PROFILE_MAX_KERNELS];
  double time_ms[IBM_PROFILE_MAX_KERNELS];
  long long timed_launches[IBM_PROFILE_MAX_KERNELS];
  double phase_bytes[5];
} ibm_profile;
int ibm_profile_reset(ibm_ctx *ctx);
/* Bracket every launch of kernel class `kernel` with CUDA events on the
 * context stream (-1: none). */
int ibm_profile_time_kernel(ibm_ctx *ctx, int kernel);
int ibm_profile_get(ibm_ctx *ctx, ibm_profile *out);
const char *ibm_kernel_name(int kernel);

/* Batching extension (independent channels stepped together; the reference
 * runs one channel per process, main.cu:249-376). Each instance is a full
 * context with its own stream: set its inputs and parameters with the ibm_*
 * calls on ibm_batch_ctx(b, i). ibm_batch_step queues one step of every
 * instance before waiting for any, so instances in graph mode (use_graph)
 * run concurrently on the GPU; host-driven instances step one after the
 * other. Each instance's results equal ibm_step's on that context alone. */
typedef struct ibm_batch ibm_batch;
int ibm_batch_create(int n, const ibm_grid_desc *grids, ibm_batch **out);
void ibm_batch_destroy(ibm_batch *b);
int ibm_batch_size(const ibm_batch *b);
ibm_ctx *ibm_batch_ctx(ibm_batch *b, int i);
/* ramps[n]; stats[n] (may be NULL). Returns the worst instance status
 * (IBM_OK < IBM_NOT_CONVERGED < errors: the first negative code); the
 * instance's own code is in stats[i].status and its message in
 * ibm_last_error(ibm_batch_ctx(b, i)). */
int ibm_batch_step(ibm_batch *b, const double *ramps, ibm_step_stats *stats);

/* Adjoint extension (the reference has none; its inputs are the ones
 * main.cu:249-376 steps with). The step is s1 = step(s0; g, nu), with
 *  - g[ny*nz] the inflow profile (y fastest): u at the inlet = ramp g in
 *    every BC cleanup (main.cu:250-251) and the inlet column's divergence
 *    lift div_bc = -g / (beta dx) (immersed_operators.hpp:223-228); the
 *    implicit-diffusion lift rhs_u_bc keeps the reference's unit base
 *    profile, as the reference builds it (immersed_operators.hpp:26);
 *  - nu the viscosity, on which the momentum operators, their row scales and
 *    rhs_u_bc depend (immersed_operators.hpp:1-177, main.cu:98-100).
 * The objective is a weighted sum over steps of the x force (drag) that
 * ibm_step_stats.force reports. ibm_step_backward maps the lambda of a
 * step's end-of-step fields (held in the context) to the lambda of its
 * step-start fields and accumulates dJ/dg and dJ/dnu; the transposed solves
 * (A^T y = c for the three momentum operators and the pressure operator)
 * run on a second context built on the transposed stencils, with the
 * solver parameters of this one. */
/* Builds the transposed-operator context and the inlet weights from beta_p
 * (cell open fractions, nx*ny*nz); clears lambdas, gradients and the tape.
 * Requires every input of ibm_step; call again after changing an operator. */
int ibm_adjoint_setup(ibm_ctx *ctx, const double *beta_p);
/* Sets the inflow profile g (host or device pointer): the inlet values and
 * the inlet column's divergence lift, computed as the setup computes them
 * (bitwise the setup's arrays when g is its uin). */
int ibm_set_inflow(ibm_ctx *ctx, const double *g);
/* ibm_step that also pushes the step onto the context's tape (device
 * memory): its start and end fields and its momentum right-hand sides and
 * solutions, what the reverse step needs of the forward computation. */
int ibm_step_forward(ibm_ctx *ctx, double ramp, ibm_step_stats *stats);
/* Pops the last taped step (the context then holds its end-of-step fields;
 * stats are the taped step's), adds weight * dF_x/d(end-of-step fields) to
 * the lambdas, and runs the reverse sweep. `ramp` must be the taped step's
 * own (IBM_ERR_ARG otherwise). */
int ibm_step_backward(ibm_ctx *ctx, double ramp, double weight, ibm_step_stats *stats);
/* Lambdas, dJ/dg and dJ/dnu to zero; tape emptied. */
int ibm_adjoint_reset(ibm_ctx *ctx);
/* Lambdas of the state (full MAC arrays and cells; NULL = zero). */
int ibm_adjoint_set(ibm_ctx *ctx, const double *lu, const double *lv, const double *lw, const double *lp);
/* Lambdas, dJ/dg[ny*nz] and dJ/dnu[1]; any pointer may be NULL. */
int ibm_adjoint_get(ibm_ctx *ctx, double *lu, double *lv, double *lw, double *lp, double *dg, double *dnu);
/* The transposed solves of the last reverse sweep: out[4] = u, v, w, p. */
int ibm_adjoint_solve_stats(ibm_ctx *ctx, ibm_solve_stats *out);
int ibm_adjoint_tape_depth(ibm_ctx *ctx);
/* Checkpoints of the state fields in device memory, by slot number, for
 * checkpointing with recomputation across many steps. */
int ibm_checkpoint_save(ibm_ctx *ctx, int slot);
int ibm_checkpoint_load(ibm_ctx *ctx, int slot);
int ibm_checkpoint_clear(ibm_ctx *ctx);

int ibm_synchronize(ibm_ctx *ctx);
void *ibm_stream(ibm_ctx *ctx);            /* the context's cudaStream_t */
long long ibm_kernel_launches(ibm_ctx *ctx); /* kernels this context has launched */
/* Name and compute capability of a device, for logs. */
int ibm_device_query(int device, char *buf, int len);

/* r = b - A x and norms[0] = ||r||_2, norms[1] = ||b||_2 for one 7-point
 * operator, allocating nothing. No counterpart in the reference: it serves
 * callers that cannot call cudaMalloc (those that give all device memory to
 * their own pool allocator, run under a fixed memory budget, or cannot take
 * the device-wide synchronisation of cudaFree), for whom creating a context
 * is not an option.
 *  - vals (7 values per row, the reference's row-major Struct layout, as
 *    ibm_set_operator takes), x, b, r (nx*ny*nz doubles each) and norms (2
 *    doubles) are caller-owned device (or managed) memory on the current
 *    device; host pointers are rejected with IBM_ERR_ARG.
 *  - nx*ny*nz above IBM_NOALLOC_MAX_ROWS returns IBM_ERR_TOO_LARGE.
 *  - r and norms must not share memory with vals, x, b or each other
 *    (IBM_ERR_ARG): r = x in place would race, since other rows still read
 *    x while r is written.
 *  - scratch is one fixed array inside the library (512 KiB per device,
 *    held until the process exits). Each call made outside stream capture
 *    looks up the array's address in the current context
 *    (cudaGetSymbolAddress), so calls after cudaDeviceReset, or with another
 *    context of the device made current, use the right address; a call
 *    made during capture reuses the address the last uncaptured call on
 *    that device found. Make the first call on a device before any stream
 *    capture, and make one uncaptured call again after a device reset
 *    before capturing.
 *  - work is queued on `stream` (a cudaStream_t; NULL = default stream) and
 *    the call returns without waiting: r and norms are valid once the stream
 *    has reached this point. Every call shares the array, which keeps the
 *    last call's contents; the counter that must start at zero is cleared on
 *    the stream before each launch. Calls whose work overlaps on the GPU
 *    (other streams, other host threads) race on the array: order them. */
#define IBM_NOALLOC_MAX_ROWS 33554432L /* 2^25 rows */
int ibm_residual_noalloc(const double *vals, int nx, int ny, int nz, const double *x, const double *b,
                         double *r, double *norms, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* IBM_GPU_H */

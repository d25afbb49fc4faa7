/*
 * ibm_oracle.h — CPU oracle for the per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker the CUDA path is compared
 * against; nothing in the product links, loads or calls it. It restates the
 * reference's timestep (main.cu:249-368) and dense kernels
 * (gpu_dense_ops.hpp:1-106) in plain C, with the linear solves done by the
 * oracle's own FP64 restarted GMRES (Jacobi or semicoarsening multigrid
 * preconditioning), restating the algorithm of HYPRE's Struct GMRES / Jacobi /
 * PFMG, which the reference calls but does not vendor (version unpinned).
 *
 * Pins: the setup arrays it consumes are bit-identical to the reference's
 * own (checked through the reference compiled from its sources); the BC and
 * convection restatements are bit-identical to the reference's CPU twins
 * (immersed_operators.hpp:990-1053); solve outputs are checked by their
 * residual against the reference-identical operators.
 */
#ifndef IBM_ORACLE_H
#define IBM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_params {
  int nx, ny, nz;
  double Lx, Ly, Lz, rho, nu, dt;
  int use_zero_initial_guess;
  double vel_tol; int vel_maxit, vel_kdim, vel_jacobi_iters;
  double p_tol; int p_maxit, p_kdim;
  int p_pc;            /* 0: Jacobi, 1: semicoarsening multigrid V-cycle */
  int mg_rap;          /* 0: Galerkin (27-point coarse stencils), 1: collapsed to 7 points */
  int mg_relax;        /* 1: weighted Jacobi, 2: red-black Gauss-Seidel */
  int mg_nu1, mg_nu2;  /* pre/post smoothing sweeps */
  double mg_omega;     /* weighted-Jacobi weight */
  int mg_coarse_max;   /* stop coarsening at or below this many points */
  int mg_max_levels;
  double mg_group_ratio; /* coarsen every direction with spacing <= ratio * smallest between
                            relaxations (0: one direction per relaxed level) */
  int mg_options;      /* bit 0: points with no coupling along the coarsening direction
                          interpolate the constant from their coupled coarse neighbours
                          (plain operator-dependent weights give them 0);
                          bit 1: hierarchy of S = W^-1 Ap, where Ap = W S with W diagonal
                          and S symmetric (found from the couplings), applied to W^-1 r */
  int mg_nu_coarse;    /* sweeps each way on relaxed levels below the finest (0: mg_nu1 / mg_nu2) */
} oracle_params;

typedef struct oracle_inputs {
  const double *Au, *Av, *Aw, *Ap; /* row-major [box rows][7]: C,-x,+x,-y,+y,-z,+z */
  const uint8_t *active_u, *active_v, *active_w, *fluid_p, *active_qu, *active_qv, *active_qw;
  const int32_t *id_u, *id_v, *id_w, *id_p, *id_qu, *id_qv, *id_qw;
  const double *scale_u, *scale_v, *scale_w, *rhs_u_bc, *rhs_v_bc, *rhs_w_bc, *div_bc_unit;
  const int32_t *D_rowptr, *D_col; const double *D_val;
  const int32_t *G_rowptr, *G_col; const double *G_val;
  const double *uin; /* ny*nz, inlet profile at Um */
} oracle_inputs;

typedef struct oracle_solve_stats { int iters; double rel_res; int status; } oracle_solve_stats;

typedef struct oracle_step_stats {
  oracle_solve_stats u, v, w, p;
  double div_l2, umax, vmax, wmax;
  int status;
  double force[3];   /* force of the fluid on the body, staircase definition (see oracle_forces) */
} oracle_step_stats;

typedef struct oracle oracle;

/* The oracle keeps the input pointers (no copy): they must outlive it. */
oracle *oracle_create(const oracle_params *prm, const oracle_inputs *in);
void oracle_destroy(oracle *o);
void oracle_set_fields(oracle *o, const double *u, const double *v, const double *w, const double *p);
void oracle_get_fields(const oracle *o, double *u, double *v, double *w, double *p);
int oracle_step(oracle *o, double ramp, oracle_step_stats *st);
/* Force of the fluid on the body from the current fields (the step fills st->force). */
void oracle_forces(const oracle *o, double f[3]);
/* Switch oracle_forces (and the adjoint's drag seed) to the cut-surface
 * force of the cylinder (xcirc, ycirc, Rcirc) with the u and v faces' open
 * fractions (full MAC layouts; copied). */
void oracle_set_body(oracle *o, double xcirc, double ycirc, double Rcirc, const double *alpha_u,
                     const double *alpha_v);

/* Pieces of the step, for kernel-level checks. */
void oracle_bc_cleanup(const oracle *o, double *u, double *v, double *w, const double *uin_step);
void oracle_convection(const oracle *o, const double *u, const double *v, const double *w,
                       double *cu, double *cv, double *cw);
void oracle_momentum_rhs(const oracle *o, const double *u, const double *v, const double *w, const double *p,
                         double *bu, double *bv, double *bw);
void oracle_pressure_rhs(const oracle *o, const double *ut, const double *vt, const double *wt, double ramp,
                         double *bp);
void oracle_tilde(const oracle *o, const double *xu, const double *xv, const double *xw, double ramp,
                  double *ut, double *vt, double *wt);
void oracle_projection(oracle *o, const double *ut, const double *vt, const double *wt, const double *xp,
                       double ramp, oracle_step_stats *st);
/* field: 0 u, 1 v, 2 w, 3 p. y = A x on the field's solve box. */
void oracle_apply_operator(const oracle *o, int field, const double *x, double *y);
int oracle_solve(oracle *o, int field, const double *b, double *x, oracle_solve_stats *st);
/* Multigrid hierarchy of the pressure operator (built on first use). */
int oracle_mg_levels(oracle *o);
int oracle_mg_level_info(oracle *o, int l, int *dims /*3*/, int *cdir, int *nslots);
int oracle_mg_level_coef(oracle *o, int l, double *coef /* [n][27] */);
void oracle_mg_vcycle(oracle *o, const double *b, double *x);

/*
 * Adjoint extension (the reference has none): reverse sweep of one step.
 * o holds the step-start fields on entry and again on return (the step is
 * recomputed from them); ot is an oracle on the transposed operators with the
 * same parameters, used for the transposed solves; beta_p (cell open
 * fractions) gives the inlet column's divergence lift, d(div_bc)/dg =
 * -1/(beta dx). On entry (lu, lv, lw, lp) is the lambda of the end-of-step
 * fields, to which weight * dF_x/d(end-of-step fields) is added (F_x the drag
 * of oracle_forces); on return it is the lambda of the step-start fields.
 * dg[ny*nz] (the inflow profile, u at the inlet = ramp g) and *dnu
 * accumulate the parameter gradient. Returns 0, or -3 when a solve failed.
 */
int oracle_step_backward(oracle *o, oracle *ot, double ramp, const double *beta_p, double weight, double *lu,
                         double *lv, double *lw, double *lp, double *dg, double *dnu);

#ifdef __cplusplus
}
#endif
#endif

/*
 * ibm_host.h — host-side (CPU) setup of the immersed-boundary channel case.
 *
 * Produces, once per case, every array the per-timestep solver consumes:
 * cut-cell fractions, active masks, 1-based active ids, the row-scaled
 * momentum operators and the sign-flipped pressure operator embedded in the
 * 7-point row-major Struct layout, the row scales and boundary vectors, and
 * the projection operators D and G as 1-based CSR.
 *
 * Replaces the reference's setup (main.cu:20-149): geometry
 * (immersed_geometry.hpp:1-167), assembly (immersed_operators.hpp:1-287,
 * 737-748), row-major embedding (solver_helpers.hpp:51-84, 227-329) and the
 * CSR build (gpu_dense_ops.hpp:32-48). Results are bit-identical to the
 * reference's on the same Params (checked by the test suite).
 *
 * Conventions: return 0 on success, negative on error; never aborts.
 */
#ifndef IBM_HOST_H
#define IBM_HOST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Geometry / physics subset of the reference's Params (common.hpp:45-66). */
typedef struct ibm_case_params {
  int nx, ny, nz;          /* pressure cells */
  double Lx, Ly, Lz;       /* channel extents */
  double rho, nu, Um, dt;  /* density, viscosity, inlet peak velocity, time step */
  int nsub_beta;           /* sub-samples per direction for cell open fractions */
  double beta_tol;         /* a cell is fluid when its open fraction exceeds this */
  double alpha_tol;        /* a face carries flux when its open fraction exceeds this */
  double xcirc, ycirc, Rcirc; /* cylinder centre and radius (full height in z) */
} ibm_case_params;

/* Active counts (the reference's Nu, Nv, Nw, Np, Nqu, Nqv, Nqw; main.cu:86-88). */
typedef struct ibm_case_counts {
  int nu, nv, nw, np, nqu, nqv, nqw;
  int n_pruned; /* fluid x-y columns removed as disconnected (immersed_geometry.hpp:117-160) */
} ibm_case_counts;

typedef struct ibm_case ibm_case;

/* Fill p with the reference defaults for the fields above (common.hpp:45-66). */
void ibm_case_params_default(ibm_case_params *p);

/* Build every setup array for p. On success *out owns them. */
int ibm_case_build(const ibm_case_params *p, ibm_case **out);
void ibm_case_free(ibm_case *c);
int ibm_case_get_counts(const ibm_case *c, ibm_case_counts *out);

/*
 * Named arrays (full MAC layouts are x-fastest; "box" layouts are the solve
 * boxes of the reference's Struct grids):
 *   beta_p f64[nx*ny*nz]   alpha_u f64[(nx+1)*ny*nz]  alpha_v f64[nx*(ny+1)*nz]  alpha_w f64[nx*ny*(nz+1)]
 *   fluid_p, active_u, active_v, active_w, active_qu, active_qv, active_qw  u8 (same layouts)
 *   id_u, id_v, id_w, id_p, id_qu, id_qv, id_qw  i32 (1-based, 0 = inactive)
 *   scale_u f64[nu+1], scale_v f64[nv+1], scale_w f64[nw+1]   (index 0 unused)
 *   rhs_u_bc f64[nu+1], rhs_v_bc f64[nv+1], rhs_w_bc f64[nw+1], div_bc_unit f64[np+1]
 *   Au_vals f64[(nx-1)*ny*nz*7], Av_vals f64[nx*(ny-1)*nz*7], Aw_vals f64[nx*ny*(nz-1)*7],
 *   Ap_vals f64[nx*ny*nz*7]   (entry-fastest: C, -x, +x, -y, +y, -z, +z)
 *   uin f64[ny*nz]  (inlet profile at Um)
 *   D_rowptr i32[np+1], D_col i32[nnz], D_val f64[nnz]   (1-based columns, sorted)
 *   G_rowptr i32[nq+1], G_col i32[nnz], G_val f64[nnz]
 * Returns the byte size (and element size) or -1 when the name is unknown.
 */
long ibm_case_array_bytes(const ibm_case *c, const char *name, int *elem_size);
const void *ibm_case_array(const ibm_case *c, const char *name);

/*
 * Case cache on disk: a versioned binary of every named array, keyed by the
 * full parameter struct. ibm_case_load returns 0 when the file holds a case
 * built with exactly *p, 1 when the file is absent or for other parameters
 * or another format version (nothing is loaded), negative on I/O errors.
 * ibm_case_build_cached loads when it can, else builds and saves.
 */
int ibm_case_save(const ibm_case *c, const char *path);
int ibm_case_load(const ibm_case_params *p, const char *path, ibm_case **out);
int ibm_case_build_cached(const ibm_case_params *p, const char *path, ibm_case **out);

/*
 * Field output in the reference's VTK format (write_vtk_cellcentered,
 * immersed_operators.hpp:1055-1076): legacy ASCII STRUCTURED_POINTS with
 * cell data ux, uy, uz (face averages), pressure and fluid_mask, values as
 * %.16e. Returns 0, -1 on bad arguments, -2 on I/O errors.
 * ibm_vtk_step_name gives the reference's per-step name (base stem +
 * "_%06d" + extension, solver_helpers.hpp:470-482) and returns its length.
 */
int ibm_write_vtk(const char *path, const double *u, const double *v, const double *w, const double *p,
                  const uint8_t *fluid_p, int nx, int ny, int nz, double Lx, double Ly, double Lz);
int ibm_vtk_step_name(const char *base, int step, char *out, int len);

/*
 * Self-check of the hash-iteration-order model used to reproduce the
 * reference's summation order: inserts ntrials random key sets into the real
 * standard-library hash map this library was compiled with and compares the
 * iteration order with the model. Returns the number of mismatches.
 */
int ibm_host_check_sum_order(int ntrials, unsigned seed);

#ifdef __cplusplus
}
#endif
#endif /* IBM_HOST_H */

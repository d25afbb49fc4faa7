// Test-only checker: the reference's own device kernels (gpu_dense_ops.hpp),
// compiled from its original location into a cubin (oracle/Makefile, target
// refcubin; output oracle/_ref/ref_kernels.cubin) that the tests load through
// the CUDA driver API and launch in the order of the reference's timestep
// (main.cu:249-351). Nothing in the product links or loads this file.
//
// The headers around gpu_dense_ops.hpp are the ones the reference's main.cu
// includes with it, in its order (main.cu:1-6): the header needs the ones
// before it, and its last function is completed by solver_helpers.hpp.
//
// The reference declares its kernels `__global__ static`, which a driver-API
// caller cannot look up by name. While its header is included, __global__ is
// read as __device__, so each kernel becomes a device function with the same
// body; the extern "C" kernels below call it unchanged, launched with the
// reference's own block size and grid, so every thread computes exactly what
// the reference's launch computes (the bodies index by blockIdx/threadIdx).
#include "common.hpp"
#include "immersed_geometry.hpp"
#include "immersed_operators.hpp"
#include "hypre_struct_utils.hpp"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
#include "gpu_dense_ops.hpp"
#include "solver_helpers.hpp"
#pragma pop_macro("__global__")

typedef unsigned char u8;

extern "C" {

__global__ void ref_apply_bc_cleanup(double *u, double *v, double *w, const u8 *au, const u8 *av, const u8 *aw,
                                     const double *uin_step, int nx, int ny, int nz) {
  k_apply_bc_cleanup(u, v, w, au, av, aw, uin_step, nx, ny, nz);
}
__global__ void ref_conv_u(double *conv, const double *u, const double *v, const double *w, const u8 *a, int nx,
                           int ny, int nz, double dx, double dy, double dz) {
  k_conv_u(conv, u, v, w, a, nx, ny, nz, dx, dy, dz);
}
__global__ void ref_conv_v(double *conv, const double *u, const double *v, const double *w, const u8 *a, int nx,
                           int ny, int nz, double dx, double dy, double dz) {
  k_conv_v(conv, u, v, w, a, nx, ny, nz, dx, dy, dz);
}
__global__ void ref_conv_w(double *conv, const double *u, const double *v, const double *w, const u8 *a, int nx,
                           int ny, int nz, double dx, double dy, double dz) {
  k_conv_w(conv, u, v, w, a, nx, ny, nz, dx, dy, dz);
}
__global__ void ref_build_u_full(double *rhsf, double *x0, const double *u, const double *conv, const double *gp,
                                 const u8 *a, const int *id, const double *rhs_bc, const double *scale, int nx,
                                 int ny, int nz, double rho, double dt, int zero) {
  k_build_u_full(rhsf, x0, u, conv, gp, a, id, rhs_bc, scale, nx, ny, nz, rho, dt, zero);
}
__global__ void ref_build_v_full(double *rhsf, double *x0, const double *v, const double *conv, const double *gp,
                                 const u8 *a, const int *id, const double *rhs_bc, const double *scale, int nx,
                                 int ny, int nz, double rho, double dt, int zero) {
  k_build_v_full(rhsf, x0, v, conv, gp, a, id, rhs_bc, scale, nx, ny, nz, rho, dt, zero);
}
__global__ void ref_build_w_full(double *rhsf, double *x0, const double *w, const double *conv, const double *gp,
                                 const u8 *a, const int *id, const double *rhs_bc, const double *scale, int nx,
                                 int ny, int nz, double rho, double dt, int zero) {
  k_build_w_full(rhsf, x0, w, conv, gp, a, id, rhs_bc, scale, nx, ny, nz, rho, dt, zero);
}
__global__ void ref_scatter_u(double *uo, const double *x, const double *base, int nx, int ny, int nz) {
  k_scatter_u(uo, x, base, nx, ny, nz);
}
__global__ void ref_scatter_v(double *vo, const double *x, const double *base, int nx, int ny, int nz) {
  k_scatter_v(vo, x, base, nx, ny, nz);
}
__global__ void ref_scatter_w(double *wo, const double *x, const double *base, int nx, int ny, int nz) {
  k_scatter_w(wo, x, base, nx, ny, nz);
}
__global__ void ref_spmv_csr_1based(int nrows, const int *rowptr, const int *colind, const double *vals,
                                    const double *x, double *y) {
  k_spmv_csr_1based(nrows, rowptr, colind, vals, x, y);
}
__global__ void ref_pack_pressure_active(double *vec, const double *p, const u8 *fluid, const int *id_p, int n) {
  k_pack_pressure_active(vec, p, fluid, id_p, n);
}
__global__ void ref_unpack_gp_u(const double *gp, double *gpx, const int *id_qu, int nx, int ny, int nz) {
  k_unpack_gp_u(gp, gpx, id_qu, nx, ny, nz);
}
__global__ void ref_unpack_gp_v(const double *gp, double *gpy, const int *id_qv, int nx, int ny, int nz, int nqu) {
  k_unpack_gp_v(gp, gpy, id_qv, nx, ny, nz, nqu);
}
__global__ void ref_unpack_gp_w(const double *gp, double *gpz, const int *id_qw, int nx, int ny, int nz, int nqu,
                                int nqv) {
  k_unpack_gp_w(gp, gpz, id_qw, nx, ny, nz, nqu, nqv);
}
__global__ void ref_pack_projection_q_u(double *q, const double *u, const int *id_qu, int nx, int ny, int nz) {
  k_pack_projection_q_u(q, u, id_qu, nx, ny, nz);
}
__global__ void ref_pack_projection_q_v(double *q, const double *v, const int *id_qv, int nx, int ny, int nz,
                                        int nqu) {
  k_pack_projection_q_v(q, v, id_qv, nx, ny, nz, nqu);
}
__global__ void ref_pack_projection_q_w(double *q, const double *w, const int *id_qw, int nx, int ny, int nz,
                                        int nqu, int nqv) {
  k_pack_projection_q_w(q, w, id_qw, nx, ny, nz, nqu, nqv);
}
__global__ void ref_build_pressure_rhs_full(double *rhsf, double *x0, const double *dqt, const double *div_bc_unit,
                                            const u8 *fluid, const int *id_p, int n, double rho, double dt,
                                            double ramp) {
  k_build_pressure_rhs_full(rhsf, x0, dqt, div_bc_unit, fluid, id_p, n, rho, dt, ramp);
}
__global__ void ref_pack_phi_active(double *phi, const double *xp, const u8 *fluid, const int *id_p, int n) {
  k_pack_phi_active(phi, xp, fluid, id_p, n);
}
__global__ void ref_apply_q_correction(double *q, const double *gphi, double factor, int nplus1) {
  k_apply_q_correction(q, gphi, factor, nplus1);
}
__global__ void ref_unpack_projection_q_u(const double *q, double *u, const int *id_qu, int nx, int ny, int nz) {
  k_unpack_projection_q_u(q, u, id_qu, nx, ny, nz);
}
__global__ void ref_unpack_projection_q_v(const double *q, double *v, const int *id_qv, int nx, int ny, int nz,
                                          int nqu) {
  k_unpack_projection_q_v(q, v, id_qv, nx, ny, nz, nqu);
}
__global__ void ref_unpack_projection_q_w(const double *q, double *w, const int *id_qw, int nx, int ny, int nz,
                                          int nqu, int nqv) {
  k_unpack_projection_q_w(q, w, id_qw, nx, ny, nz, nqu, nqv);
}
__global__ void ref_add_pressure_phi(double *p, const double *phi, const u8 *fluid, const int *id_p, int n) {
  k_add_pressure_phi(p, phi, fluid, id_p, n);
}

}  // extern "C"

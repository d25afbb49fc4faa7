/*
 * ibm_oracle.c — CPU oracle for the per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (see ibm_oracle.h).
 * Only tests, the smoke check and the benchmark's CPU-baseline leg load it.
 *
 * Floating-point evaluation order is spelled out explicitly (fma() where a
 * fused multiply-add is meant, separate operations otherwise) and the file is
 * built with -ffp-contract=off, so the results are the same on every host.
 * Dot products are summed over fixed 4096-row chunks, then the chunk sums in
 * order, so results do not depend on the thread count.
 */
#include "ibm_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define CHUNK 4096L

typedef struct { int n[3]; long N; } box3;

typedef struct {
  box3 b;
  int cdir;                 /* direction coarsened to reach the next level, -1 on the coarsest */
  int relax;                /* 0 inside a coarsening group: restrict / interpolate only */
  double *A;                /* [N][27], slot = (ox+1) + 3(oy+1) + 9(oz+1) */
  double *wd;               /* omega / diag */
  double *invd;             /* 1 / diag */
  double *pm, *pp;          /* interpolation weights at points odd along cdir */
  double *bv, *xv, *rv;     /* work vectors */
  double *dense_inv;        /* coarsest: explicit inverse [N][N] */
  int ns;                   /* slots of A that are nonzero somewhere on the level */
  int slot[27];             /* those slots, in increasing slot order */
  double *Ac;               /* [N][ns]: A restricted to those slots */
} mg_level;

struct oracle {
  oracle_params prm;
  oracle_inputs in;
  int nx, ny, nz;
  double dx, dy, dz;
  int nU, nV, nW, nP, nQu, nQv, nQw, nQ;
  box3 bu, bv, bw, bp;
  double *u, *v, *w, *p;
  double *invd[4];          /* Jacobi inverse diagonals of the four operators */
  int mg_built;
  int mg_sym;               /* the hierarchy is built on W^-1 Ap */
  double *mg_winv;          /* 1 / W (ones when not symmetrized) */
  int nlev;
  mg_level lev[40];
  /* the body, for the cut-surface force (oracle_set_body) */
  int body_set;
  double xcirc, ycirc, Rcirc;
  double *alpha_u, *alpha_v;
};

/* ------------------------------------------------------------------------ */
/* small helpers                                                             */
/* ------------------------------------------------------------------------ */
static void *xcalloc(size_t n, size_t s) {
  void *p = calloc(n ? n : 1, s);
  if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
  return p;
}
static int max_id(const int32_t *id, long n) {
  int m = 0;
  for (long i = 0; i < n; ++i) if (id[i] > m) m = id[i];
  return m;
}
static double dot(const double *a, const double *b, long n) {
  long nch = (n + CHUNK - 1) / CHUNK;
  double *part = (double *)xcalloc((size_t)nch, sizeof(double));
#pragma omp parallel for schedule(static)
  for (long c = 0; c < nch; ++c) {
    long lo = c * CHUNK, hi = lo + CHUNK < n ? lo + CHUNK : n;
    double s = 0.0;
    for (long i = lo; i < hi; ++i) s = fma(a[i], b[i], s);
    part[c] = s;
  }
  double s = 0.0;
  for (long c = 0; c < nch; ++c) s += part[c];
  free(part);
  return s;
}
/* out[k] = dot(V + k N, w, N) for k < m, each summed exactly as dot() sums
 * (per-chunk fused multiply-adds in index order, chunks in order), in one
 * pass over w. */
static void multi_dot(const double *V, long N, int m, const double *w, double *out) {
  long nch = (N + CHUNK - 1) / CHUNK;
  double *part = (double *)xcalloc((size_t)nch * (size_t)(m ? m : 1), sizeof(double));
#pragma omp parallel for schedule(static)
  for (long c = 0; c < nch; ++c) {
    long lo = c * CHUNK, hi = lo + CHUNK < N ? lo + CHUNK : N;
    for (int k = 0; k < m; ++k) {
      const double *a = V + (size_t)k * N;
      double s = 0.0;
      for (long i = lo; i < hi; ++i) s = fma(a[i], w[i], s);
      part[(size_t)k * nch + c] = s;
    }
  }
  for (int k = 0; k < m; ++k) {
    double s = 0.0;
    for (long c = 0; c < nch; ++c) s += part[(size_t)k * nch + c];
    out[k] = s;
  }
  free(part);
}
/* w[t] -= sum_k h[k] V_k[t] for t in each chunk (k ascending), then, in the
 * same pass, the chunk's partial products V_k . w (part_dots[k nch + c]) or
 * w . w (part_norm[c]) of the updated w, each summed as dot() sums a chunk. */
static void orth_update(const double *V, long N, int m, const double *h, double *w, double *part_dots,
                        double *part_norm) {
  long nch = (N + CHUNK - 1) / CHUNK;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < nch; ++c) {
    long lo = c * CHUNK, hi = lo + CHUNK < N ? lo + CHUNK : N;
    for (int k = 0; k < m; ++k) {
      const double hk = -h[k];
      const double *vk = V + (size_t)k * N;
      for (long t = lo; t < hi; ++t) w[t] = fma(hk, vk[t], w[t]);
    }
    if (part_dots)
      for (int k = 0; k < m; ++k) {
        const double *vk = V + (size_t)k * N;
        double s = 0.0;
        for (long t = lo; t < hi; ++t) s = fma(vk[t], w[t], s);
        part_dots[(size_t)k * nch + c] = s;
      }
    if (part_norm) {
      double s = 0.0;
      for (long t = lo; t < hi; ++t) s = fma(w[t], w[t], s);
      part_norm[c] = s;
    }
  }
}
static void sum_parts(const double *part, long nch, int m, double *out) {
  for (int k = 0; k < m; ++k) {
    double s = 0.0;
    for (long c = 0; c < nch; ++c) s += part[(size_t)k * nch + c];
    out[k] = s;
  }
}
static long U3(const oracle *o, int i, int j, int k) { return ((long)k * o->ny + j) * (o->nx + 1) + i; }
static long V3(const oracle *o, int i, int j, int k) { return ((long)k * (o->ny + 1) + j) * o->nx + i; }
static long W3(const oracle *o, int i, int j, int k) { return ((long)k * o->ny + j) * o->nx + i; }

static const double *op_vals(const oracle *o, int f) {
  return f == 0 ? o->in.Au : f == 1 ? o->in.Av : f == 2 ? o->in.Aw : o->in.Ap;
}
static const box3 *op_box(const oracle *o, int f) {
  return f == 0 ? &o->bu : f == 1 ? &o->bv : f == 2 ? &o->bw : &o->bp;
}

/* y = A x for a 7-point row-major operator; accumulation order C,-x,+x,-y,+y,-z,+z */
static void spmv7(const box3 *b, const double *A, const double *x, double *y) {
  const int nx = b->n[0], ny = b->n[1], nz = b->n[2];
  const long sy = nx, sz = (long)nx * ny;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        long r = k * sz + j * sy + i;
        const double *a = A + 7 * r;
        double acc = 0.0;
        acc = fma(a[0], x[r], acc);
        acc = fma(a[1], i > 0 ? x[r - 1] : 0.0, acc);
        acc = fma(a[2], i < nx - 1 ? x[r + 1] : 0.0, acc);
        acc = fma(a[3], j > 0 ? x[r - sy] : 0.0, acc);
        acc = fma(a[4], j < ny - 1 ? x[r + sy] : 0.0, acc);
        acc = fma(a[5], k > 0 ? x[r - sz] : 0.0, acc);
        acc = fma(a[6], k < nz - 1 ? x[r + sz] : 0.0, acc);
        y[r] = acc;
      }
}

/* ------------------------------------------------------------------------ */
/* dense per-step operations (gpu_dense_ops.hpp semantics)                   */
/* ------------------------------------------------------------------------ */

/* BC cleanup in the order of the CPU twin (immersed_operators.hpp:1036-1053):
 * boundary planes first (the outlet copies u[nx-1] before any zeroing), then
 * inactive interior faces. Inactive w faces use the mask one plane below, as
 * the device kernel does (gpu_dense_ops.hpp:9); the masks are z-invariant. */
void oracle_bc_cleanup(const oracle *o, double *u, double *v, double *w, const double *uin_step) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) {
      u[U3(o, 0, j, k)] = uin_step[j + (long)ny * k];
      u[U3(o, nx, j, k)] = u[U3(o, nx - 1, j, k)];
    }
  for (int k = 0; k < nz; ++k)
    for (int i = 0; i < nx; ++i) { v[V3(o, i, 0, k)] = 0.0; v[V3(o, i, ny, k)] = 0.0; }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) { w[W3(o, i, j, 0)] = 0.0; w[W3(o, i, j, nz)] = 0.0; }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i < nx; ++i)
        if (!o->in.active_u[U3(o, i, j, k)]) u[U3(o, i, j, k)] = 0.0;
  for (int k = 0; k < nz; ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        if (!o->in.active_v[V3(o, i, j, k)]) v[V3(o, i, j, k)] = 0.0;
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        if (!o->in.active_w[W3(o, i, j, k - 1)]) w[W3(o, i, j, k)] = 0.0;
}

static double uval(const oracle *o, const double *u, int i, int j, int k, double fb) {
  if (i < 0 || i > o->nx || j < 0 || j >= o->ny || k < 0 || k >= o->nz) return fb;
  return u[U3(o, i, j, k)];
}
static double vval(const oracle *o, const double *v, int i, int j, int k, double fb) {
  if (i < 0 || i >= o->nx || j < 0 || j > o->ny || k < 0 || k >= o->nz) return fb;
  return v[V3(o, i, j, k)];
}
static double wval(const oracle *o, const double *w, int i, int j, int k, double fb) {
  if (i < 0 || i >= o->nx || j < 0 || j >= o->ny || k < 0 || k > o->nz) return fb;
  return w[W3(o, i, j, k)];
}

/* Centred advective form (gpu_dense_ops.hpp:12-14; immersed_operators.hpp:990-1034). */
void oracle_convection(const oracle *o, const double *u, const double *v, const double *w,
                       double *cu, double *cv, double *cw) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const double tdx = 2 * o->dx, tdy = 2 * o->dy, tdz = 2 * o->dz;
  memset(cu, 0, sizeof(double) * (size_t)(nx + 1) * ny * nz);
  memset(cv, 0, sizeof(double) * (size_t)nx * (ny + 1) * nz);
  memset(cw, 0, sizeof(double) * (size_t)nx * ny * (nz + 1));
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i < nx; ++i) {
        if (!o->in.active_u[U3(o, i, j, k)]) continue;
        double uc = u[U3(o, i, j, k)];
        double va = 0.25 * (vval(o, v, i - 1, j, k, 0.0) + vval(o, v, i - 1, j + 1, k, 0.0) +
                            vval(o, v, i, j, k, 0.0) + vval(o, v, i, j + 1, k, 0.0));
        double wa = 0.25 * (wval(o, w, i - 1, j, k, 0.0) + wval(o, w, i - 1, j, k + 1, 0.0) +
                            wval(o, w, i, j, k, 0.0) + wval(o, w, i, j, k + 1, 0.0));
        double ue = uval(o, u, i + 1, j, k, uc), uw = uval(o, u, i - 1, j, k, uc);
        double un = uval(o, u, i, j + 1, k, uc), us = uval(o, u, i, j - 1, k, uc);
        double ut = uval(o, u, i, j, k + 1, uc), ub = uval(o, u, i, j, k - 1, uc);
        cu[U3(o, i, j, k)] = uc * (ue - uw) / tdx + va * (un - us) / tdy + wa * (ut - ub) / tdz;
      }
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (!o->in.active_v[V3(o, i, j, k)]) continue;
        double vc = v[V3(o, i, j, k)];
        double ua = 0.25 * (uval(o, u, i, j - 1, k, 0.0) + uval(o, u, i + 1, j - 1, k, 0.0) +
                            uval(o, u, i, j, k, 0.0) + uval(o, u, i + 1, j, k, 0.0));
        double wa = 0.25 * (wval(o, w, i, j - 1, k, 0.0) + wval(o, w, i, j, k, 0.0) +
                            wval(o, w, i, j - 1, k + 1, 0.0) + wval(o, w, i, j, k + 1, 0.0));
        double ve = vval(o, v, i + 1, j, k, vc), vw = vval(o, v, i - 1, j, k, vc);
        double vn = vval(o, v, i, j + 1, k, vc), vs = vval(o, v, i, j - 1, k, vc);
        double vt = vval(o, v, i, j, k + 1, vc), vb = vval(o, v, i, j, k - 1, vc);
        cv[V3(o, i, j, k)] = ua * (ve - vw) / tdx + vc * (vn - vs) / tdy + wa * (vt - vb) / tdz;
      }
#pragma omp parallel for schedule(static)
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (!o->in.active_w[W3(o, i, j, k - 1)]) continue;
        double wc = w[W3(o, i, j, k)];
        double ua = 0.25 * (uval(o, u, i, j, k - 1, 0.0) + uval(o, u, i + 1, j, k - 1, 0.0) +
                            uval(o, u, i, j, k, 0.0) + uval(o, u, i + 1, j, k, 0.0));
        double va = 0.25 * (vval(o, v, i, j, k - 1, 0.0) + vval(o, v, i, j + 1, k - 1, 0.0) +
                            vval(o, v, i, j, k, 0.0) + vval(o, v, i, j + 1, k, 0.0));
        double we = wval(o, w, i + 1, j, k, wc), ww = wval(o, w, i - 1, j, k, wc);
        double wn = wval(o, w, i, j + 1, k, wc), ws = wval(o, w, i, j - 1, k, wc);
        double wt = wval(o, w, i, j, k + 1, wc), wb = wval(o, w, i, j, k - 1, wc);
        cw[W3(o, i, j, k)] = ua * (we - ww) / tdx + va * (wn - ws) / tdy + wc * (wt - wb) / tdz;
      }
}

/* y[row] = sum over the sorted CSR row of val * x[col], as a fused multiply-add
 * chain in column order (gpu_dense_ops.hpp:61-68); x and y are 1-based. */
static void csr_apply(const int32_t *rp, const int32_t *col, const double *val, long nrows,
                      const double *x, double *y) {
#pragma omp parallel for schedule(static)
  for (long r = 0; r < nrows; ++r) {
    double s = 0.0;
    for (int t = rp[r]; t < rp[r + 1]; ++t) s = fma(val[t], x[col[t]], s);
    y[r + 1] = s;
  }
}

/* G p unpacked onto the three face arrays (gpu_dense_ops.hpp:70-78). */
static void gradient_faces(const oracle *o, const double *p, double *gx, double *gy, double *gz) {
  const long NP = (long)o->nx * o->ny * o->nz;
  double *pv = (double *)xcalloc((size_t)o->nP + 1, sizeof(double));
  double *gp = (double *)xcalloc((size_t)o->nQ + 1, sizeof(double));
  for (long c = 0; c < NP; ++c)
    if (o->in.fluid_p[c] && o->in.id_p[c] > 0) pv[o->in.id_p[c]] = p[c];
  csr_apply(o->in.G_rowptr, o->in.G_col, o->in.G_val, o->nQ, pv, gp);
  const long NU = (long)(o->nx + 1) * o->ny * o->nz, NV = (long)o->nx * (o->ny + 1) * o->nz,
             NW = (long)o->nx * o->ny * (o->nz + 1);
  for (long f = 0; f < NU; ++f) { int id = o->in.id_qu[f]; gx[f] = id > 0 ? gp[id] : 0.0; }
  for (long f = 0; f < NV; ++f) { int id = o->in.id_qv[f]; gy[f] = id > 0 ? gp[o->nQu + id] : 0.0; }
  for (long f = 0; f < NW; ++f) { int id = o->in.id_qw[f]; gz[f] = id > 0 ? gp[o->nQu + o->nQv + id] : 0.0; }
  free(pv); free(gp);
}

/* rhs = ((rho/dt) u - rho conv - gp + rhs_bc[id]) scale[id] on active faces
 * (gpu_dense_ops.hpp:16-18). The reference's kernel is compiled by nvcc with
 * contraction on: its first difference becomes fma(rho/dt, u, -(rho conv))
 * (found bit for bit against that kernel built from the reference's sources);
 * the other operations are rounded one by one. */
static double mom_rhs(double a, double rho, double uc, double conv, double gp, double bc, double sc) {
  double t2 = rho * conv;
  double t = fma(a, uc, -t2);
  t = t - gp;
  t = t + bc;
  return t * sc;
}

void oracle_momentum_rhs(const oracle *o, const double *u, const double *v, const double *w, const double *p,
                         double *bu, double *bv, double *bw) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const long NU = (long)(nx + 1) * ny * nz, NV = (long)nx * (ny + 1) * nz, NW = (long)nx * ny * (nz + 1);
  double *cu = (double *)xcalloc((size_t)NU, 8), *cv = (double *)xcalloc((size_t)NV, 8), *cw = (double *)xcalloc((size_t)NW, 8);
  double *gx = (double *)xcalloc((size_t)NU, 8), *gy = (double *)xcalloc((size_t)NV, 8), *gz = (double *)xcalloc((size_t)NW, 8);
  oracle_convection(o, u, v, w, cu, cv, cw);
  gradient_faces(o, p, gx, gy, gz);
  const double rho = o->prm.rho, a = o->prm.rho / o->prm.dt;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i < nx; ++i) {
        long f = U3(o, i, j, k), r = ((long)k * ny + j) * (nx - 1) + (i - 1);
        int id = o->in.id_u[f];
        bu[r] = (id > 0 && o->in.active_u[f]) ? mom_rhs(a, rho, u[f], cu[f], gx[f], o->in.rhs_u_bc[id], o->in.scale_u[id]) : 0.0;
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        long f = V3(o, i, j, k), r = ((long)k * (ny - 1) + (j - 1)) * nx + i;
        int id = o->in.id_v[f];
        bv[r] = (id > 0 && o->in.active_v[f]) ? mom_rhs(a, rho, v[f], cv[f], gy[f], o->in.rhs_v_bc[id], o->in.scale_v[id]) : 0.0;
      }
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        long f = W3(o, i, j, k), r = ((long)(k - 1) * ny + j) * nx + i;
        int id = o->in.id_w[f];
        bw[r] = (id > 0 && o->in.active_w[f]) ? mom_rhs(a, rho, w[f], cw[f], gz[f], o->in.rhs_w_bc[id], o->in.scale_w[id]) : 0.0;
      }
  free(cu); free(cv); free(cw); free(gx); free(gy); free(gz);
}

/* Pack the q-active faces (gpu_dense_ops.hpp:80-85) into a 1-based vector. */
static void pack_q(const oracle *o, const double *u, const double *v, const double *w, double *q) {
  const long NU = (long)(o->nx + 1) * o->ny * o->nz, NV = (long)o->nx * (o->ny + 1) * o->nz,
             NW = (long)o->nx * o->ny * (o->nz + 1);
  memset(q, 0, sizeof(double) * ((size_t)o->nQ + 1));
  for (long f = 0; f < NU; ++f) { int id = o->in.id_qu[f]; if (id > 0) q[id] = u[f]; }
  for (long f = 0; f < NV; ++f) { int id = o->in.id_qv[f]; if (id > 0) q[o->nQu + id] = v[f]; }
  for (long f = 0; f < NW; ++f) { int id = o->in.id_qw[f]; if (id > 0) q[o->nQu + o->nQv + id] = w[f]; }
}

/* b_p = -(rho/dt) (D q~ + ramp div_bc) on fluid cells (gpu_dense_ops.hpp:87-90). */
void oracle_pressure_rhs(const oracle *o, const double *ut, const double *vt, const double *wt, double ramp,
                         double *bp) {
  const long NP = (long)o->nx * o->ny * o->nz;
  double *q = (double *)xcalloc((size_t)o->nQ + 1, 8), *dq = (double *)xcalloc((size_t)o->nP + 1, 8);
  pack_q(o, ut, vt, wt, q);
  csr_apply(o->in.D_rowptr, o->in.D_col, o->in.D_val, o->nP, q, dq);
  const double na = -(o->prm.rho / o->prm.dt);
  for (long c = 0; c < NP; ++c) {
    int id = o->in.id_p[c];
    double r = 0.0;
    if (o->in.fluid_p[c] && id > 0) r = na * fma(ramp, o->in.div_bc_unit[id], dq[id]);
    bp[c] = r;
  }
  free(q); free(dq);
}

void oracle_apply_operator(const oracle *o, int field, const double *x, double *y) {
  spmv7(op_box(o, field), op_vals(o, field), x, y);
}

/* ------------------------------------------------------------------------ */
/* semicoarsening multigrid (PFMG-style: one direction per level,            */
/* operator-dependent interpolation, R = P^T, Galerkin coarse operators)     */
/* ------------------------------------------------------------------------ */
static const int k7to27[7] = {13, 12, 14, 10, 16, 4, 22};
static int slot_off(int s, int d) { return d == 0 ? s % 3 - 1 : d == 1 ? (s / 3) % 3 - 1 : s / 9 - 1; }


/* Operator-dependent interpolation weights (PFMG's: minus the couplings to the
 * lower / upper neighbour along cdir over the sum of the in-plane entries).
 * With mg_options bit 0, a coupled point that has no coupling along cdir
 * (0/0 above, e.g. a cut cell between the cylinder and a closed face) takes
 * the constant from those of its two coarse neighbours that are coupled
 * points, so that interpolation keeps reproducing constants there. */
static void mg_interp_weights(const oracle *o, mg_level *L) {
  const int d = L->cdir;
  const long N = L->b.N;
  L->pm = (double *)xcalloc((size_t)N, 8);
  L->pp = (double *)xcalloc((size_t)N, 8);
  uint8_t *coupled = (uint8_t *)xcalloc((size_t)N, 1);
  for (long r = 0; r < N; ++r)
    for (int s = 0; s < 27; ++s)
      if (s != 13 && L->A[27 * r + s] != 0.0) { coupled[r] = 1; break; }
  const long stride = d == 0 ? 1 : d == 1 ? L->b.n[0] : (long)L->b.n[0] * L->b.n[1];
  for (long r = 0; r < N; ++r) {
    const double *a = L->A + 27 * r;
    double c0 = 0.0, cm = 0.0, cp = 0.0;
    for (int s = 0; s < 27; ++s) {
      int od = slot_off(s, d);
      if (od == 0) c0 += a[s]; else if (od < 0) cm += a[s]; else cp += a[s];
    }
    if ((o->prm.mg_options & 1) && coupled[r] && cm == 0.0 && cp == 0.0) {
      const int idx[3] = {(int)(r % L->b.n[0]), (int)((r / L->b.n[0]) % L->b.n[1]),
                          (int)(r / ((long)L->b.n[0] * L->b.n[1]))};
      const int lo = idx[d] > 0 && coupled[r - stride];
      const int hi = idx[d] < L->b.n[d] - 1 && coupled[r + stride];
      if (lo + hi > 0) {
        L->pm[r] = lo ? 1.0 / (lo + hi) : 0.0;
        L->pp[r] = hi ? 1.0 / (lo + hi) : 0.0;
      }
      continue;
    }
    if (c0 != 0.0) { L->pm[r] = -cm / c0; L->pp[r] = -cp / c0; }
  }
  free(coupled);
}

/* Diagonal symmetrizer of a 7-point operator: W with A = W S, S symmetric.
 * Each connected set of coupled rows is walked breadth first from its lowest
 * row (w = 1), neighbours in slot order, w_c = w_r A[c][r] / A[r][c]; then
 * every coupling is checked. Returns 0 (and leaves winv at 1) when A is not
 * of that form. winv = 1 / w. */
static int mg_symmetrizer(const double *A7, const box3 *b, double *winv) {
  const long N = b->N;
  double *w = (double *)xcalloc((size_t)N, 8);
  long *queue = (long *)xcalloc((size_t)N, sizeof(long));
  uint8_t *seen = (uint8_t *)xcalloc((size_t)N, 1);
  const long sy = b->n[0], sz = (long)b->n[0] * b->n[1];
  const long off[7] = {0, -1, 1, -sy, sy, -sz, sz};
  static const int opp[7] = {0, 2, 1, 4, 3, 6, 5};
  int ok = 1;
  for (long root = 0; root < N && ok; ++root) {
    if (seen[root]) continue;
    seen[root] = 1;
    w[root] = 1.0;
    long head = 0, tail = 0;
    queue[tail++] = root;
    while (head < tail && ok) {
      const long r = queue[head++];
      const int i = (int)(r % b->n[0]), j = (int)((r / b->n[0]) % b->n[1]), k = (int)(r / sz);
      const int in[7] = {1, i > 0, i < b->n[0] - 1, j > 0, j < b->n[1] - 1, k > 0, k < b->n[2] - 1};
      for (int s = 1; s < 7; ++s) {
        if (!in[s] || A7[7 * r + s] == 0.0) continue;
        const long c = r + off[s];
        const double back = A7[7 * c + opp[s]];
        if (back == 0.0) { ok = 0; break; }
        if (seen[c]) continue;
        seen[c] = 1;
        w[c] = w[r] * back / A7[7 * r + s];
        queue[tail++] = c;
      }
    }
  }
  for (long r = 0; r < N && ok; ++r) {
    const int i = (int)(r % b->n[0]), j = (int)((r / b->n[0]) % b->n[1]), k = (int)(r / sz);
    const int in[7] = {1, i > 0, i < b->n[0] - 1, j > 0, j < b->n[1] - 1, k > 0, k < b->n[2] - 1};
    for (int s = 1; s < 7; ++s) {
      if (!in[s]) continue;
      const double x = A7[7 * r + s] / w[r], y = A7[7 * (r + off[s]) + opp[s]] / w[r + off[s]];
      if (fabs(x - y) > 1e-10 * fmax(fabs(x), fabs(y))) { ok = 0; break; }
    }
  }
  for (long r = 0; r < N; ++r) winv[r] = ok ? 1.0 / w[r] : 1.0;
  free(w); free(queue); free(seen);
  return ok;
}

static long lidx(const box3 *b, int i, int j, int k) { return ((long)k * b->n[1] + j) * b->n[0] + i; }

/* Coarse operator R A P for coarsening in direction d: each coarse point sums,
 * in a fixed order, over the three fine points it restricts from, their
 * stencil entries, and the coarse points interpolating each neighbour. */
static void mg_rap(const mg_level *F, mg_level *C) {
  const int d = F->cdir;
  const box3 *fb = &F->b, *cb = &C->b;
  C->A = (double *)xcalloc((size_t)cb->N * 27, 8);
#pragma omp parallel for schedule(static)
  for (long I = 0; I < cb->N; ++I) {
    int ci[3] = {(int)(I % cb->n[0]), (int)((I / cb->n[0]) % cb->n[1]), (int)(I / ((long)cb->n[0] * cb->n[1]))};
    double *ac = C->A + 27 * I;
    for (int fo = -1; fo <= 1; ++fo) {
      int f[3] = {ci[0], ci[1], ci[2]};
      f[d] = 2 * ci[d] + fo;
      if (f[d] < 0 || f[d] >= fb->n[d]) continue;
      long fr = lidx(fb, f[0], f[1], f[2]);
      double rw = fo == 0 ? 1.0 : (fo < 0 ? F->pp[fr] : F->pm[fr]);
      if (rw == 0.0) continue;
      const double *af = F->A + 27 * fr;
      for (int s = 0; s < 27; ++s) {
        if (af[s] == 0.0) continue;
        int g[3] = {f[0] + slot_off(s, 0), f[1] + slot_off(s, 1), f[2] + slot_off(s, 2)};
        if (g[0] < 0 || g[0] >= fb->n[0] || g[1] < 0 || g[1] >= fb->n[1] || g[2] < 0 || g[2] >= fb->n[2]) continue;
        long gr = lidx(fb, g[0], g[1], g[2]);
        double ra = rw * af[s];
        int jc[2]; double pw[2]; int nt = 0;
        if ((g[d] & 1) == 0) { jc[0] = g[d] / 2; pw[0] = 1.0; nt = 1; }
        else {
          jc[0] = (g[d] - 1) / 2; pw[0] = F->pm[gr]; nt = 1;
          if ((g[d] + 1) / 2 < cb->n[d]) { jc[1] = (g[d] + 1) / 2; pw[1] = F->pp[gr]; nt = 2; }
        }
        for (int t = 0; t < nt; ++t) {
          if (pw[t] == 0.0) continue;
          int o3[3] = {slot_off(s, 0), slot_off(s, 1), slot_off(s, 2)};
          o3[d] = jc[t] - ci[d];
          int sc = (o3[0] + 1) + 3 * (o3[1] + 1) + 9 * (o3[2] + 1);
          ac[sc] = ac[sc] + ra * pw[t];
        }
      }
    }
  }
}

/* Collapse a 27-point stencil to 7 points keeping the action on constants and
 * on linear functions: an entry at offset o with m nonzero components moves to
 * the m axis neighbours along those components and is removed m-1 times from
 * the centre. */
/* Collapse a 27-point coarse stencil to 7 points: each off-axis entry moves
 * to the axis neighbours it spans, the centre keeping the row sum. With
 * mg_options bit 0, only coupled axis neighbours receive it (moving a
 * coupling onto an uncoupled point, such as a solid cell of the cylinder,
 * would turn a Neumann wall into a Dirichlet one on the coarse grid); with
 * none the entry is lumped into the centre. */
static void mg_collapse7(const oracle *o, mg_level *L) {
  const long N = L->b.N;
  const int aware = o->prm.mg_options & 1;
  uint8_t *coupled = (uint8_t *)xcalloc((size_t)N, 1);
  for (long r = 0; r < N; ++r)
    for (int s = 0; s < 27; ++s)
      if (s != 13 && L->A[27 * r + s] != 0.0) { coupled[r] = 1; break; }
  const long st[3] = {1, L->b.n[0], (long)L->b.n[0] * L->b.n[1]};
  for (long r = 0; r < N; ++r) {
    double *a = L->A + 27 * r;
    for (int s = 0; s < 27; ++s) {
      int o3[3] = {slot_off(s, 0), slot_off(s, 1), slot_off(s, 2)};
      int m = (o3[0] != 0) + (o3[1] != 0) + (o3[2] != 0);
      if (m < 2 || a[s] == 0.0) continue;
      double e = a[s];
      a[s] = 0.0;
      int t = 0;
      for (int dd = 0; dd < 3; ++dd) {
        if (!o3[dd]) continue;
        if (aware && !coupled[r + o3[dd] * st[dd]]) continue;
        int q[3] = {0, 0, 0};
        q[dd] = o3[dd];
        int sq = (q[0] + 1) + 3 * (q[1] + 1) + 9 * (q[2] + 1);
        a[sq] = a[sq] + e;
        ++t;
      }
      a[13] = a[13] - (double)(t - 1) * e;
    }
  }
  free(coupled);
}

/* y = A x on a multigrid level, over the level's nonzero slots only, in slot
 * order. Equal bit for bit to the product over all 27 slots for finite x: the sum starts at +0 and a fused multiply-add never turns it
 * into -0, so adding an exact-zero product leaves it unchanged. */
static void spmv_level(const mg_level *L, const double *x, double *y) {
  const int nx = L->b.n[0], ny = L->b.n[1], nz = L->b.n[2], ns = L->ns;
  long off[27];
  int ox[27], oy[27], oz[27];
  for (int q = 0; q < ns; ++q) {
    const int s = L->slot[q];
    ox[q] = s % 3 - 1; oy[q] = (s / 3) % 3 - 1; oz[q] = s / 9 - 1;
    off[q] = ((long)oz[q] * ny + oy[q]) * nx + ox[q];
  }
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) {
      const int inner = k > 0 && k < nz - 1 && j > 0 && j < ny - 1;
      for (int i = 0; i < nx; ++i) {
        const long r = ((long)k * ny + j) * nx + i;
        const double *a = L->Ac + (long)ns * r;
        double acc = 0.0;
        if (inner && i > 0 && i < nx - 1) {
          for (int q = 0; q < ns; ++q) acc = fma(a[q], x[r + off[q]], acc);
        } else {
          for (int q = 0; q < ns; ++q) {
            const int ii = i + ox[q], jj = j + oy[q], kk = k + oz[q];
            const int in = ii >= 0 && ii < nx && jj >= 0 && jj < ny && kk >= 0 && kk < nz;
            acc = fma(a[q], in ? x[r + off[q]] : 0.0, acc);
          }
        }
        y[r] = acc;
      }
    }
}

static void mg_finish_level(const oracle *o, mg_level *L) {
  int used[27] = {0};
  for (long r = 0; r < L->b.N; ++r)
    for (int s = 0; s < 27; ++s)
      if (L->A[27 * r + s] != 0.0) used[s] = 1;
  L->ns = 0;
  for (int s = 0; s < 27; ++s)
    if (used[s]) L->slot[L->ns++] = s;
  L->Ac = (double *)xcalloc((size_t)L->b.N * (size_t)(L->ns ? L->ns : 1), 8);
  for (long r = 0; r < L->b.N; ++r)
    for (int q = 0; q < L->ns; ++q) L->Ac[(long)L->ns * r + q] = L->A[27 * r + L->slot[q]];
  L->invd = (double *)xcalloc((size_t)L->b.N, 8);
  L->wd = (double *)xcalloc((size_t)L->b.N, 8);
  for (long r = 0; r < L->b.N; ++r) {
    double dgl = L->A[27 * r + 13];
    L->invd[r] = dgl != 0.0 ? 1.0 / dgl : 0.0;
    L->wd[r] = o->prm.mg_omega * L->invd[r];
  }
  L->bv = (double *)xcalloc((size_t)L->b.N, 8);
  L->xv = (double *)xcalloc((size_t)L->b.N, 8);
  L->rv = (double *)xcalloc((size_t)L->b.N, 8);
}

/* Explicit inverse by Gauss-Jordan elimination with partial pivoting. */
static void dense_inverse(const double *A27, const box3 *b, double *inv) {
  const long n = b->N;
  double *M = (double *)xcalloc((size_t)(n * n), 8);
  for (long r = 0; r < n; ++r) {
    int i = (int)(r % b->n[0]), j = (int)((r / b->n[0]) % b->n[1]), k = (int)(r / ((long)b->n[0] * b->n[1]));
    for (int s = 0; s < 27; ++s) {
      int ii = i + slot_off(s, 0), jj = j + slot_off(s, 1), kk = k + slot_off(s, 2);
      if (ii < 0 || ii >= b->n[0] || jj < 0 || jj >= b->n[1] || kk < 0 || kk >= b->n[2]) continue;
      M[r * n + lidx(b, ii, jj, kk)] += A27[27 * r + s];
    }
  }
  for (long r = 0; r < n; ++r)
    for (long c = 0; c < n; ++c) inv[r * n + c] = (r == c) ? 1.0 : 0.0;
  for (long c = 0; c < n; ++c) {
    long piv = c;
    for (long r = c + 1; r < n; ++r) if (fabs(M[r * n + c]) > fabs(M[piv * n + c])) piv = r;
    if (piv != c)
      for (long t = 0; t < n; ++t) {
        double x = M[c * n + t]; M[c * n + t] = M[piv * n + t]; M[piv * n + t] = x;
        x = inv[c * n + t]; inv[c * n + t] = inv[piv * n + t]; inv[piv * n + t] = x;
      }
    double pv = M[c * n + c];
    if (pv == 0.0) continue;
    double ip = 1.0 / pv;
    for (long t = 0; t < n; ++t) { M[c * n + t] *= ip; inv[c * n + t] *= ip; }
    for (long r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = M[r * n + c];
      if (f == 0.0) continue;
      for (long t = 0; t < n; ++t) { M[r * n + t] -= f * M[c * n + t]; inv[r * n + t] -= f * inv[c * n + t]; }
    }
  }
  free(M);
}

static void mg_build(oracle *o) {
  if (o->mg_built) return;
  mg_level *L0 = &o->lev[0];
  L0->b = o->bp;
  L0->A = (double *)xcalloc((size_t)L0->b.N * 27, 8);
  o->mg_winv = (double *)xcalloc((size_t)L0->b.N, 8);
  const int sym = (o->prm.mg_options & 2) ? mg_symmetrizer(o->in.Ap, &L0->b, o->mg_winv) : 0;
  if (!sym)
    for (long r = 0; r < L0->b.N; ++r) o->mg_winv[r] = 1.0;
  o->mg_sym = sym;
  for (long r = 0; r < L0->b.N; ++r)
    for (int s = 0; s < 7; ++s) {
      const double a = o->in.Ap[7 * r + s];
      L0->A[27 * r + k7to27[s]] = sym ? a * o->mg_winv[r] : a;
    }
  double h[3] = {o->dx, o->dy, o->dz};
  int queue[3], nq = 0;  /* directions still to coarsen in the current group */
  int l = 0;
  for (;;) {
    mg_level *F = &o->lev[l];
    mg_finish_level(o, F);
    /* A group starts at a relaxed level: every direction whose spacing is
     * within mg_group_ratio of the smallest is coarsened once, smallest
     * spacing first; the levels inside the group are not relaxed. A ratio of
     * 0 gives one direction per relaxed level. */
    F->relax = (nq == 0);
    if (nq == 0) {
      double hmin = 0.0;
      int any = 0;
      for (int dd = 0; dd < 3; ++dd)
        if (F->b.n[dd] > 1 && (!any || h[dd] < hmin)) { hmin = h[dd]; any = 1; }
      int cand[3], nc = 0;
      for (int dd = 0; dd < 3; ++dd)
        if (F->b.n[dd] > 1 && (h[dd] == hmin || (o->prm.mg_group_ratio > 0.0 && h[dd] <= o->prm.mg_group_ratio * hmin)))
          cand[nc++] = dd;
      for (int a = 0; a < nc; ++a)
        for (int b2 = a + 1; b2 < nc; ++b2)
          if (h[cand[b2]] < h[cand[a]]) { int t = cand[a]; cand[a] = cand[b2]; cand[b2] = t; }
      if (o->prm.mg_group_ratio <= 0.0 && nc > 1) nc = 1;
      for (int a = 0; a < nc; ++a) queue[a] = cand[nc - 1 - a];
      nq = nc;
    }
    int d = -1;
    while (nq > 0 && d < 0) {
      int q = queue[--nq];
      if (F->b.n[q] > 1) d = q;
    }
    if (F->b.N <= o->prm.mg_coarse_max || l + 1 >= o->prm.mg_max_levels || d < 0 || l + 1 >= 40) {
      F->cdir = -1;
      F->relax = 1;
      F->dense_inv = (double *)xcalloc((size_t)(F->b.N * F->b.N), 8);
      dense_inverse(F->A, &F->b, F->dense_inv);
      break;
    }
    F->cdir = d;
    h[d] *= 2.0;
    mg_interp_weights(o, F);
    mg_level *C = &o->lev[l + 1];
    C->b = F->b;
    C->b.n[d] = (F->b.n[d] + 1) / 2;
    C->b.N = (long)C->b.n[0] * C->b.n[1] * C->b.n[2];
    mg_rap(F, C);
    if (o->prm.mg_rap == 1) mg_collapse7(o, C);
    ++l;
  }
  o->nlev = l + 1;
  o->mg_built = 1;
}

/* One relaxation sweep; zero_guess: x starts from 0. */
static void mg_relax(const oracle *o, const mg_level *L, const double *b, double *x, int zero_guess) {
  const long N = L->b.N;
  if (o->prm.mg_relax == 2) {
    /* two-colour relaxation: in each colour phase the points of that colour
     * update from the values at the start of the phase */
    if (zero_guess) memset(x, 0, sizeof(double) * (size_t)N);
    double *snap = (double *)xcalloc((size_t)N, 8);
    for (int color = 0; color < 2; ++color) {
      memcpy(snap, x, sizeof(double) * (size_t)N);
#pragma omp parallel for schedule(static)
      for (long r = 0; r < N; ++r) {
        int i = (int)(r % L->b.n[0]), j = (int)((r / L->b.n[0]) % L->b.n[1]), k = (int)(r / ((long)L->b.n[0] * L->b.n[1]));
        if (((i + j + k) & 1) != color) continue;
        const double *a = L->A + 27 * r;
        double acc = 0.0;
        for (int s = 0; s < 27; ++s) {
          int ii = i + slot_off(s, 0), jj = j + slot_off(s, 1), kk = k + slot_off(s, 2);
          double xv = (ii >= 0 && ii < L->b.n[0] && jj >= 0 && jj < L->b.n[1] && kk >= 0 && kk < L->b.n[2]) ? snap[lidx(&L->b, ii, jj, kk)] : 0.0;
          acc = fma(a[s], xv, acc);
        }
        x[r] = fma(L->invd[r], b[r] - acc, snap[r]);
      }
    }
    free(snap);
    return;
  }
  if (zero_guess) {
#pragma omp parallel for schedule(static)
    for (long r = 0; r < N; ++r) x[r] = L->wd[r] * b[r];
    return;
  }
  double *ax = (double *)xcalloc((size_t)N, 8);
  spmv_level(L, x, ax);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < N; ++r) x[r] = fma(L->wd[r], b[r] - ax[r], x[r]);
  free(ax);
}

static void mg_cycle(oracle *o, int l, const double *b, double *x) {
  mg_level *L = &o->lev[l];
  const long N = L->b.N;
  if (L->cdir < 0) {
    for (long r = 0; r < N; ++r) {
      double acc = 0.0;
      for (long c = 0; c < N; ++c) acc = fma(L->dense_inv[r * N + c], b[c], acc);
      x[r] = acc;
    }
    return;
  }
  const int c1 = (l > 0 && o->prm.mg_nu_coarse > 0) ? o->prm.mg_nu_coarse : o->prm.mg_nu1;
  const int c2 = (l > 0 && o->prm.mg_nu_coarse > 0) ? o->prm.mg_nu_coarse : o->prm.mg_nu2;
  const int nu1 = L->relax ? c1 : 0, nu2 = L->relax ? c2 : 0;
  for (int s = 0; s < nu1; ++s) mg_relax(o, L, b, x, s == 0);
  if (nu1 == 0) memset(x, 0, sizeof(double) * (size_t)N);
  double *ax = L->rv;
  if (nu1 == 0) memcpy(ax, b, sizeof(double) * (size_t)N);
  else {
    spmv_level(L, x, ax);
#pragma omp parallel for schedule(static)
    for (long r = 0; r < N; ++r) ax[r] = b[r] - ax[r];
  }
  mg_level *C = &o->lev[l + 1];
  const int d = L->cdir;
#pragma omp parallel for schedule(static)
  for (long I = 0; I < C->b.N; ++I) {
    int ci[3] = {(int)(I % C->b.n[0]), (int)((I / C->b.n[0]) % C->b.n[1]), (int)(I / ((long)C->b.n[0] * C->b.n[1]))};
    double acc = 0.0;
    for (int fo = -1; fo <= 1; ++fo) {
      int f[3] = {ci[0], ci[1], ci[2]};
      f[d] = 2 * ci[d] + fo;
      if (f[d] < 0 || f[d] >= L->b.n[d]) continue;
      long fr = lidx(&L->b, f[0], f[1], f[2]);
      double rw = fo == 0 ? 1.0 : (fo < 0 ? L->pp[fr] : L->pm[fr]);
      acc = fma(rw, ax[fr], acc);
    }
    C->bv[I] = acc;
  }
  mg_cycle(o, l + 1, C->bv, C->xv);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < N; ++r) {
    int f[3] = {(int)(r % L->b.n[0]), (int)((r / L->b.n[0]) % L->b.n[1]), (int)(r / ((long)L->b.n[0] * L->b.n[1]))};
    double corr;
    if ((f[d] & 1) == 0) {
      int c3[3] = {f[0], f[1], f[2]}; c3[d] = f[d] / 2;
      corr = C->xv[lidx(&C->b, c3[0], c3[1], c3[2])];
    } else {
      int c0[3] = {f[0], f[1], f[2]}; c0[d] = (f[d] - 1) / 2;
      double x0 = C->xv[lidx(&C->b, c0[0], c0[1], c0[2])], x1 = 0.0;
      if ((f[d] + 1) / 2 < C->b.n[d]) { int c1[3] = {f[0], f[1], f[2]}; c1[d] = (f[d] + 1) / 2; x1 = C->xv[lidx(&C->b, c1[0], c1[1], c1[2])]; }
      corr = fma(L->pp[r], x1, L->pm[r] * x0);
    }
    x[r] = x[r] + corr;
  }
  for (int s = 0; s < nu2; ++s) mg_relax(o, L, b, x, 0);
}

void oracle_mg_vcycle(oracle *o, const double *b, double *x) {
  mg_build(o);
  if (!o->mg_sym) { mg_cycle(o, 0, b, x); return; }
  const long N = o->lev[0].b.N;
  double *bs = (double *)xcalloc((size_t)N, 8);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < N; ++r) bs[r] = b[r] * o->mg_winv[r];
  mg_cycle(o, 0, bs, x);
  free(bs);
}
int oracle_mg_levels(oracle *o) { mg_build(o); return o->nlev; }
int oracle_mg_level_info(oracle *o, int l, int *dims, int *cdir, int *nslots) {
  mg_build(o);
  if (l < 0 || l >= o->nlev) return -1;
  dims[0] = o->lev[l].b.n[0]; dims[1] = o->lev[l].b.n[1]; dims[2] = o->lev[l].b.n[2];
  *cdir = o->lev[l].cdir;
  *nslots = 27;
  return 0;
}
int oracle_mg_level_coef(oracle *o, int l, double *coef) {
  mg_build(o);
  if (l < 0 || l >= o->nlev) return -1;
  memcpy(coef, o->lev[l].A, sizeof(double) * 27 * (size_t)o->lev[l].b.N);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* restarted, right-preconditioned GMRES with classical Gram-Schmidt applied  */
/* twice (restating HYPRE_StructGMRESSolve: stop when ||r||/||b|| <= tol,    */
/* confirm with the true residual, restart from it)                          */
/* ------------------------------------------------------------------------ */
static void precond(oracle *o, int field, const double *v, double *z) {
  const box3 *b = op_box(o, field);
  const long N = b->N;
  if (field == 3 && o->prm.p_pc == 1) { oracle_mg_vcycle(o, v, z); return; }
  const int sweeps = field == 3 ? 1 : (o->prm.vel_jacobi_iters > 0 ? o->prm.vel_jacobi_iters : 1);
  const double *id = o->invd[field];
#pragma omp parallel for schedule(static)
  for (long r = 0; r < N; ++r) z[r] = v[r] * id[r];
  if (sweeps > 1) {
    double *az = (double *)xcalloc((size_t)N, 8);
    for (int s = 1; s < sweeps; ++s) {
      spmv7(b, op_vals(o, field), z, az);
#pragma omp parallel for schedule(static)
      for (long r = 0; r < N; ++r) z[r] = fma(id[r], v[r] - az[r], z[r]);
    }
    free(az);
  }
}

int oracle_solve(oracle *o, int field, const double *b, double *x, oracle_solve_stats *st) {
  const box3 *bx = op_box(o, field);
  const long N = bx->N;
  const double tol = field == 3 ? o->prm.p_tol : o->prm.vel_tol;
  const int maxit = field == 3 ? o->prm.p_maxit : o->prm.vel_maxit;
  const int kdim = field == 3 ? o->prm.p_kdim : o->prm.vel_kdim;
  const double *A = op_vals(o, field);
  double *V = (double *)xcalloc((size_t)(kdim + 1) * (size_t)N, 8);
  double *r = (double *)xcalloc((size_t)N, 8), *z = (double *)xcalloc((size_t)N, 8), *wv = (double *)xcalloc((size_t)N, 8);
  double *H = (double *)xcalloc((size_t)(kdim + 1) * kdim, 8);
  double *cs = (double *)xcalloc((size_t)kdim + 1, 8), *sn = (double *)xcalloc((size_t)kdim + 1, 8);
  double *g = (double *)xcalloc((size_t)kdim + 1, 8), *y = (double *)xcalloc((size_t)kdim + 1, 8);
  double *hc = (double *)xcalloc((size_t)kdim + 2, 8);
  const long nch = (N + CHUNK - 1) / CHUNK;
  double *part = (double *)xcalloc((size_t)nch * (size_t)(kdim + 1), 8);
#define HH(i, j) H[(size_t)(i) * kdim + (j)]
  const double b_norm = sqrt(dot(b, b, N));
  spmv7(bx, A, x, r);
#pragma omp parallel for schedule(static)
  for (long t = 0; t < N; ++t) r[t] = b[t] - r[t];
  double r_norm = sqrt(dot(r, r, N));
  int iters = 0, converged = 0;
  const double den = b_norm > 0.0 ? b_norm : r_norm;
  const double eps = tol * den;
  double real_old = b_norm;
  if (r_norm == 0.0) converged = 1;
  while (!converged) {
    if (r_norm <= eps) { converged = 1; break; }
    if (iters >= maxit) break;
#pragma omp parallel for schedule(static)
    for (long t = 0; t < N; ++t) V[t] = r[t] / r_norm;
    g[0] = r_norm;
    int i = 0, claimed = 0;
    while (i < kdim && iters < maxit) {
      precond(o, field, V + (size_t)i * N, z);
      spmv7(bx, A, z, wv);
      /* classical Gram-Schmidt twice: hc = V^T w, w -= V hc, twice; then
       * ||w||. Each update is fused with the products that follow it, chunk
       * by chunk (the sums are those of dot(): per-chunk fused
       * multiply-adds in index order, chunks added in order). */
      multi_dot(V, N, i + 1, wv, hc);
      for (int k = 0; k <= i; ++k) HH(k, i) = hc[k];
      orth_update(V, N, i + 1, hc, wv, part, NULL);
      sum_parts(part, nch, i + 1, hc);
      for (int k = 0; k <= i; ++k) HH(k, i) = HH(k, i) + hc[k];
      orth_update(V, N, i + 1, hc, wv, NULL, part);
      sum_parts(part, nch, 1, hc);
      double hn = sqrt(hc[0]);
      HH(i + 1, i) = hn;
      if (hn != 0.0) {
#pragma omp parallel for schedule(static)
        for (long t = 0; t < N; ++t) V[(size_t)(i + 1) * N + t] = wv[t] / hn;
      }
      for (int j = 0; j < i; ++j) {
        double t0 = HH(j, i);
        HH(j, i) = sn[j] * HH(j + 1, i) + cs[j] * t0;
        HH(j + 1, i) = -sn[j] * t0 + cs[j] * HH(j + 1, i);
      }
      double gam = sqrt(HH(i + 1, i) * HH(i + 1, i) + HH(i, i) * HH(i, i));
      if (gam == 0.0) gam = 2.220446049250313e-16;
      cs[i] = HH(i, i) / gam;
      sn[i] = HH(i + 1, i) / gam;
      g[i + 1] = -sn[i] * g[i];
      g[i] = cs[i] * g[i];
      HH(i, i) = sn[i] * HH(i + 1, i) + cs[i] * HH(i, i);
      ++i; ++iters;
      r_norm = fabs(g[i]);
      if (r_norm <= eps) { claimed = 1; break; }
    }
    for (int k = i - 1; k >= 0; --k) {
      double t0 = g[k];
      for (int j = k + 1; j < i; ++j) t0 -= HH(k, j) * y[j];
      y[k] = t0 / HH(k, k);
    }
#pragma omp parallel for schedule(static)
    for (long c0 = 0; c0 < N; c0 += CHUNK) {
      const long c1 = c0 + CHUNK < N ? c0 + CHUNK : N;
      for (long t = c0; t < c1; ++t) wv[t] = 0.0;
      for (int k = 0; k < i; ++k) {
        const double yk = y[k];
        const double *vk = V + (size_t)k * N;
        for (long t = c0; t < c1; ++t) wv[t] = fma(yk, vk[t], wv[t]);
      }
    }
    precond(o, field, wv, z);
#pragma omp parallel for schedule(static)
    for (long t = 0; t < N; ++t) x[t] = x[t] + z[t];
    spmv7(bx, A, x, r);
#pragma omp parallel for schedule(static)
    for (long t = 0; t < N; ++t) r[t] = b[t] - r[t];
    double rt = sqrt(dot(r, r, N));
    r_norm = rt;
    if (rt <= eps) { converged = 1; break; }
    /* stagnation: HYPRE stops and reports success (no error below max_iter) */
    if (claimed && rt >= real_old) { converged = 1; break; }
    real_old = rt;
  }
#undef HH
  st->iters = iters;
  st->rel_res = b_norm > 0.0 ? r_norm / b_norm : r_norm;
  st->status = converged ? 0 : 1;
  free(V); free(r); free(z); free(wv); free(H); free(cs); free(sn); free(g); free(y); free(hc); free(part);
  return st->status;
}

/* ------------------------------------------------------------------------ */
/* lifecycle and the full step                                               */
/* ------------------------------------------------------------------------ */
oracle *oracle_create(const oracle_params *prm, const oracle_inputs *in) {
  oracle *o = (oracle *)xcalloc(1, sizeof(oracle));
  o->prm = *prm;
  o->in = *in;
  o->nx = prm->nx; o->ny = prm->ny; o->nz = prm->nz;
  o->dx = prm->Lx / prm->nx; o->dy = prm->Ly / prm->ny; o->dz = prm->Lz / prm->nz;
  const long NU = (long)(o->nx + 1) * o->ny * o->nz, NV = (long)o->nx * (o->ny + 1) * o->nz,
             NW = (long)o->nx * o->ny * (o->nz + 1), NP = (long)o->nx * o->ny * o->nz;
  o->nU = max_id(in->id_u, NU); o->nV = max_id(in->id_v, NV); o->nW = max_id(in->id_w, NW);
  o->nP = max_id(in->id_p, NP);
  o->nQu = max_id(in->id_qu, NU); o->nQv = max_id(in->id_qv, NV); o->nQw = max_id(in->id_qw, NW);
  o->nQ = o->nQu + o->nQv + o->nQw;
  o->bu = (box3){{o->nx - 1, o->ny, o->nz}, (long)(o->nx - 1) * o->ny * o->nz};
  o->bv = (box3){{o->nx, o->ny - 1, o->nz}, (long)o->nx * (o->ny - 1) * o->nz};
  o->bw = (box3){{o->nx, o->ny, o->nz - 1}, (long)o->nx * o->ny * (o->nz - 1)};
  o->bp = (box3){{o->nx, o->ny, o->nz}, NP};
  o->u = (double *)xcalloc((size_t)NU, 8); o->v = (double *)xcalloc((size_t)NV, 8);
  o->w = (double *)xcalloc((size_t)NW, 8); o->p = (double *)xcalloc((size_t)NP, 8);
  for (int f = 0; f < 4; ++f) {
    const box3 *b = op_box(o, f);
    const double *A = op_vals(o, f);
    o->invd[f] = (double *)xcalloc((size_t)b->N, 8);
    for (long r = 0; r < b->N; ++r) o->invd[f][r] = A[7 * r] != 0.0 ? 1.0 / A[7 * r] : 0.0;
  }
  return o;
}

void oracle_destroy(oracle *o) {
  if (!o) return;
  free(o->u); free(o->v); free(o->w); free(o->p);
  for (int f = 0; f < 4; ++f) free(o->invd[f]);
  free(o->mg_winv);
  free(o->alpha_u); free(o->alpha_v);
  for (int l = 0; l < o->nlev; ++l) {
    mg_level *L = &o->lev[l];
    free(L->A); free(L->wd); free(L->invd); free(L->pm); free(L->pp); free(L->bv); free(L->xv); free(L->rv);
    free(L->dense_inv); free(L->Ac);
  }
  free(o);
}

void oracle_set_fields(oracle *o, const double *u, const double *v, const double *w, const double *p) {
  const long NU = (long)(o->nx + 1) * o->ny * o->nz, NV = (long)o->nx * (o->ny + 1) * o->nz,
             NW = (long)o->nx * o->ny * (o->nz + 1), NP = (long)o->nx * o->ny * o->nz;
  if (u) memcpy(o->u, u, 8 * (size_t)NU);
  if (v) memcpy(o->v, v, 8 * (size_t)NV);
  if (w) memcpy(o->w, w, 8 * (size_t)NW);
  if (p) memcpy(o->p, p, 8 * (size_t)NP);
}

void oracle_get_fields(const oracle *o, double *u, double *v, double *w, double *p) {
  const long NU = (long)(o->nx + 1) * o->ny * o->nz, NV = (long)o->nx * (o->ny + 1) * o->nz,
             NW = (long)o->nx * o->ny * (o->nz + 1), NP = (long)o->nx * o->ny * o->nz;
  if (u) memcpy(u, o->u, 8 * (size_t)NU);
  if (v) memcpy(v, o->v, 8 * (size_t)NV);
  if (w) memcpy(w, o->w, 8 * (size_t)NW);
  if (p) memcpy(p, o->p, 8 * (size_t)NP);
}

/* u~ = u with the solve-box interior replaced by x, then the BC cleanup
 * (gpu_dense_ops.hpp:20-22, main.cu:307-312). */
void oracle_tilde(const oracle *o, const double *xu, const double *xv, const double *xw, double ramp,
                  double *ut, double *vt, double *wt) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const long NU = (long)(nx + 1) * ny * nz, NV = (long)nx * (ny + 1) * nz, NW = (long)nx * ny * (nz + 1);
  memcpy(ut, o->u, 8 * (size_t)NU); memcpy(vt, o->v, 8 * (size_t)NV); memcpy(wt, o->w, 8 * (size_t)NW);
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) for (int i = 1; i < nx; ++i)
    ut[U3(o, i, j, k)] = xu[((long)k * ny + j) * (nx - 1) + (i - 1)];
  for (int k = 0; k < nz; ++k) for (int j = 1; j < ny; ++j) for (int i = 0; i < nx; ++i)
    vt[V3(o, i, j, k)] = xv[((long)k * (ny - 1) + (j - 1)) * nx + i];
  for (int k = 1; k < nz; ++k) for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i)
    wt[W3(o, i, j, k)] = xw[((long)(k - 1) * ny + j) * nx + i];
  double *uin = (double *)xcalloc((size_t)ny * nz, 8);
  for (long t = 0; t < (long)ny * nz; ++t) uin[t] = ramp * o->in.uin[t];
  oracle_bc_cleanup(o, ut, vt, wt, uin);
  free(uin);
}

/* Projection and diagnostics (main.cu:338-363): q = q~ - (dt/rho) G phi,
 * u = u~ with q unpacked, BC cleanup, p += phi; writes the oracle's fields. */
void oracle_projection(oracle *o, const double *ut, const double *vt, const double *wt, const double *xp,
                       double ramp, oracle_step_stats *st) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const long NU = (long)(nx + 1) * ny * nz, NV = (long)nx * (ny + 1) * nz, NW = (long)nx * ny * (nz + 1),
             NP = (long)nx * ny * nz;
  double *uin = (double *)xcalloc((size_t)ny * nz, 8);
  for (long t = 0; t < (long)ny * nz; ++t) uin[t] = ramp * o->in.uin[t];
  double *phi = (double *)xcalloc((size_t)o->nP + 1, 8), *gphi = (double *)xcalloc((size_t)o->nQ + 1, 8);
  double *q = (double *)xcalloc((size_t)o->nQ + 1, 8);
  for (long c = 0; c < NP; ++c)
    if (o->in.fluid_p[c] && o->in.id_p[c] > 0) phi[o->in.id_p[c]] = xp[c];
  pack_q(o, ut, vt, wt, q);
  csr_apply(o->in.G_rowptr, o->in.G_col, o->in.G_val, o->nQ, phi, gphi);
  const double factor = o->prm.dt / o->prm.rho;
  for (long t = 1; t <= o->nQ; ++t) q[t] = fma(-factor, gphi[t], q[t]);
  memcpy(o->u, ut, 8 * (size_t)NU); memcpy(o->v, vt, 8 * (size_t)NV); memcpy(o->w, wt, 8 * (size_t)NW);
  for (long f = 0; f < NU; ++f) { int id = o->in.id_qu[f]; if (id > 0) o->u[f] = q[id]; }
  for (long f = 0; f < NV; ++f) { int id = o->in.id_qv[f]; if (id > 0) o->v[f] = q[o->nQu + id]; }
  for (long f = 0; f < NW; ++f) { int id = o->in.id_qw[f]; if (id > 0) o->w[f] = q[o->nQu + o->nQv + id]; }
  oracle_bc_cleanup(o, o->u, o->v, o->w, uin);
  for (long c = 0; c < NP; ++c)
    if (o->in.fluid_p[c] && o->in.id_p[c] > 0) o->p[c] = o->p[c] + phi[o->in.id_p[c]];
  double *dv = (double *)xcalloc((size_t)o->nP + 1, 8);
  csr_apply(o->in.D_rowptr, o->in.D_col, o->in.D_val, o->nP, q, dv);
  double div2 = 0.0;
  for (int i = 1; i <= o->nP; ++i) {
    double d = dv[i] + ramp * o->in.div_bc_unit[i];
    div2 += d * d;
  }
  st->div_l2 = sqrt(div2 / (o->nP > 1 ? o->nP : 1));
  double um = 0.0, vm = 0.0, wm = 0.0;
  for (long f = 0; f < NU; ++f) um = fmax(um, fabs(o->u[f]));
  for (long f = 0; f < NV; ++f) vm = fmax(vm, fabs(o->v[f]));
  for (long f = 0; f < NW; ++f) wm = fmax(wm, fabs(o->w[f]));
  st->umax = um; st->vmax = vm; st->wmax = wm;
  oracle_forces(o, st->force);
  free(phi); free(gphi); free(q); free(dv); free(uin);
}

/* Force of the fluid on the body from the end-of-step fields on the staircase
 * of non-fluid cells (the reference computes none; the library's k_forces
 * uses the same definition): pressure p times the shared face area on every
 * fluid/non-fluid cell pair, towards the non-fluid cell; wall shear
 * 2 rho nu u / h times the face area on every face velocity between two fluid
 * cells whose two neighbours across a direction are non-fluid. */
static int o_fluid(const oracle *o, int i, int j, int k) {
  const long c = ((long)k * o->ny + j) * o->nx + i;
  return o->in.fluid_p[c] && o->in.id_p[c] > 0;
}
static int o_solid(const oracle *o, int i, int j, int k) {
  return i >= 0 && i < o->nx && j >= 0 && j < o->ny && k >= 0 && k < o->nz && !o_fluid(o, i, j, k);
}
/* Distance from P along the segment P->S to the cylinder surface, +inf when
 * the segment does not reach it: the reference's segmentCircleDistance
 * (common.hpp:262-280), the root t in [0, 1] of |P + t (S - P) - C| = R
 * nearest P, times |S - P|. */
static double seg_circle(const oracle *o, double xP, double yP, double xS, double yS) {
  const double ddx = xS - xP, ddy = yS - yP;
  const double a = ddx * ddx + ddy * ddy;
  if (a <= 0.0) return INFINITY;
  const double ox = xP - o->xcirc, oy = yP - o->ycirc;
  const double b = 2.0 * (ddx * ox + ddy * oy);
  const double c = ox * ox + oy * oy - o->Rcirc * o->Rcirc;
  const double disc = b * b - 4.0 * a * c;
  if (disc < 0.0) return INFINITY;
  const double sd = sqrt(disc > 0.0 ? disc : 0.0);
  const double t1 = (-b - sd) / (2.0 * a), t2 = (-b + sd) / (2.0 * a);
  double t = INFINITY;
  if (t1 >= 0.0 && t1 <= 1.0) t = t1;
  else if (t2 >= 0.0 && t2 <= 1.0) t = t2;
  if (!isfinite(t)) return INFINITY;
  return sqrt(a) * t;
}
static double inv_seg(const oracle *o, double xP, double yP, double xS, double yS) {
  const double d = seg_circle(o, xP, yP, xS, yS);
  return isfinite(d) ? 1.0 / d : 0.0;
}

/* The cut-surface shear weight of one velocity row: sum over the directions
 * where the row meets the body (an inactive neighbour that is not a domain
 * boundary, as the momentum operators decide it, immersed_operators.hpp:1-177)
 * of the control-volume face area over the distance to the cylinder, times
 * rho. field 0, 1, 2 = u, v, w; (i, j, k) the face. */
static double cut_shear_weight(const oracle *o, int field, int i, int j, int k) {
  const int nx = o->nx, ny = o->ny;
  const double dx = o->dx, dy = o->dy, dz = o->dz, ax = dy * dz, ay = dx * dz;
  double s = 0.0;
  if (field == 0) {
    const double xP = i * dx, yP = (j + 0.5) * dy;
#define AU(ii, jj) (o->in.active_u[U3(o, ii, jj, k)] != 0)
    if (!(i > 1 && AU(i - 1, j)) && i != 1) s += ax * inv_seg(o, xP, yP, xP - dx, yP);
    if (!(i < nx - 1 && AU(i + 1, j)) && i != nx - 1) s += ax * inv_seg(o, xP, yP, xP + dx, yP);
    if (!(j > 0 && AU(i, j - 1)) && j != 0) s += ay * inv_seg(o, xP, yP, xP, yP - dy);
    if (!(j < ny - 1 && AU(i, j + 1)) && j != ny - 1) s += ay * inv_seg(o, xP, yP, xP, yP + dy);
#undef AU
  } else if (field == 1) {
    const double xP = (i + 0.5) * dx, yP = j * dy;
#define AV(ii, jj) (o->in.active_v[V3(o, ii, jj, k)] != 0)
    if (!(i > 0 && AV(i - 1, j)) && i != 0) s += ax * inv_seg(o, xP, yP, xP - dx, yP);
    if (!(i < nx - 1 && AV(i + 1, j)) && i != nx - 1) s += ax * inv_seg(o, xP, yP, xP + dx, yP);
    if (!(j > 1 && AV(i, j - 1)) && j != 1) s += ay * inv_seg(o, xP, yP, xP, yP - dy);
    if (!(j < ny - 1 && AV(i, j + 1)) && j != ny - 1) s += ay * inv_seg(o, xP, yP, xP, yP + dy);
#undef AV
  } else {
    const double xP = (i + 0.5) * dx, yP = (j + 0.5) * dy;
#define AW(ii, jj) (o->in.active_w[W3(o, ii, jj, k)] != 0)
    if (!(i > 0 && AW(i - 1, j)) && i != 0) s += ax * inv_seg(o, xP, yP, xP - dx, yP);
    if (!(i < nx - 1 && AW(i + 1, j)) && i != nx - 1) s += ax * inv_seg(o, xP, yP, xP + dx, yP);
    if (!(j > 0 && AW(i, j - 1)) && j != 0) s += ay * inv_seg(o, xP, yP, xP, yP - dy);
    if (!(j < ny - 1 && AW(i, j + 1)) && j != ny - 1) s += ay * inv_seg(o, xP, yP, xP, yP + dy);
#undef AW
  }
  return o->prm.rho * s;
}

/* Pressure weights of a fluid cell for the x and y force: the cell's part of
 * the body surface, -sum over its faces of alpha_f A_f n_f. A face to a
 * non-fluid cell is closed (the body's surface), a domain-boundary face open;
 * so the faces of the fluid cells close around the body and a uniform
 * pressure gives no force. */
static void cut_pressure_weight(const oracle *o, int i, int j, int k, double *wx, double *wy) {
  const int nx = o->nx, ny = o->ny;
  const double ax = o->dy * o->dz, ay = o->dx * o->dz;
  const double aw = i > 0 ? (o_fluid(o, i - 1, j, k) ? o->alpha_u[U3(o, i, j, k)] : 0.0) : 1.0;
  const double ae = i < nx - 1 ? (o_fluid(o, i + 1, j, k) ? o->alpha_u[U3(o, i + 1, j, k)] : 0.0) : 1.0;
  const double as = j > 0 ? (o_fluid(o, i, j - 1, k) ? o->alpha_v[V3(o, i, j, k)] : 0.0) : 1.0;
  const double an = j < ny - 1 ? (o_fluid(o, i, j + 1, k) ? o->alpha_v[V3(o, i, j + 1, k)] : 0.0) : 1.0;
  *wx = (aw - ae) * ax;
  *wy = (as - an) * ay;
}

void oracle_set_body(oracle *o, double xcirc, double ycirc, double Rcirc, const double *alpha_u,
                     const double *alpha_v) {
  const long NU = (long)(o->nx + 1) * o->ny * o->nz, NV = (long)o->nx * (o->ny + 1) * o->nz;
  free(o->alpha_u); free(o->alpha_v);
  o->alpha_u = (double *)xcalloc((size_t)NU, 8);
  o->alpha_v = (double *)xcalloc((size_t)NV, 8);
  memcpy(o->alpha_u, alpha_u, sizeof(double) * (size_t)NU);
  memcpy(o->alpha_v, alpha_v, sizeof(double) * (size_t)NV);
  o->xcirc = xcirc; o->ycirc = ycirc; o->Rcirc = Rcirc;
  o->body_set = 1;
}

/* Cut-surface force: shear nu w u over the u, v, w rows, then pressure over
 * the fluid cells. */
static void forces_cut(const oracle *o, double f[3]) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const double nu = o->prm.nu;
  f[0] = f[1] = f[2] = 0.0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i < nx; ++i)
        if (o->in.active_u[U3(o, i, j, k)]) f[0] += nu * cut_shear_weight(o, 0, i, j, k) * o->u[U3(o, i, j, k)];
  for (int k = 0; k < nz; ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        if (o->in.active_v[V3(o, i, j, k)]) f[1] += nu * cut_shear_weight(o, 1, i, j, k) * o->v[V3(o, i, j, k)];
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        if (o->in.active_w[W3(o, i, j, k)]) f[2] += nu * cut_shear_weight(o, 2, i, j, k) * o->w[W3(o, i, j, k)];
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (!o_fluid(o, i, j, k)) continue;
        double wx, wy;
        cut_pressure_weight(o, i, j, k, &wx, &wy);
        const double pc = o->p[((long)k * ny + j) * nx + i];
        f[0] += wx * pc;
        f[1] += wy * pc;
      }
}

void oracle_forces(const oracle *o, double f[3]) {
  if (o->body_set) {
    forces_cut(o, f);
    return;
  }
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const double dx = o->dx, dy = o->dy, dz = o->dz, t2 = 2.0 * o->prm.rho * o->prm.nu;
  const double ax = dy * dz, ay = dx * dz, az = dx * dy;
  f[0] = f[1] = f[2] = 0.0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (!o_fluid(o, i, j, k)) continue;
        const double pc = o->p[((long)k * ny + j) * nx + i];
        if (o_solid(o, i + 1, j, k)) f[0] += pc * ax;
        if (o_solid(o, i - 1, j, k)) f[0] -= pc * ax;
        if (o_solid(o, i, j + 1, k)) f[1] += pc * ay;
        if (o_solid(o, i, j - 1, k)) f[1] -= pc * ay;
        if (o_solid(o, i, j, k + 1)) f[2] += pc * az;
        if (o_solid(o, i, j, k - 1)) f[2] -= pc * az;
        if (i > 0 && o_fluid(o, i - 1, j, k)) {
          const double t = t2 * o->u[((long)k * ny + j) * (nx + 1) + i];
          if (o_solid(o, i - 1, j + 1, k) && o_solid(o, i, j + 1, k)) f[0] += t * dx * dz / dy;
          if (o_solid(o, i - 1, j - 1, k) && o_solid(o, i, j - 1, k)) f[0] += t * dx * dz / dy;
          if (o_solid(o, i - 1, j, k + 1) && o_solid(o, i, j, k + 1)) f[0] += t * dx * dy / dz;
          if (o_solid(o, i - 1, j, k - 1) && o_solid(o, i, j, k - 1)) f[0] += t * dx * dy / dz;
        }
        if (j > 0 && o_fluid(o, i, j - 1, k)) {
          const double t = t2 * o->v[((long)k * (ny + 1) + j) * nx + i];
          if (o_solid(o, i + 1, j - 1, k) && o_solid(o, i + 1, j, k)) f[1] += t * dy * dz / dx;
          if (o_solid(o, i - 1, j - 1, k) && o_solid(o, i - 1, j, k)) f[1] += t * dy * dz / dx;
          if (o_solid(o, i, j - 1, k + 1) && o_solid(o, i, j, k + 1)) f[1] += t * dx * dy / dz;
          if (o_solid(o, i, j - 1, k - 1) && o_solid(o, i, j, k - 1)) f[1] += t * dx * dy / dz;
        }
        if (k > 0 && o_fluid(o, i, j, k - 1)) {
          const double t = t2 * o->w[((long)k * ny + j) * nx + i];
          if (o_solid(o, i + 1, j, k - 1) && o_solid(o, i + 1, j, k)) f[2] += t * dz * dy / dx;
          if (o_solid(o, i - 1, j, k - 1) && o_solid(o, i - 1, j, k)) f[2] += t * dz * dy / dx;
          if (o_solid(o, i, j + 1, k - 1) && o_solid(o, i, j + 1, k)) f[2] += t * dz * dx / dy;
          if (o_solid(o, i, j - 1, k - 1) && o_solid(o, i, j - 1, k)) f[2] += t * dz * dx / dy;
        }
      }
}

static int all_finite(const double *x, long n) {
  for (long i = 0; i < n; ++i) if (!isfinite(x[i])) return 0;
  return 1;
}

/* One timestep, in the order of main.cu:249-368. */
int oracle_step(oracle *o, double ramp, oracle_step_stats *st) {
  memset(st, 0, sizeof(*st));
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const long NU = (long)(nx + 1) * ny * nz, NV = (long)nx * (ny + 1) * nz, NW = (long)nx * ny * (nz + 1),
             NP = (long)nx * ny * nz;
  double *uin = (double *)xcalloc((size_t)ny * nz, 8);
  for (long t = 0; t < (long)ny * nz; ++t) uin[t] = ramp * o->in.uin[t];
  oracle_bc_cleanup(o, o->u, o->v, o->w, uin);
  double *bu = (double *)xcalloc((size_t)o->bu.N, 8), *bv = (double *)xcalloc((size_t)o->bv.N, 8),
         *bw = (double *)xcalloc((size_t)o->bw.N, 8), *bp = (double *)xcalloc((size_t)NP, 8);
  double *xu = (double *)xcalloc((size_t)o->bu.N, 8), *xv = (double *)xcalloc((size_t)o->bv.N, 8),
         *xw = (double *)xcalloc((size_t)o->bw.N, 8), *xp = (double *)xcalloc((size_t)NP, 8);
  oracle_momentum_rhs(o, o->u, o->v, o->w, o->p, bu, bv, bw);
  if (!o->prm.use_zero_initial_guess) {
    for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) for (int i = 1; i < nx; ++i)
      xu[((long)k * ny + j) * (nx - 1) + (i - 1)] = o->u[U3(o, i, j, k)];
    for (int k = 0; k < nz; ++k) for (int j = 1; j < ny; ++j) for (int i = 0; i < nx; ++i)
      xv[((long)k * (ny - 1) + (j - 1)) * nx + i] = o->v[V3(o, i, j, k)];
    for (int k = 1; k < nz; ++k) for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i)
      xw[((long)(k - 1) * ny + j) * nx + i] = o->w[W3(o, i, j, k)];
  }
  oracle_solve(o, 0, bu, xu, &st->u);
  oracle_solve(o, 1, bv, xv, &st->v);
  oracle_solve(o, 2, bw, xw, &st->w);
  int rc = 0;
  if (!all_finite(xu, o->bu.N) || !all_finite(xv, o->bv.N) || !all_finite(xw, o->bw.N)) { rc = -3; goto done; }
  {
    double *ut = (double *)xcalloc((size_t)NU, 8), *vt = (double *)xcalloc((size_t)NV, 8), *wt = (double *)xcalloc((size_t)NW, 8);
    oracle_tilde(o, xu, xv, xw, ramp, ut, vt, wt);
    oracle_pressure_rhs(o, ut, vt, wt, ramp, bp);
    oracle_solve(o, 3, bp, xp, &st->p);
    if (!all_finite(xp, NP)) rc = -3;
    else oracle_projection(o, ut, vt, wt, xp, ramp, st);
    free(ut); free(vt); free(wt);
  }
done:
  st->status = rc;
  free(uin); free(bu); free(bv); free(bw); free(bp); free(xu); free(xv); free(xw); free(xp);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* adjoint of one step (the adjoint extension; the reference has none)      */
/* ------------------------------------------------------------------------ */

static int u_in(const oracle *o, int i, int j, int k) {
  return !(i < 0 || i > o->nx || j < 0 || j >= o->ny || k < 0 || k >= o->nz);
}
static int v_in(const oracle *o, int i, int j, int k) {
  return !(i < 0 || i >= o->nx || j < 0 || j > o->ny || k < 0 || k >= o->nz);
}
static int w_in(const oracle *o, int i, int j, int k) {
  return !(i < 0 || i >= o->nx || j < 0 || j >= o->ny || k < 0 || k > o->nz);
}

/* Adjoint of oracle_bc_cleanup with inlet values ramp * g, in reverse order:
 * the lambdas of the faces the cleanup overwrites become 0, the outlet copy
 * u[nx] = u[nx-1] hands its lambda to u[nx-1], and the inlet lambdas times
 * ramp accumulate into dg[j + ny k]. */
static void bc_adjoint(const oracle *o, double *lu, double *lv, double *lw, double ramp, double *dg) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        if (!o->in.active_w[W3(o, i, j, k - 1)]) lw[W3(o, i, j, k)] = 0.0;
  for (int k = 0; k < nz; ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        if (!o->in.active_v[V3(o, i, j, k)]) lv[V3(o, i, j, k)] = 0.0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i < nx; ++i)
        if (!o->in.active_u[U3(o, i, j, k)]) lu[U3(o, i, j, k)] = 0.0;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) { lw[W3(o, i, j, 0)] = 0.0; lw[W3(o, i, j, nz)] = 0.0; }
  for (int k = 0; k < nz; ++k)
    for (int i = 0; i < nx; ++i) { lv[V3(o, i, 0, k)] = 0.0; lv[V3(o, i, ny, k)] = 0.0; }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) {
      lu[U3(o, nx - 1, j, k)] += lu[U3(o, nx, j, k)];
      lu[U3(o, nx, j, k)] = 0.0;
      if (dg) dg[j + (long)ny * k] += ramp * lu[U3(o, 0, j, k)];
      lu[U3(o, 0, j, k)] = 0.0;
    }
}

/* Scatter helpers of the convection adjoint: add to a neighbour when it lies
 * inside its array, else to the centre (the forward's fallback) or nowhere
 * (the averages' zero fallback). */
static void add_u(const oracle *o, double *lu, int i, int j, int k, double g, long fb) {
  if (u_in(o, i, j, k)) lu[U3(o, i, j, k)] += g; else if (fb >= 0) lu[fb] += g;
}
static void add_v(const oracle *o, double *lv, int i, int j, int k, double g, long fb) {
  if (v_in(o, i, j, k)) lv[V3(o, i, j, k)] += g; else if (fb >= 0) lv[fb] += g;
}
static void add_w(const oracle *o, double *lw, int i, int j, int k, double g, long fb) {
  if (w_in(o, i, j, k)) lw[W3(o, i, j, k)] += g; else if (fb >= 0) lw[fb] += g;
}

/* lambda += J^T lc for the centred advective form of oracle_convection,
 * linearised at (u, v, w); lc is zero where no convection is computed. */
static void conv_adjoint(const oracle *o, const double *u, const double *v, const double *w, const double *lcu,
                         const double *lcv, const double *lcw, double *lu, double *lv, double *lw) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const double tdx = 2 * o->dx, tdy = 2 * o->dy, tdz = 2 * o->dz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i < nx; ++i) {
        const long f = U3(o, i, j, k);
        const double g = lcu[f];
        if (g == 0.0) continue;
        const double uc = u[f];
        const double va = 0.25 * (vval(o, v, i - 1, j, k, 0.0) + vval(o, v, i - 1, j + 1, k, 0.0) +
                                  vval(o, v, i, j, k, 0.0) + vval(o, v, i, j + 1, k, 0.0));
        const double wa = 0.25 * (wval(o, w, i - 1, j, k, 0.0) + wval(o, w, i - 1, j, k + 1, 0.0) +
                                  wval(o, w, i, j, k, 0.0) + wval(o, w, i, j, k + 1, 0.0));
        const double ue = uval(o, u, i + 1, j, k, uc), uw = uval(o, u, i - 1, j, k, uc);
        const double un = uval(o, u, i, j + 1, k, uc), us = uval(o, u, i, j - 1, k, uc);
        const double ut = uval(o, u, i, j, k + 1, uc), ub = uval(o, u, i, j, k - 1, uc);
        const double gx = g / tdx, gy = g / tdy, gz = g / tdz;
        lu[f] += gx * (ue - uw);
        add_u(o, lu, i + 1, j, k, gx * uc, f); add_u(o, lu, i - 1, j, k, -gx * uc, f);
        add_u(o, lu, i, j + 1, k, gy * va, f); add_u(o, lu, i, j - 1, k, -gy * va, f);
        add_u(o, lu, i, j, k + 1, gz * wa, f); add_u(o, lu, i, j, k - 1, -gz * wa, f);
        const double cv = 0.25 * gy * (un - us), cw = 0.25 * gz * (ut - ub);
        add_v(o, lv, i - 1, j, k, cv, -1); add_v(o, lv, i - 1, j + 1, k, cv, -1);
        add_v(o, lv, i, j, k, cv, -1); add_v(o, lv, i, j + 1, k, cv, -1);
        add_w(o, lw, i - 1, j, k, cw, -1); add_w(o, lw, i - 1, j, k + 1, cw, -1);
        add_w(o, lw, i, j, k, cw, -1); add_w(o, lw, i, j, k + 1, cw, -1);
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long f = V3(o, i, j, k);
        const double g = lcv[f];
        if (g == 0.0) continue;
        const double vc = v[f];
        const double ua = 0.25 * (uval(o, u, i, j - 1, k, 0.0) + uval(o, u, i + 1, j - 1, k, 0.0) +
                                  uval(o, u, i, j, k, 0.0) + uval(o, u, i + 1, j, k, 0.0));
        const double wa = 0.25 * (wval(o, w, i, j - 1, k, 0.0) + wval(o, w, i, j, k, 0.0) +
                                  wval(o, w, i, j - 1, k + 1, 0.0) + wval(o, w, i, j, k + 1, 0.0));
        const double ve = vval(o, v, i + 1, j, k, vc), vw = vval(o, v, i - 1, j, k, vc);
        const double vn = vval(o, v, i, j + 1, k, vc), vs = vval(o, v, i, j - 1, k, vc);
        const double vt = vval(o, v, i, j, k + 1, vc), vb = vval(o, v, i, j, k - 1, vc);
        const double gx = g / tdx, gy = g / tdy, gz = g / tdz;
        lv[f] += gy * (vn - vs);
        add_v(o, lv, i + 1, j, k, gx * ua, f); add_v(o, lv, i - 1, j, k, -gx * ua, f);
        add_v(o, lv, i, j + 1, k, gy * vc, f); add_v(o, lv, i, j - 1, k, -gy * vc, f);
        add_v(o, lv, i, j, k + 1, gz * wa, f); add_v(o, lv, i, j, k - 1, -gz * wa, f);
        const double cu = 0.25 * gx * (ve - vw), cw = 0.25 * gz * (vt - vb);
        add_u(o, lu, i, j - 1, k, cu, -1); add_u(o, lu, i + 1, j - 1, k, cu, -1);
        add_u(o, lu, i, j, k, cu, -1); add_u(o, lu, i + 1, j, k, cu, -1);
        add_w(o, lw, i, j - 1, k, cw, -1); add_w(o, lw, i, j, k, cw, -1);
        add_w(o, lw, i, j - 1, k + 1, cw, -1); add_w(o, lw, i, j, k + 1, cw, -1);
      }
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long f = W3(o, i, j, k);
        const double g = lcw[f];
        if (g == 0.0) continue;
        const double wc = w[f];
        const double ua = 0.25 * (uval(o, u, i, j, k - 1, 0.0) + uval(o, u, i + 1, j, k - 1, 0.0) +
                                  uval(o, u, i, j, k, 0.0) + uval(o, u, i + 1, j, k, 0.0));
        const double va = 0.25 * (vval(o, v, i, j, k - 1, 0.0) + vval(o, v, i, j + 1, k - 1, 0.0) +
                                  vval(o, v, i, j, k, 0.0) + vval(o, v, i, j + 1, k, 0.0));
        const double we = wval(o, w, i + 1, j, k, wc), ww = wval(o, w, i - 1, j, k, wc);
        const double wn = wval(o, w, i, j + 1, k, wc), ws = wval(o, w, i, j - 1, k, wc);
        const double wt = wval(o, w, i, j, k + 1, wc), wb = wval(o, w, i, j, k - 1, wc);
        const double gx = g / tdx, gy = g / tdy, gz = g / tdz;
        lw[f] += gz * (wt - wb);
        add_w(o, lw, i + 1, j, k, gx * ua, f); add_w(o, lw, i - 1, j, k, -gx * ua, f);
        add_w(o, lw, i, j + 1, k, gy * va, f); add_w(o, lw, i, j - 1, k, -gy * va, f);
        add_w(o, lw, i, j, k + 1, gz * wc, f); add_w(o, lw, i, j, k - 1, -gz * wc, f);
        const double cu = 0.25 * gx * (we - ww), cv = 0.25 * gy * (wn - ws);
        add_u(o, lu, i, j, k - 1, cu, -1); add_u(o, lu, i + 1, j, k - 1, cu, -1);
        add_u(o, lu, i, j, k, cu, -1); add_u(o, lu, i + 1, j, k, cu, -1);
        add_v(o, lv, i, j, k - 1, cv, -1); add_v(o, lv, i, j + 1, k - 1, cv, -1);
        add_v(o, lv, i, j, k, cv, -1); add_v(o, lv, i, j + 1, k, cv, -1);
      }
}

/* lambda += weight dF_x/d(u, p) for the x force of oracle_forces at the
 * oracle's current fields; *dnu += weight dF_x/dnu (the shear terms are
 * proportional to nu). */
static void force_x_adjoint(const oracle *o, double weight, double *lu, double *lp, double *dnu) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  if (o->body_set) {  /* cut-surface force: linear in u and p */
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 1; i < nx; ++i) {
          const long f = U3(o, i, j, k);
          if (!o->in.active_u[f]) continue;
          const double s = cut_shear_weight(o, 0, i, j, k);
          lu[f] += weight * o->prm.nu * s;
          *dnu += weight * s * o->u[f];
        }
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          if (!o_fluid(o, i, j, k)) continue;
          double wx, wy;
          cut_pressure_weight(o, i, j, k, &wx, &wy);
          lp[((long)k * ny + j) * nx + i] += weight * wx;
        }
    return;
  }
  const double dx = o->dx, dy = o->dy, dz = o->dz, t2 = 2.0 * o->prm.rho * o->prm.nu;
  const double ax = dy * dz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (!o_fluid(o, i, j, k)) continue;
        const long c = ((long)k * ny + j) * nx + i;
        if (o_solid(o, i + 1, j, k)) lp[c] += weight * ax;
        if (o_solid(o, i - 1, j, k)) lp[c] -= weight * ax;
        if (i > 0 && o_fluid(o, i - 1, j, k)) {
          double s = 0.0;
          if (o_solid(o, i - 1, j + 1, k) && o_solid(o, i, j + 1, k)) s += dx * dz / dy;
          if (o_solid(o, i - 1, j - 1, k) && o_solid(o, i, j - 1, k)) s += dx * dz / dy;
          if (o_solid(o, i - 1, j, k + 1) && o_solid(o, i, j, k + 1)) s += dx * dy / dz;
          if (o_solid(o, i - 1, j, k - 1) && o_solid(o, i, j, k - 1)) s += dx * dy / dz;
          const long f = U3(o, i, j, k);
          lu[f] += weight * t2 * s;
          *dnu += weight * 2.0 * o->prm.rho * o->u[f] * s;
        }
      }
}

/* z += A^T-like transpose of a 1-based CSR: z[col] += val * y[row]. */
static void csr_apply_t(const int32_t *rp, const int32_t *col, const double *val, long nrows, const double *y,
                        double *z) {
  for (long r = 0; r < nrows; ++r)
    for (int t = rp[r]; t < rp[r + 1]; ++t) z[col[t]] += val[t] * y[r + 1];
}

/* Reverse sweep of one step (see ibm_oracle.h). */
int oracle_step_backward(oracle *o, oracle *ot, double ramp, const double *beta_p, double weight, double *lu,
                         double *lv, double *lw, double *lp, double *dg, double *dnu) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const long NU = (long)(nx + 1) * ny * nz, NV = (long)nx * (ny + 1) * nz, NW = (long)nx * ny * (nz + 1),
             NP = (long)nx * ny * nz;
  const double a = o->prm.rho / o->prm.dt, rho = o->prm.rho, nu = o->prm.nu, factor = o->prm.dt / o->prm.rho;
  double *u0 = (double *)xcalloc((size_t)NU, 8), *v0 = (double *)xcalloc((size_t)NV, 8),
         *w0 = (double *)xcalloc((size_t)NW, 8), *p0 = (double *)xcalloc((size_t)NP, 8);
  oracle_get_fields(o, u0, v0, w0, p0);
  /* recompute: U1 = BC(U0), the momentum right-hand sides and solutions, and
   * the end-of-step fields (the objective's linearisation point) */
  double *uin = (double *)xcalloc((size_t)ny * nz, 8);
  for (long t = 0; t < (long)ny * nz; ++t) uin[t] = ramp * o->in.uin[t];
  oracle_bc_cleanup(o, o->u, o->v, o->w, uin);
  double *u1 = (double *)xcalloc((size_t)NU, 8), *v1 = (double *)xcalloc((size_t)NV, 8),
         *w1 = (double *)xcalloc((size_t)NW, 8);
  memcpy(u1, o->u, 8 * (size_t)NU); memcpy(v1, o->v, 8 * (size_t)NV); memcpy(w1, o->w, 8 * (size_t)NW);
  const long nb[3] = {o->bu.N, o->bv.N, o->bw.N};
  double *b[3], *x[3];
  for (int f = 0; f < 3; ++f) { b[f] = (double *)xcalloc((size_t)nb[f], 8); x[f] = (double *)xcalloc((size_t)nb[f], 8); }
  oracle_momentum_rhs(o, o->u, o->v, o->w, o->p, b[0], b[1], b[2]);
  oracle_solve_stats ss;
  int rc = 0;
  for (int f = 0; f < 3; ++f) { oracle_solve(o, f, b[f], x[f], &ss); if (ss.status < 0) rc = -3; }
  {
    double *ut = (double *)xcalloc((size_t)NU, 8), *vt = (double *)xcalloc((size_t)NV, 8), *wt = (double *)xcalloc((size_t)NW, 8);
    double *bp = (double *)xcalloc((size_t)NP, 8), *xp = (double *)xcalloc((size_t)NP, 8);
    oracle_step_stats st;
    oracle_tilde(o, x[0], x[1], x[2], ramp, ut, vt, wt);
    oracle_pressure_rhs(o, ut, vt, wt, ramp, bp);
    oracle_solve(o, 3, bp, xp, &ss);
    oracle_projection(o, ut, vt, wt, xp, ramp, &st);
    free(ut); free(vt); free(wt); free(bp); free(xp);
  }
  /* the objective's share of this step: weight * F_x at the end-of-step fields */
  if (weight != 0.0) force_x_adjoint(o, weight, lu, lp, dnu);
  /* BC cleanup after the projection */
  bc_adjoint(o, lu, lv, lw, ramp, dg);
  /* projection: q = q~ - (dt/rho) G phi, p += phi */
  double *lq = (double *)xcalloc((size_t)o->nQ + 1, 8), *lphi = (double *)xcalloc((size_t)o->nP + 1, 8);
  pack_q(o, lu, lv, lw, lq);
  csr_apply_t(o->in.G_rowptr, o->in.G_col, o->in.G_val, o->nQ, lq, lphi);
  double *rphi = (double *)xcalloc((size_t)NP, 8), *mu = (double *)xcalloc((size_t)NP, 8);
  for (long c = 0; c < NP; ++c) {
    const int id = o->in.id_p[c];
    if (o->in.fluid_p[c] && id > 0) rphi[c] = lp[c] - factor * lphi[id];
  }
  /* pressure solve: mu = Ap^-T lambda_phi */
  oracle_solve(ot, 3, rphi, mu, &ss);
  if (ss.status < 0) rc = -3;
  /* pressure right-hand side: b_p = -(rho/dt) (D q~ + ramp div_bc(g)) */
  double *ldq = (double *)xcalloc((size_t)o->nP + 1, 8);
  memset(lq, 0, sizeof(double) * ((size_t)o->nQ + 1));
  for (long c = 0; c < NP; ++c) {
    const int id = o->in.id_p[c];
    if (!(o->in.fluid_p[c] && id > 0)) continue;
    ldq[id] = -a * mu[c];
    const int i = (int)(c % nx);
    if (i == 0 && dg) {
      const long jk = c / nx;
      dg[jk] += a * ramp * mu[c] / (beta_p[c] * o->dx);
    }
  }
  csr_apply_t(o->in.D_rowptr, o->in.D_col, o->in.D_val, o->nP, ldq, lq);
  for (long f = 0; f < NU; ++f) { int id = o->in.id_qu[f]; if (id > 0) lu[f] += lq[id]; }
  for (long f = 0; f < NV; ++f) { int id = o->in.id_qv[f]; if (id > 0) lv[f] += lq[o->nQu + id]; }
  for (long f = 0; f < NW; ++f) { int id = o->in.id_qw[f]; if (id > 0) lw[f] += lq[o->nQu + o->nQv + id]; }
  /* BC cleanup of u~ */
  bc_adjoint(o, lu, lv, lw, ramp, dg);
  /* scatter: the solve-box interior of u~ is x, the rest is U1 */
  double *lx[3];
  for (int f = 0; f < 3; ++f) lx[f] = (double *)xcalloc((size_t)nb[f], 8);
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) for (int i = 1; i < nx; ++i) {
    const long f = U3(o, i, j, k);
    lx[0][((long)k * ny + j) * (nx - 1) + (i - 1)] = lu[f]; lu[f] = 0.0;
  }
  for (int k = 0; k < nz; ++k) for (int j = 1; j < ny; ++j) for (int i = 0; i < nx; ++i) {
    const long f = V3(o, i, j, k);
    lx[1][((long)k * (ny - 1) + (j - 1)) * nx + i] = lv[f]; lv[f] = 0.0;
  }
  for (int k = 1; k < nz; ++k) for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) {
    const long f = W3(o, i, j, k);
    lx[2][((long)(k - 1) * ny + j) * nx + i] = lw[f]; lw[f] = 0.0;
  }
  /* momentum solves: lambda_b = A^-T lambda_x; dnu from A(nu) and b(nu) */
  double *lcu = (double *)xcalloc((size_t)NU, 8), *lcv = (double *)xcalloc((size_t)NV, 8),
         *lcw = (double *)xcalloc((size_t)NW, 8);
  double *lgu = (double *)xcalloc((size_t)NU, 8), *lgv = (double *)xcalloc((size_t)NV, 8),
         *lgw = (double *)xcalloc((size_t)NW, 8);
  for (int fld = 0; fld < 3; ++fld) {
    double *lb = (double *)xcalloc((size_t)nb[fld], 8);
    oracle_solve(ot, fld, lx[fld], lb, &ss);
    if (ss.status < 0) rc = -3;
    const int bx = fld == 0 ? nx - 1 : nx, by = fld == 1 ? ny - 1 : ny, bz = fld == 2 ? nz - 1 : nz;
    for (int k = 0; k < bz; ++k)
      for (int j = 0; j < by; ++j)
        for (int i = 0; i < bx; ++i) {
          const long r = ((long)k * by + j) * bx + i;
          long f;
          int id, act;
          double sc, bc;
          if (fld == 0) {
            f = U3(o, i + 1, j, k); id = o->in.id_u[f]; act = o->in.active_u[f];
            sc = id > 0 ? o->in.scale_u[id] : 0.0; bc = id > 0 ? o->in.rhs_u_bc[id] : 0.0;
          } else if (fld == 1) {
            f = V3(o, i, j + 1, k); id = o->in.id_v[f]; act = o->in.active_v[f];
            sc = id > 0 ? o->in.scale_v[id] : 0.0; bc = id > 0 ? o->in.rhs_v_bc[id] : 0.0;
          } else {
            f = W3(o, i, j, k + 1); id = o->in.id_w[f]; act = o->in.active_w[f];
            sc = id > 0 ? o->in.scale_w[id] : 0.0; bc = id > 0 ? o->in.rhs_w_bc[id] : 0.0;
          }
          if (!(id > 0 && act)) continue;
          *dnu += lb[r] * (a * sc * x[fld][r] + sc * bc - b[fld][r]) / nu;
          const double lt = sc * lb[r];
          double *lf = fld == 0 ? lu : fld == 1 ? lv : lw;
          double *lc = fld == 0 ? lcu : fld == 1 ? lcv : lcw;
          double *lg = fld == 0 ? lgu : fld == 1 ? lgv : lgw;
          lf[f] += a * lt;
          lc[f] = -rho * lt;
          lg[f] = -lt;
        }
    free(lb);
  }
  /* convection at U1 (the w rows use the active mask one plane below) */
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        if (!o->in.active_w[W3(o, i, j, k - 1)]) lcw[W3(o, i, j, k)] = 0.0;
  for (long f = 0; f < NU; ++f) if (!o->in.active_u[f]) lcu[f] = 0.0;
  for (long f = 0; f < NV; ++f) if (!o->in.active_v[f]) lcv[f] = 0.0;
  conv_adjoint(o, u1, v1, w1, lcu, lcv, lcw, lu, lv, lw);
  /* gradient of p^n on the q-faces */
  memset(lq, 0, sizeof(double) * ((size_t)o->nQ + 1));
  memset(lphi, 0, sizeof(double) * ((size_t)o->nP + 1));
  pack_q(o, lgu, lgv, lgw, lq);
  csr_apply_t(o->in.G_rowptr, o->in.G_col, o->in.G_val, o->nQ, lq, lphi);
  for (long c = 0; c < NP; ++c) {
    const int id = o->in.id_p[c];
    if (o->in.fluid_p[c] && id > 0) lp[c] += lphi[id];
  }
  /* BC cleanup at the start of the step */
  bc_adjoint(o, lu, lv, lw, ramp, dg);
  oracle_set_fields(o, u0, v0, w0, p0);
  free(u0); free(v0); free(w0); free(p0); free(uin); free(u1); free(v1); free(w1);
  for (int f = 0; f < 3; ++f) { free(b[f]); free(x[f]); free(lx[f]); }
  free(lq); free(lphi); free(rphi); free(mu); free(ldq);
  free(lcu); free(lcv); free(lcw); free(lgu); free(lgv); free(lgw);
  return rc;
}

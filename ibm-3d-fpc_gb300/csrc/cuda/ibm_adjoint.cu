// Reverse sweep of one step (the adjoint extension; the reference has none).
//
// Each kernel is the transpose of one dense piece of the step (ibm_step.cu),
// linearised where the piece is nonlinear (the convection, at the post-BC
// step-start velocities). Gathers where the transpose has a fixed shape (G^T,
// D^T, the BC and the scatter); FP64 atomics for the convection, whose
// transpose scatters each face's lambda to its 14 inputs. The sums are not
// bitwise reproducible from run to run; the checks use tolerances.
#include <algorithm>
#include <cmath>

#include "ibm_adjoint.cuh"

namespace ibm {

AdjState::~AdjState() {
  if (gexec) cudaGraphExecDestroy(gexec);
  if (hweight) cudaFreeHost(hweight);
}

namespace {

int adj_grid(long n) {
  const long b = (n + kThreads - 1) / kThreads;
  return (int)std::max(1L, std::min(b, (long)sm_count() * 8));
}

struct ADims {
  int nx, ny, nz;
  __device__ long U(int i, int j, int k) const { return ((long)k * ny + j) * (nx + 1) + i; }
  __device__ long V(int i, int j, int k) const { return ((long)k * (ny + 1) + j) * nx + i; }
  __device__ long W(int i, int j, int k) const { return ((long)k * ny + j) * nx + i; }
  __device__ long P(int i, int j, int k) const { return ((long)k * ny + j) * nx + i; }
  __device__ bool u_in(int i, int j, int k) const { return i >= 0 && i <= nx && j >= 0 && j < ny && k >= 0 && k < nz; }
  __device__ bool v_in(int i, int j, int k) const { return i >= 0 && i < nx && j >= 0 && j <= ny && k >= 0 && k < nz; }
  __device__ bool w_in(int i, int j, int k) const { return i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k <= nz; }
};
ADims adims(const ibm_ctx *c) { return ADims{c->g.nx, c->g.ny, c->g.nz}; }

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double s[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) s[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += s[q];
  return t;  // valid in thread 0
}

__global__ void k_transpose7(const double *c, Box b, double *rows) {
  const long n = b.n, sy = b.nx, sz = (long)b.nx * b.ny;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    const int i = (int)(r % b.nx), j = (int)((r / b.nx) % b.ny), k = (int)(r / sz);
    double *o = rows + 7 * r;
    o[0] = c[r];
    o[1] = i > 0 ? c[2 * n + r - 1] : 0.0;
    o[2] = i < b.nx - 1 ? c[1 * n + r + 1] : 0.0;
    o[3] = j > 0 ? c[4 * n + r - sy] : 0.0;
    o[4] = j < b.ny - 1 ? c[3 * n + r + sy] : 0.0;
    o[5] = k > 0 ? c[6 * n + r - sz] : 0.0;
    o[6] = k < b.nz - 1 ? c[5 * n + r + sz] : 0.0;
  }
}

__global__ void k_zero_lists(double *u, const int *lu, int nu_, double *v, const int *lv, int nv_, double *w,
                             const int *lw, int nw_) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nu_ || t < nv_ || t < nw_;
       t += (long)gridDim.x * blockDim.x) {
    if (t < nu_) u[lu[t]] = 0.0;
    if (t < nv_) v[lv[t]] = 0.0;
    if (t < nw_) w[lw[t]] = 0.0;
  }
}

// Reverse of the boundary planes of the BC cleanup (k_bc_planes): outlet copy
// u[nx] = u[nx-1], inlet u[0] = ramp g, wall v and w set to zero.
__global__ void k_bc_planes_t(double *lu, double *lv, double *lw, double *dg, const double *rampp, ADims d) {
  const double ramp = *rampp;
  const long n = std::max((long)d.ny * d.nz, std::max((long)d.nx * d.nz, (long)d.nx * d.ny));
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    if (t < (long)d.ny * d.nz) {
      const int j = (int)(t % d.ny), k = (int)(t / d.ny);
      const long fo = d.U(d.nx, j, k), fl = d.U(d.nx - 1, j, k), fi = d.U(0, j, k);
      lu[fl] += lu[fo];
      lu[fo] = 0.0;
      dg[t] += ramp * lu[fi];
      lu[fi] = 0.0;
    }
    if (t < (long)d.nx * d.nz) {
      const int i = (int)(t % d.nx), k = (int)(t / d.nx);
      lv[d.V(i, 0, k)] = 0.0;
      lv[d.V(i, d.ny, k)] = 0.0;
    }
    if (t < (long)d.nx * d.ny) {
      lw[t] = 0.0;
      lw[(long)d.nz * d.nx * d.ny + t] = 0.0;
    }
  }
}

// The x force of k_forces (staircase definition) is linear in p and u:
// lambda += weight dF_x/d(p, u), acc += weight dF_x/dnu.
__global__ void k_force_t(const uint8_t *fc, const double *u, double *lu, double *lp, double *acc, ADims d,
                          double dx, double dy, double dz, double rho, double nu, const double *weightp) {
  const double weight = *weightp;
  if (weight == 0.0) return;
  const long NP = (long)d.nx * d.ny * d.nz;
  auto fluid = [&](int i, int j, int k) { return (fc[d.P(i, j, k)] & kFluid) != 0; };
  auto solid = [&](int i, int j, int k) {
    return i >= 0 && i < d.nx && j >= 0 && j < d.ny && k >= 0 && k < d.nz && !fluid(i, j, k);
  };
  const double ax = dy * dz, t2 = 2.0 * rho * nu;
  double dn = 0.0;
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < NP; c += (long)gridDim.x * blockDim.x) {
    if (!(fc[c] & kFluid)) continue;
    const int i = (int)(c % d.nx), j = (int)((c / d.nx) % d.ny), k = (int)(c / ((long)d.nx * d.ny));
    double g = 0.0;
    if (solid(i + 1, j, k)) g += weight * ax;
    if (solid(i - 1, j, k)) g -= weight * ax;
    lp[c] += g;
    if (i > 0 && fluid(i - 1, j, k)) {
      double s = 0.0;
      if (solid(i - 1, j + 1, k) && solid(i, j + 1, k)) s += dx * dz / dy;
      if (solid(i - 1, j - 1, k) && solid(i, j - 1, k)) s += dx * dz / dy;
      if (solid(i - 1, j, k + 1) && solid(i, j, k + 1)) s += dx * dy / dz;
      if (solid(i - 1, j, k - 1) && solid(i, j, k - 1)) s += dx * dy / dz;
      if (s != 0.0) {
        const long f = d.U(i, j, k);
        lu[f] += weight * t2 * s;
        dn += weight * 2.0 * rho * u[f] * s;
      }
    }
  }
  const double b = block_sum(dn);
  if (threadIdx.x == 0 && b != 0.0) atomicAdd(acc, b);
}

// G^T of face lambdas at each fluid cell: mode 0 writes base + coef G^T l
// (0 on non-fluid cells), mode 1 adds coef G^T l to out on fluid cells.
// G's face coefficients: [f] for the lower cell, [NF + f] for the upper cell.
struct GradTArgs {
  ADims d;
  const uint8_t *fu, *fv, *fw, *fc;
  const double *Gu, *Gv, *Gw;
  const double *lu, *lv, *lw;
  const double *base;
  double coef;
  double *out;
  int mode;
};
__global__ void k_grad_t(GradTArgs A) {
  const ADims &d = A.d;
  const long NU = (long)(d.nx + 1) * d.ny * d.nz, NV = (long)d.nx * (d.ny + 1) * d.nz,
             NW = (long)d.nx * d.ny * (d.nz + 1), NP = (long)d.nx * d.ny * d.nz;
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < NP; c += (long)gridDim.x * blockDim.x) {
    if (!(A.fc[c] & kFluid)) {
      if (A.mode == 0) A.out[c] = 0.0;
      continue;
    }
    const int i = (int)(c % d.nx), j = (int)((c / d.nx) % d.ny), k = (int)(c / ((long)d.nx * d.ny));
    double s = 0.0;
    long f = d.U(i, j, k);
    if (A.fu[f] & kQFace) s += A.Gu[NU + f] * A.lu[f];
    f = d.U(i + 1, j, k);
    if (A.fu[f] & kQFace) s += A.Gu[f] * A.lu[f];
    f = d.V(i, j, k);
    if (A.fv[f] & kQFace) s += A.Gv[NV + f] * A.lv[f];
    f = d.V(i, j + 1, k);
    if (A.fv[f] & kQFace) s += A.Gv[f] * A.lv[f];
    f = d.W(i, j, k);
    if (A.fw[f] & kQFace) s += A.Gw[NW + f] * A.lw[f];
    f = d.W(i, j, k + 1);
    if (A.fw[f] & kQFace) s += A.Gw[f] * A.lw[f];
    if (A.mode == 0) A.out[c] = A.base[c] + A.coef * s;
    else A.out[c] += A.coef * s;
  }
}

// lambda += coef D^T mu on the q-faces: a face's D coefficients are the
// lower cell's east / north / top slot and the upper cell's west / south /
// bottom slot (Dc [6][NP]: u_w, u_e, v_s, v_n, w_b, w_t).
__global__ void k_div_t(ADims d, const uint8_t *fu, const uint8_t *fv, const uint8_t *fw, const uint8_t *fc,
                        const double *Dc, const double *mu, double coef, double *lu, double *lv, double *lw) {
  const long NU = (long)(d.nx + 1) * d.ny * d.nz, NV = (long)d.nx * (d.ny + 1) * d.nz,
             NW = (long)d.nx * d.ny * (d.nz + 1), NP = (long)d.nx * d.ny * d.nz;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < NU + NV + NW; t += (long)gridDim.x * blockDim.x) {
    long lo = -1, hi = -1;
    int slo = 0, shi = 0;
    double *l;
    long f;
    if (t < NU) {
      f = t;
      if (!(fu[f] & kQFace)) continue;
      const int i = (int)(f % (d.nx + 1));
      const long q = f / (d.nx + 1);
      const int j = (int)(q % d.ny), k = (int)(q / d.ny);
      if (i > 0) { lo = d.P(i - 1, j, k); slo = 1; }
      if (i < d.nx) { hi = d.P(i, j, k); shi = 0; }
      l = lu;
    } else if (t < NU + NV) {
      f = t - NU;
      if (!(fv[f] & kQFace)) continue;
      const int i = (int)(f % d.nx);
      const long q = f / d.nx;
      const int j = (int)(q % (d.ny + 1)), k = (int)(q / (d.ny + 1));
      if (j > 0) { lo = d.P(i, j - 1, k); slo = 3; }
      if (j < d.ny) { hi = d.P(i, j, k); shi = 2; }
      l = lv;
    } else {
      f = t - NU - NV;
      if (!(fw[f] & kQFace)) continue;
      const long plane = (long)d.nx * d.ny;
      const int k = (int)(f / plane);
      const long c0 = f - (long)k * plane;
      if (k > 0) { lo = c0 + (long)(k - 1) * plane; slo = 5; }
      if (k < d.nz) { hi = c0 + (long)k * plane; shi = 4; }
      l = lw;
    }
    double s = 0.0;
    if (lo >= 0 && (fc[lo] & kFluid)) s += Dc[(long)slo * NP + lo] * mu[lo];
    if (hi >= 0 && (fc[hi] & kFluid)) s += Dc[(long)shi * NP + hi] * mu[hi];
    l[f] += coef * s;
  }
}

// dg += coef ramp mu / (beta dx) on the inlet column (cell (0, j, k) = t nx).
__global__ void k_inlet_t(double *dg, const double *mu, const double *winl, double coef, const double *ramp, int nx,
                          int nyz) {
  coef *= *ramp;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nyz; t += gridDim.x * blockDim.x)
    if (winl[t] != 0.0) dg[t] += coef * mu[(long)t * nx] * winl[t];
}

// lx = lambda at the solve-box interior faces (box row order), which become 0.
__global__ void k_scatter_t(ADims d, double *lu, double *lv, double *lw, double *xu, double *xv, double *xw) {
  const long nu_ = (long)(d.nx - 1) * d.ny * d.nz, nv_ = (long)d.nx * (d.ny - 1) * d.nz,
             nw_ = (long)d.nx * d.ny * (d.nz - 1);
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nu_ + nv_ + nw_; t += (long)gridDim.x * blockDim.x) {
    if (t < nu_) {
      const long r = t;
      const int i = (int)(r % (d.nx - 1)) + 1;
      const long q = r / (d.nx - 1);
      const long f = d.U(i, (int)(q % d.ny), (int)(q / d.ny));
      xu[r] = lu[f];
      lu[f] = 0.0;
    } else if (t < nu_ + nv_) {
      const long r = t - nu_;
      const int i = (int)(r % d.nx);
      const long q = r / d.nx;
      const long f = d.V(i, (int)(q % (d.ny - 1)) + 1, (int)(q / (d.ny - 1)));
      xv[r] = lv[f];
      lv[f] = 0.0;
    } else {
      const long r = t - nu_ - nv_;
      const long f = r + (long)d.nx * d.ny;  // w box rows are the faces of planes 1..nz-1
      xw[r] = lw[f];
      lw[f] = 0.0;
    }
  }
}

// From lb = A^-T lx on the box rows: b = ((rho/dt) u - rho conv - G p + bc) sc
// gives lambda_u += (rho/dt) sc lb, conv lambda -rho sc lb (where the
// convection is computed), gradient lambda -sc lb (q-faces); with A and b
// depending on nu through the row scale (A = sc (rho/dt I + nu L)):
// dJ/dnu += lb (rho/dt sc x + sc bc - b) / nu (using A x = b).
struct MomTArgs {
  ADims d;
  const uint8_t *fu, *fv, *fw;
  const double *sc[3], *bc[3], *b[3], *x[3], *lb[3];
  long nb[3];
  double *lu, *lv, *lw, *cu, *cv, *cw, *gu, *gv, *gw;
  double a, rho, nu;
  double *acc;
};
__global__ void k_mom_t(MomTArgs A) {
  const ADims &d = A.d;
  const long total = A.nb[0] + A.nb[1] + A.nb[2];
  const long plane = (long)d.nx * d.ny;
  double dn = 0.0;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    int fld;
    long r, f;
    if (t < A.nb[0]) {
      fld = 0; r = t;
      const int i = (int)(r % (d.nx - 1)) + 1;
      const long q = r / (d.nx - 1);
      f = d.U(i, (int)(q % d.ny), (int)(q / d.ny));
    } else if (t < A.nb[0] + A.nb[1]) {
      fld = 1; r = t - A.nb[0];
      const int i = (int)(r % d.nx);
      const long q = r / d.nx;
      f = d.V(i, (int)(q % (d.ny - 1)) + 1, (int)(q / (d.ny - 1)));
    } else {
      fld = 2; r = t - A.nb[0] - A.nb[1];
      f = r + plane;
    }
    const uint8_t fl = fld == 0 ? A.fu[f] : fld == 1 ? A.fv[f] : A.fw[f];
    if (!(fl & kRhsRow)) continue;
    const double sc = A.sc[fld][r], lb = A.lb[fld][r];
    dn += lb * (A.a * sc * A.x[fld][r] + sc * A.bc[fld][r] - A.b[fld][r]);
    const double lt = sc * lb;
    const bool conv = fld < 2 ? (fl & kActive) != 0 : (A.fw[f - plane] & kActive) != 0;
    double *lf = fld == 0 ? A.lu : fld == 1 ? A.lv : A.lw;
    double *lc = fld == 0 ? A.cu : fld == 1 ? A.cv : A.cw;
    double *lg = fld == 0 ? A.gu : fld == 1 ? A.gv : A.gw;
    lf[f] += A.a * lt;
    if (conv) lc[f] = -A.rho * lt;
    if (fl & kQFace) lg[f] = -lt;
  }
  const double s = block_sum(dn);
  if (threadIdx.x == 0 && s != 0.0) atomicAdd(A.acc, s / A.nu);
}

// Transpose of the centred advective form (k_momentum_rhs), linearised at
// (u, v, w): each face with a convection lambda g adds g times the partial
// derivatives to its inputs; an out-of-range neighbour falls back to the
// centre value (its share goes to the centre), an out-of-range velocity of an
// average falls back to 0 (no share).
struct ConvTArgs {
  ADims d;
  const double *u, *v, *w, *cu, *cv, *cw;
  double *lu, *lv, *lw;
  double rtx, rty, rtz;  // 1 / (2 dx), 1 / (2 dy), 1 / (2 dz)
};
__device__ __forceinline__ double ldu(const ConvTArgs &A, int i, int j, int k, double fb) {
  return A.d.u_in(i, j, k) ? A.u[A.d.U(i, j, k)] : fb;
}
__device__ __forceinline__ double ldv(const ConvTArgs &A, int i, int j, int k, double fb) {
  return A.d.v_in(i, j, k) ? A.v[A.d.V(i, j, k)] : fb;
}
__device__ __forceinline__ double ldw(const ConvTArgs &A, int i, int j, int k, double fb) {
  return A.d.w_in(i, j, k) ? A.w[A.d.W(i, j, k)] : fb;
}
__device__ __forceinline__ void addu(const ConvTArgs &A, int i, int j, int k, double g, long fb) {
  if (A.d.u_in(i, j, k)) atomicAdd(&A.lu[A.d.U(i, j, k)], g);
  else if (fb >= 0) atomicAdd(&A.lu[fb], g);
}
__device__ __forceinline__ void addv(const ConvTArgs &A, int i, int j, int k, double g, long fb) {
  if (A.d.v_in(i, j, k)) atomicAdd(&A.lv[A.d.V(i, j, k)], g);
  else if (fb >= 0) atomicAdd(&A.lv[fb], g);
}
__device__ __forceinline__ void addw(const ConvTArgs &A, int i, int j, int k, double g, long fb) {
  if (A.d.w_in(i, j, k)) atomicAdd(&A.lw[A.d.W(i, j, k)], g);
  else if (fb >= 0) atomicAdd(&A.lw[fb], g);
}
__global__ void k_conv_t(ConvTArgs A) {
  const ADims &d = A.d;
  const long NU = (long)(d.nx + 1) * d.ny * d.nz, NV = (long)d.nx * (d.ny + 1) * d.nz,
             NW = (long)d.nx * d.ny * (d.nz + 1);
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < NU + NV + NW; t += (long)gridDim.x * blockDim.x) {
    if (t < NU) {
      const long f = t;
      const double g = A.cu[f];
      if (g == 0.0) continue;
      const int i = (int)(f % (d.nx + 1));
      const long q = f / (d.nx + 1);
      const int j = (int)(q % d.ny), k = (int)(q / d.ny);
      const double uc = A.u[f];
      const double va = 0.25 * (ldv(A, i - 1, j, k, 0.0) + ldv(A, i - 1, j + 1, k, 0.0) + ldv(A, i, j, k, 0.0) +
                                ldv(A, i, j + 1, k, 0.0));
      const double wa = 0.25 * (ldw(A, i - 1, j, k, 0.0) + ldw(A, i - 1, j, k + 1, 0.0) + ldw(A, i, j, k, 0.0) +
                                ldw(A, i, j, k + 1, 0.0));
      const double ue = ldu(A, i + 1, j, k, uc), uw = ldu(A, i - 1, j, k, uc);
      const double un = ldu(A, i, j + 1, k, uc), us = ldu(A, i, j - 1, k, uc);
      const double ut = ldu(A, i, j, k + 1, uc), ub = ldu(A, i, j, k - 1, uc);
      const double gx = g * A.rtx, gy = g * A.rty, gz = g * A.rtz;
      atomicAdd(&A.lu[f], gx * (ue - uw));
      addu(A, i + 1, j, k, gx * uc, f); addu(A, i - 1, j, k, -gx * uc, f);
      addu(A, i, j + 1, k, gy * va, f); addu(A, i, j - 1, k, -gy * va, f);
      addu(A, i, j, k + 1, gz * wa, f); addu(A, i, j, k - 1, -gz * wa, f);
      const double cv = 0.25 * gy * (un - us), cw = 0.25 * gz * (ut - ub);
      addv(A, i - 1, j, k, cv, -1); addv(A, i - 1, j + 1, k, cv, -1);
      addv(A, i, j, k, cv, -1); addv(A, i, j + 1, k, cv, -1);
      addw(A, i - 1, j, k, cw, -1); addw(A, i - 1, j, k + 1, cw, -1);
      addw(A, i, j, k, cw, -1); addw(A, i, j, k + 1, cw, -1);
    } else if (t < NU + NV) {
      const long f = t - NU;
      const double g = A.cv[f];
      if (g == 0.0) continue;
      const int i = (int)(f % d.nx);
      const long q = f / d.nx;
      const int j = (int)(q % (d.ny + 1)), k = (int)(q / (d.ny + 1));
      const double vc = A.v[f];
      const double ua = 0.25 * (ldu(A, i, j - 1, k, 0.0) + ldu(A, i + 1, j - 1, k, 0.0) + ldu(A, i, j, k, 0.0) +
                                ldu(A, i + 1, j, k, 0.0));
      const double wa = 0.25 * (ldw(A, i, j - 1, k, 0.0) + ldw(A, i, j, k, 0.0) + ldw(A, i, j - 1, k + 1, 0.0) +
                                ldw(A, i, j, k + 1, 0.0));
      const double ve = ldv(A, i + 1, j, k, vc), vw = ldv(A, i - 1, j, k, vc);
      const double vn = ldv(A, i, j + 1, k, vc), vs = ldv(A, i, j - 1, k, vc);
      const double vt = ldv(A, i, j, k + 1, vc), vb = ldv(A, i, j, k - 1, vc);
      const double gx = g * A.rtx, gy = g * A.rty, gz = g * A.rtz;
      atomicAdd(&A.lv[f], gy * (vn - vs));
      addv(A, i + 1, j, k, gx * ua, f); addv(A, i - 1, j, k, -gx * ua, f);
      addv(A, i, j + 1, k, gy * vc, f); addv(A, i, j - 1, k, -gy * vc, f);
      addv(A, i, j, k + 1, gz * wa, f); addv(A, i, j, k - 1, -gz * wa, f);
      const double cu = 0.25 * gx * (ve - vw), cw = 0.25 * gz * (vt - vb);
      addu(A, i, j - 1, k, cu, -1); addu(A, i + 1, j - 1, k, cu, -1);
      addu(A, i, j, k, cu, -1); addu(A, i + 1, j, k, cu, -1);
      addw(A, i, j - 1, k, cw, -1); addw(A, i, j, k, cw, -1);
      addw(A, i, j - 1, k + 1, cw, -1); addw(A, i, j, k + 1, cw, -1);
    } else {
      const long f = t - NU - NV;
      const double g = A.cw[f];
      if (g == 0.0) continue;
      const long plane = (long)d.nx * d.ny;
      const int k = (int)(f / plane);
      const long rem = f - (long)k * plane;
      const int j = (int)(rem / d.nx), i = (int)(rem % d.nx);
      const double wc = A.w[f];
      const double ua = 0.25 * (ldu(A, i, j, k - 1, 0.0) + ldu(A, i + 1, j, k - 1, 0.0) + ldu(A, i, j, k, 0.0) +
                                ldu(A, i + 1, j, k, 0.0));
      const double va = 0.25 * (ldv(A, i, j, k - 1, 0.0) + ldv(A, i, j + 1, k - 1, 0.0) + ldv(A, i, j, k, 0.0) +
                                ldv(A, i, j + 1, k, 0.0));
      const double we = ldw(A, i + 1, j, k, wc), ww = ldw(A, i - 1, j, k, wc);
      const double wn = ldw(A, i, j + 1, k, wc), ws = ldw(A, i, j - 1, k, wc);
      const double wt = ldw(A, i, j, k + 1, wc), wb = ldw(A, i, j, k - 1, wc);
      const double gx = g * A.rtx, gy = g * A.rty, gz = g * A.rtz;
      atomicAdd(&A.lw[f], gz * (wt - wb));
      addw(A, i + 1, j, k, gx * ua, f); addw(A, i - 1, j, k, -gx * ua, f);
      addw(A, i, j + 1, k, gy * va, f); addw(A, i, j - 1, k, -gy * va, f);
      addw(A, i, j, k + 1, gz * wc, f); addw(A, i, j, k - 1, -gz * wc, f);
      const double cu = 0.25 * gx * (we - ww), cv = 0.25 * gy * (wn - ws);
      addu(A, i, j, k - 1, cu, -1); addu(A, i + 1, j, k - 1, cu, -1);
      addu(A, i, j, k, cu, -1); addu(A, i + 1, j, k, cu, -1);
      addv(A, i, j, k - 1, cv, -1); addv(A, i, j + 1, k - 1, cv, -1);
      addv(A, i, j, k, cv, -1); addv(A, i, j + 1, k, cv, -1);
    }
  }
}

__global__ void k_wscale(const double *x, const double *winv, double *y, long n, int divide) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    y[r] = divide ? x[r] / winv[r] : x[r] * winv[r];
}

// u at the inlet = g (the BC cleanup multiplies by the ramp); the inlet
// column's divergence lift 0 - g / (beta dx), the operations of the setup.
__global__ void k_set_inflow(const double *g, const double *bdx, double *uin, double *div_bc, int nx, int nyz) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nyz; t += gridDim.x * blockDim.x) {
    uin[t] = g[t];
    if (bdx[t] != 0.0) div_bc[(long)t * nx] = __dsub_rn(0.0, __ddiv_rn(g[t], bdx[t]));
  }
}

}  // namespace

void launch_transpose7(cudaStream_t st, const double *planes, const Box &b, double *rows) {
  LaunchScope ls(K_SETUP, st, 112.0 * b.n);
  k_transpose7<<<adj_grid(b.n), kThreads, 0, st>>>(planes, b, rows);
}

void adj_bc(ibm_ctx *c, double *lu, double *lv, double *lw, const double *ramp) {
  const ADims d = adims(c);
  const long m = std::max((long)c->zl_u.n, std::max((long)c->zl_v.n, (long)c->zl_w.n));
  if (m > 0) {
    LaunchScope ls(K_ADJOINT, c->st, 12.0 * (double)(c->zl_u.n + c->zl_v.n + c->zl_w.n));
    k_zero_lists<<<adj_grid(m), kThreads, 0, c->st>>>(lu, c->zl_u.p, (int)c->zl_u.n, lv, c->zl_v.p, (int)c->zl_v.n,
                                                      lw, c->zl_w.p, (int)c->zl_w.n);
  }
  const long n = std::max((long)d.ny * d.nz, std::max((long)d.nx * d.nz, (long)d.nx * d.ny));
  LaunchScope ls(K_ADJOINT, c->st, 40.0 * d.ny * d.nz + 16.0 * d.nx * d.nz + 16.0 * d.nx * d.ny);
  k_bc_planes_t<<<adj_grid(n), kThreads, 0, c->st>>>(lu, lv, lw, c->adj->dg.p, ramp, d);
}

void adj_force(ibm_ctx *c, const double *weight) {
  AdjState &a = *c->adj;
  if (c->prm.compute_forces == 2) {
    adj_force_cut(c, weight, a.lu.p, a.lp.p, a.acc.p);
    return;
  }
  LaunchScope ls(K_ADJOINT, c->st, 1.0 * c->g.NP + 24.0 * c->g.NU + 16.0 * c->g.NP);
  k_force_t<<<adj_grid(c->g.NP), kThreads, 0, c->st>>>(c->fc.p, c->u.p, a.lu.p, a.lp.p, a.acc.p, adims(c), c->g.dx,
                                                      c->g.dy, c->g.dz, c->g.rho, c->g.nu, weight);
}

void adj_projection(ibm_ctx *c, double *rphi) {
  AdjState &a = *c->adj;
  GradTArgs A;
  A.d = adims(c);
  A.fu = c->fu.p; A.fv = c->fv.p; A.fw = c->fw.p; A.fc = c->fc.p;
  A.Gu = c->Gu.p; A.Gv = c->Gv.p; A.Gw = c->Gw.p;
  A.lu = a.lu.p; A.lv = a.lv.p; A.lw = a.lw.p;
  A.base = a.lp.p;
  A.coef = -(c->g.dt / c->g.rho);
  A.out = rphi;
  A.mode = 0;
  const double faces = (double)(c->g.NU + c->g.NV + c->g.NW);
  LaunchScope ls(K_ADJOINT, c->st, 25.0 * faces + 17.0 * c->g.NP);
  k_grad_t<<<adj_grid(c->g.NP), kThreads, 0, c->st>>>(A);
}

void adj_divergence(ibm_ctx *c, const double *mu, const double *ramp) {
  AdjState &a = *c->adj;
  const double faces = (double)(c->g.NU + c->g.NV + c->g.NW);
  const double rdt = c->g.rho / c->g.dt;
  {
    LaunchScope ls(K_ADJOINT, c->st, 17.0 * faces + 57.0 * c->g.NP);
    k_div_t<<<adj_grid(c->g.NU + c->g.NV + c->g.NW), kThreads, 0, c->st>>>(
        adims(c), c->fu.p, c->fv.p, c->fw.p, c->fc.p, c->Dc.p, mu, -rdt, a.lu.p, a.lv.p, a.lw.p);
  }
  const int nyz = c->g.ny * c->g.nz;
  LaunchScope ls(K_ADJOINT, c->st, 32.0 * nyz);
  k_inlet_t<<<adj_grid(nyz), kThreads, 0, c->st>>>(a.dg.p, mu, a.winl.p, rdt, ramp, c->g.nx, nyz);
}

void adj_scatter(ibm_ctx *c, double *const *lx) {
  AdjState &a = *c->adj;
  const long n = c->g.bu.n + c->g.bv.n + c->g.bw.n;
  LaunchScope ls(K_ADJOINT, c->st, 24.0 * n);
  k_scatter_t<<<adj_grid(n), kThreads, 0, c->st>>>(adims(c), a.lu.p, a.lv.p, a.lw.p, lx[0], lx[1], lx[2]);
}

void adj_momentum(ibm_ctx *c, const double *const *lb) {
  AdjState &a = *c->adj;
  a.cu.zero(c->st); a.cv.zero(c->st); a.cw.zero(c->st);
  a.gu.zero(c->st); a.gv.zero(c->st); a.gw.zero(c->st);
  MomTArgs M;
  M.d = adims(c);
  M.fu = c->fu.p; M.fv = c->fv.p; M.fw = c->fw.p;
  for (int f = 0; f < 3; ++f) {
    M.sc[f] = c->scale_box[f].p; M.bc[f] = c->bc_box[f].p; M.b[f] = c->bb[f].p; M.x[f] = c->xb[f].p;
    M.lb[f] = lb[f];
  }
  M.nb[0] = c->g.bu.n; M.nb[1] = c->g.bv.n; M.nb[2] = c->g.bw.n;
  M.lu = a.lu.p; M.lv = a.lv.p; M.lw = a.lw.p;
  M.cu = a.cu.p; M.cv = a.cv.p; M.cw = a.cw.p;
  M.gu = a.gu.p; M.gv = a.gv.p; M.gw = a.gw.p;
  M.a = c->g.rho / c->g.dt; M.rho = c->g.rho; M.nu = c->g.nu;
  M.acc = a.acc.p;
  const long n = M.nb[0] + M.nb[1] + M.nb[2];
  {
    LaunchScope ls(K_ADJOINT, c->st, 65.0 * n);
    k_mom_t<<<adj_grid(n), kThreads, 0, c->st>>>(M);
  }
  ConvTArgs C;
  C.d = M.d;
  C.u = a.u1.p; C.v = a.v1.p; C.w = a.w1.p;
  C.cu = a.cu.p; C.cv = a.cv.p; C.cw = a.cw.p;
  C.lu = a.lu.p; C.lv = a.lv.p; C.lw = a.lw.p;
  C.rtx = 1.0 / (2 * c->g.dx); C.rty = 1.0 / (2 * c->g.dy); C.rtz = 1.0 / (2 * c->g.dz);
  const double faces = (double)(c->g.NU + c->g.NV + c->g.NW);
  LaunchScope ls(K_ADJOINT, c->st, 32.0 * faces);
  k_conv_t<<<adj_grid(c->g.NU + c->g.NV + c->g.NW), kThreads, 0, c->st>>>(C);
}

void adj_gradient(ibm_ctx *c) {
  AdjState &a = *c->adj;
  GradTArgs A;
  A.d = adims(c);
  A.fu = c->fu.p; A.fv = c->fv.p; A.fw = c->fw.p; A.fc = c->fc.p;
  A.Gu = c->Gu.p; A.Gv = c->Gv.p; A.Gw = c->Gw.p;
  A.lu = a.gu.p; A.lv = a.gv.p; A.lw = a.gw.p;
  A.base = nullptr;
  A.coef = 1.0;
  A.out = a.lp.p;
  A.mode = 1;
  const double faces = (double)(c->g.NU + c->g.NV + c->g.NW);
  LaunchScope ls(K_ADJOINT, c->st, 25.0 * faces + 17.0 * c->g.NP);
  k_grad_t<<<adj_grid(c->g.NP), kThreads, 0, c->st>>>(A);
}

void adj_wscale(ibm_ctx *c, const double *x, double *y, bool divide) {
  LaunchScope ls(K_ADJOINT, c->st, 24.0 * c->g.NP);
  k_wscale<<<adj_grid(c->g.NP), kThreads, 0, c->st>>>(x, c->p_winv.p, y, c->g.NP, divide ? 1 : 0);
}

void adj_set_inflow(ibm_ctx *c, const double *g) {
  AdjState &a = *c->adj;
  const int nyz = c->g.ny * c->g.nz;
  LaunchScope ls(K_SETUP, c->st, 32.0 * nyz);
  k_set_inflow<<<adj_grid(nyz), kThreads, 0, c->st>>>(g, a.bdx.p, c->uin.p, c->div_bc_cell.p, c->g.nx, nyz);
}

}  // namespace ibm

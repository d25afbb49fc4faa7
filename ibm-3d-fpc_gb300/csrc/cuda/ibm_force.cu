// Cut-surface force of the fluid on the body (compute_forces = 2), and its
// adjoint. The reference computes no force; this one is built on its own
// immersed-boundary discretisation so that it measures what the discrete
// equations exchange with the body:
//
//  - shear: where a velocity row of the momentum operators meets the body
//    (an inactive neighbour that is not a domain boundary), the reference
//    adds the wall flux nu u_P / d_P over the control-volume face, d_P being
//    the distance along the segment to the neighbour up to the cylinder
//    surface (immersed_operators.hpp:21-33, 67-87, 142-155 with
//    segmentCircleDistance, common.hpp:262-280); the body receives
//    rho nu u_P A / d_P along that velocity component;
//  - pressure: a fluid cell's part of the body surface is, by the divergence
//    theorem, n A = -sum over its faces of alpha_f A_f n_f (alpha the faces'
//    open fractions, a face to a non-fluid cell closed, so the fluid cells'
//    faces close around the body); the body receives p_c times that, so
//    F_x += p_c (alpha_w - alpha_e) dy dz and F_y += p_c (alpha_s - alpha_n)
//    dx dz (the cylinder spans the height: no z term).
//
// With every open fraction 0 or 1 the pressure part is the staircase force.
// The force is linear in (u, v, w, p), so ibm_set_body turns the geometry into
// a sparse list of (field, index, component, weight) and a step's force is a
// weighted sum over it (nu times the weight for velocity entries).
#include <cmath>
#include <vector>

#include "ibm_assembly.cuh"
#include "ibm_common.cuh"
#include "ibm_ctx.cuh"

namespace ibm {

namespace {

template <class T>
void upload_vec(DBuf<T> &dst, const std::vector<T> &h, cudaStream_t st) {
  dst.alloc(h.empty() ? 1 : h.size());
  if (!h.empty()) IBM_CUDA_TRY(cudaMemcpyAsync(dst.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
}

// entry code: field (0 u, 1 v, 2 w, 3 p) in bits 0-1, component in bits 2-3
__device__ __forceinline__ int cf_field(uint8_t c) { return c & 3; }
__device__ __forceinline__ int cf_comp(uint8_t c) { return (c >> 2) & 3; }

// Force = sum over the entries, nu times the velocity entries; block partials
// summed in block order by the last block (deterministic).
__global__ void __launch_bounds__(kThreads) k_forces_cut(const uint8_t *code, const int *idx, const double *w,
                                                         long n, const double *u, const double *v,
                                                         const double *wv, const double *p, double nu,
                                                         double *part, StepDiag *dg) {
  double f[3] = {0.0, 0.0, 0.0};
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const uint8_t c = code[e];
    const int fld = cf_field(c), q = cf_comp(c);
    const long i = idx[e];
    const double x = fld == 0 ? u[i] : fld == 1 ? v[i] : fld == 2 ? wv[i] : p[i];
    const double t = fld == 3 ? w[e] * x : nu * w[e] * x;
    if (q == 0) f[0] += t;
    else if (q == 1) f[1] += t;
    else f[2] += t;
  }
  __shared__ double s[3][kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int q = 0; q < 3; ++q) {
    const double t = warp_sum(f[q]);
    if (lane == 0) s[q][warp] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < 3; ++q) {
      double a = 0.0;
      for (int k = 0; k < kWarps; ++k) a += s[q][k];
      part[3 * blockIdx.x + q] = a;
    }
  }
  __threadfence();
  __syncthreads();
  __shared__ int last;
  if (threadIdx.x == 0) last = (atomicAdd(&dg->fticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    for (int q = 0; q < 3; ++q) {
      double a = 0.0;
      for (int b = 0; b < (int)gridDim.x; ++b) a += __ldcg(&part[3 * b + q]);
      dg->force[q] = a;
    }
    dg->fticket = 0;
  }
}

// Adjoint of the x force: lambda_p += weight w (pressure entries), lambda_u
// += weight nu w (u entries), acc += weight sum w u (dF_x/dnu). Every index
// appears once per (field, component), so the adds do not collide.
__global__ void k_force_cut_t(const uint8_t *code, const int *idx, const double *w, long n, const double *u,
                              double *lu, double *lp, double *acc, double nu, const double *weightp) {
  const double weight = *weightp;
  if (weight == 0.0) return;
  double dn = 0.0;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const uint8_t c = code[e];
    if (cf_comp(c) != 0) continue;
    const int fld = cf_field(c);
    const long i = idx[e];
    if (fld == 3) {
      lp[i] += weight * w[e];
    } else if (fld == 0) {
      lu[i] += weight * nu * w[e];
      dn += weight * w[e] * u[i];
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ double s[kWarps];
  const double t = warp_sum(dn);
  if (lane == 0) s[warp] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int k = 0; k < kWarps; ++k) a += s[k];
    if (a != 0.0) atomicAdd(acc, a);
  }
}

int force_blocks(long n) { return (int)std::max(1L, std::min((n + kThreads - 1) / kThreads, 256L)); }

}  // namespace

void launch_forces_cut(ibm_ctx *c) {
  if (!c->body_set) throw Error(IBM_ERR_STATE, "compute_forces 2: call ibm_set_body first");
  const long n = c->cf_n;
  LaunchScope ls(K_DIAG, c->st, 21.0 * (double)n);
  k_forces_cut<<<force_blocks(n), kThreads, 0, c->st>>>(c->cf_code.p, c->cf_idx.p, c->cf_w.p, n, c->u.p, c->v.p,
                                                        c->w.p, c->p.p, c->g.nu, c->part.p, c->diag.p);
}

void adj_force_cut(ibm_ctx *c, const double *weight, double *lu, double *lp, double *acc) {
  if (!c->body_set) throw Error(IBM_ERR_STATE, "compute_forces 2: call ibm_set_body first");
  const long n = c->cf_n;
  LaunchScope ls(K_ADJOINT, c->st, 29.0 * (double)n);
  k_force_cut_t<<<force_blocks(n), kThreads, 0, c->st>>>(c->cf_code.p, c->cf_idx.p, c->cf_w.p, n, c->u.p, lu, lp,
                                                         acc, c->g.nu, weight);
}

// Host: the sparse force entries of a cylinder (xcirc, ycirc, Rcirc) on the
// context's grid and masks, with the faces' open fractions.
void build_cut_force(ibm_ctx *c, double xcirc, double ycirc, double Rcirc, const std::vector<double> &alpha_u,
                     const std::vector<double> &alpha_v) {
  const Geometry &g = c->g;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const double dx = c->grid.Lx / nx, dy = c->grid.Ly / ny, dz = c->grid.Lz / nz, rho = c->grid.rho;
  asmb::Geo geo;
  geo.nx = nx; geo.ny = ny; geo.nz = nz;
  geo.Lx = c->grid.Lx; geo.Ly = c->grid.Ly; geo.Lz = c->grid.Lz;
  geo.rho = rho; geo.nu = c->grid.nu; geo.dt = c->grid.dt;
  geo.xcirc = xcirc; geo.ycirc = ycirc; geo.Rcirc = Rcirc;
  const std::vector<uint8_t> &au = c->h_act_u, &av = c->h_act_v, &aw = c->h_act_w, &fp = c->h_fluid;
  auto U = [&](int i, int j, int k) { return ((long)k * ny + j) * (nx + 1) + i; };
  auto V = [&](int i, int j, int k) { return ((long)k * (ny + 1) + j) * nx + i; };
  auto W = [&](int i, int j, int k) { return ((long)k * ny + j) * nx + i; };
  auto inv_d = [&](double xP, double yP, double xS, double yS) {
    const double d = asmb::ray_circle(xP, yP, xS, yS, geo);
    return std::isfinite(d) ? 1.0 / d : 0.0;
  };
  std::vector<uint8_t> code;
  std::vector<int> idx;
  std::vector<double> wt;
  auto put = [&](int field, int comp, long i, double w) {
    if (w == 0.0) return;
    code.push_back((uint8_t)(field | (comp << 2)));
    idx.push_back((int)i);
    wt.push_back(w);
  };
  const double ax = dy * dz, ay = dx * dz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i < nx; ++i) {  // u rows
        if (!au[U(i, j, k)]) continue;
        const double xP = i * dx, yP = (j + 0.5) * dy;
        double s = 0.0;
        if (!(i > 1 && au[U(i - 1, j, k)]) && i != 1) s += ax * inv_d(xP, yP, xP - dx, yP);
        if (!(i < nx - 1 && au[U(i + 1, j, k)]) && i != nx - 1) s += ax * inv_d(xP, yP, xP + dx, yP);
        if (!(j > 0 && au[U(i, j - 1, k)]) && j != 0) s += ay * inv_d(xP, yP, xP, yP - dy);
        if (!(j < ny - 1 && au[U(i, j + 1, k)]) && j != ny - 1) s += ay * inv_d(xP, yP, xP, yP + dy);
        put(0, 0, U(i, j, k), rho * s);
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {  // v rows
        if (!av[V(i, j, k)]) continue;
        const double xP = (i + 0.5) * dx, yP = j * dy;
        double s = 0.0;
        if (!(i > 0 && av[V(i - 1, j, k)]) && i != 0) s += ax * inv_d(xP, yP, xP - dx, yP);
        if (!(i < nx - 1 && av[V(i + 1, j, k)]) && i != nx - 1) s += ax * inv_d(xP, yP, xP + dx, yP);
        if (!(j > 1 && av[V(i, j - 1, k)]) && j != 1) s += ay * inv_d(xP, yP, xP, yP - dy);
        if (!(j < ny - 1 && av[V(i, j + 1, k)]) && j != ny - 1) s += ay * inv_d(xP, yP, xP, yP + dy);
        put(1, 1, V(i, j, k), rho * s);
      }
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {  // w rows
        if (!aw[W(i, j, k)]) continue;
        const double xP = (i + 0.5) * dx, yP = (j + 0.5) * dy;
        double s = 0.0;
        if (!(i > 0 && aw[W(i - 1, j, k)]) && i != 0) s += ax * inv_d(xP, yP, xP - dx, yP);
        if (!(i < nx - 1 && aw[W(i + 1, j, k)]) && i != nx - 1) s += ax * inv_d(xP, yP, xP + dx, yP);
        if (!(j > 0 && aw[W(i, j - 1, k)]) && j != 0) s += ay * inv_d(xP, yP, xP, yP - dy);
        if (!(j < ny - 1 && aw[W(i, j + 1, k)]) && j != ny - 1) s += ay * inv_d(xP, yP, xP, yP + dy);
        put(2, 2, W(i, j, k), rho * s);
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {  // pressure on fluid cells
        const long cc = W(i, j, k);
        if (!fp[cc]) continue;
        // a face to a non-fluid cell is closed (body surface), a domain face open
        const double aw_ = i > 0 ? (fp[W(i - 1, j, k)] ? alpha_u[U(i, j, k)] : 0.0) : 1.0;
        const double ae = i < nx - 1 ? (fp[W(i + 1, j, k)] ? alpha_u[U(i + 1, j, k)] : 0.0) : 1.0;
        const double as = j > 0 ? (fp[W(i, j - 1, k)] ? alpha_v[V(i, j, k)] : 0.0) : 1.0;
        const double an = j < ny - 1 ? (fp[W(i, j + 1, k)] ? alpha_v[V(i, j + 1, k)] : 0.0) : 1.0;
        put(3, 0, cc, (aw_ - ae) * ax);
        put(3, 1, cc, (as - an) * ay);
      }
  c->cf_n = (long)code.size();
  upload_vec(c->cf_code, code, c->st);
  upload_vec(c->cf_idx, idx, c->st);
  upload_vec(c->cf_w, wt, c->st);
  c->body_set = true;
}

}  // namespace ibm

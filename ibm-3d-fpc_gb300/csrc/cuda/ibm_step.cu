// Dense per-step kernels: boundary conditions, convection + pressure gradient
// + momentum right-hand side, solution scatter, divergence + pressure
// right-hand side, projection, and the per-step diagnostics.
//
// They restate gpu_dense_ops.hpp with the reference's active-id packing
// replaced by structured stencils: D and G become per-cell / per-face
// coefficients (converted from the reference CSR), so q, the packed pressure
// vector and the unpack kernels disappear. Every floating-point operation is
// written out (fma() where the reference's device code fuses a CSR
// accumulation, separately rounded operations elsewhere) so the CPU oracle
// reproduces the results bit for bit.
#include <cmath>

#include "ibm_ctx.cuh"
#include "ibm_df.cuh"
#include "ibm_step.cuh"

namespace ibm {

namespace {

// Division by a grid extent with a multiply-high (Granlund-Montgomery): flat
// face and cell indices stay below 2^32, and a 64-bit integer division would
// cost a long instruction sequence per use in kernels whose FP64 work is
// already the bound.
struct IDiv {
  unsigned d;
  FastDiv f;
};
inline IDiv make_idiv(int d) { return IDiv{(unsigned)d, make_fastdiv((unsigned)d)}; }
struct Dims {
  int nx, ny, nz;
  IDiv dnx, dnx1, dnxm, dny, dny1, dnym;  // nx, nx + 1, nx - 1, ny, ny + 1, ny - 1
};
// q = n / D, returns n - q D.
__device__ __forceinline__ int udivmod(long n, const IDiv &D, long &q) {
  const unsigned qq = fast_div((unsigned)n, D.f);
  q = (long)qq;
  return (int)((unsigned)n - qq * D.d);
}

__device__ __forceinline__ long U3(const Dims &d, int i, int j, int k) { return ((long)k * d.ny + j) * (d.nx + 1) + i; }
__device__ __forceinline__ long V3(const Dims &d, int i, int j, int k) { return ((long)k * (d.ny + 1) + j) * d.nx + i; }
__device__ __forceinline__ long W3(const Dims &d, int i, int j, int k) { return ((long)k * d.ny + j) * d.nx + i; }
__device__ __forceinline__ long P3(const Dims &d, int i, int j, int k) { return ((long)k * d.ny + j) * d.nx + i; }

// x / b correctly rounded for a divisor known in advance, without a division:
// rb = RN(1/b) is computed once on the host, q0 = RN(x rb) is within an ulp of
// x / b, and one correction with the exact remainder r = x - b q0 (a single
// FMA) gives RN(x / b) (Markstein, IBM J. Res. Dev. 34(1), 1990; the final
// step of the IA-64 division sequences). A zero remainder keeps q0, which
// also keeps the sign of a zero quotient; a non-finite q0 is returned as is.
// Equal to IEEE division whenever x / b and x rb are normal numbers. A
// division by the grid spacing this way costs 3 FP64 operations instead of
// the dozen or so of an IEEE division, and the convection kernel is bound by
// the FP64 pipe on GB300.
//
// A divisor that is a power of two, b = 2^p2 (the grid spacing when the
// domain length over the cell count is one, e.g. 2.5 / 640 = 2^-8), needs no
// correction: x / 2^p2 = x 2^-p2 exactly, so a normal result only moves the
// exponent (integer pipe), and the other cases (zero, subnormal, infinite,
// NaN) take one FP64 multiply by the exact 2^-p2.
constexpr int kNotPow2 = 1 << 20;
struct KnownDiv {
  double b, rb;
  int p2;  // b == 2^p2, else kNotPow2
};
inline KnownDiv make_known_div(double b) {
  KnownDiv k;
  k.b = b;
  k.rb = 1.0 / b;
  k.p2 = kNotPow2;
  int e = 0;
  if (std::frexp(b, &e) == 0.5 && e - 1 > -1000 && e - 1 < 1000) k.p2 = e - 1;
  return k;
}
__device__ __forceinline__ double div_known(double x, KnownDiv k) {
  if (k.p2 != kNotPow2) {
    const long long bits = __double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7FF), ne = e - k.p2;
    if (e != 0 && e != 0x7FF && ne > 0 && ne < 0x7FF) return __longlong_as_double(bits - (long long)k.p2 * (1LL << 52));
    return __dmul_rn(x, k.rb);
  }
  const double q0 = __dmul_rn(x, k.rb);
  const double r = fma(-q0, k.b, x);
  // r == 0 or r not finite, tested on the bits (integer pipe; FP64 compares
  // would take FP64 issue slots, the scarce resource of this kernel)
  const unsigned long long rb = (unsigned long long)__double_as_longlong(r);
  const bool keep = (rb << 1) == 0ull || (rb & 0x7FF0000000000000ull) == 0x7FF0000000000000ull;
  return keep ? q0 : fma(r, k.rb, q0);
}

// 0.25 x, exactly: for |x| >= 2^-1020 the product only lowers the exponent
// by two, done on the bits; zeros, subnormal-range and non-finite values take
// the FP64 multiply (same result either way).
__device__ __forceinline__ double quarter(double x) {
  const long long b = __double_as_longlong(x);
  const long long e = b & 0x7FF0000000000000LL;
  if (e > (2LL << 52) && e != 0x7FF0000000000000LL) return __longlong_as_double(b - (2LL << 52));
  return __dmul_rn(0.25, x);
}

// Centred advective term, separately rounded operations in the reference's order.
__device__ __forceinline__ double advect(double c, double dm, double dp, KnownDiv tdx, double a2, double em, double ep,
                                         KnownDiv tdy, double a3, double fm, double fp, KnownDiv tdz) {
  const double t1 = div_known(__dmul_rn(c, __dsub_rn(dp, dm)), tdx);
  const double t2 = div_known(__dmul_rn(a2, __dsub_rn(ep, em)), tdy);
  const double t3 = div_known(__dmul_rn(a3, __dsub_rn(fp, fm)), tdz);
  return __dadd_rn(__dadd_rn(t1, t2), t3);
}
__device__ __forceinline__ double avg4(double a, double b, double c, double d) {
  return quarter(__dadd_rn(__dadd_rn(__dadd_rn(a, b), c), d));
}
// ((rho/dt) u - rho conv - gp + bc) * scale (gpu_dense_ops.hpp:16-18). The
// reference leaves this expression to nvcc, which contracts its first
// difference into one fused multiply-add, fma(rho/dt, u, -(rho conv)); the
// rest is rounded operation by operation. Spelled out here so the result is
// bitwise the reference kernel's (checked against the reference's own kernel
// compiled from its sources).
__device__ __forceinline__ double mom_rhs(double a, double rho, double uc, double conv, double gp, double bc,
                                          double sc) {
  double t = fma(a, uc, -__dmul_rn(rho, conv));
  t = __dsub_rn(t, gp);
  t = __dadd_rn(t, bc);
  return __dmul_rn(t, sc);
}
// G applied to a cell field at one face: lower cell first (column order).
__device__ __forceinline__ double grad_face(double gl, double pl, double gr, double pr) {
  return fma(gr, pr, fma(gl, pl, 0.0));
}

// ------------------------------------------------------------------ BC
// Boundary planes (inlet ramp * uin, outlet copy, wall zeros).
__global__ void k_bc_planes(double *u, double *v, double *w, const double *uin, const double *ramp, Dims d) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long)d.ny * d.nz) {
    long kq;
    const int j = udivmod(t, d.dny, kq), k = (int)kq;
    u[U3(d, 0, j, k)] = __dmul_rn(*ramp, uin[t]);
    u[U3(d, d.nx, j, k)] = u[U3(d, d.nx - 1, j, k)];
  }
  if (t < (long)d.nx * d.nz) {
    long kq;
    const int i = udivmod(t, d.dnx, kq), k = (int)kq;
    v[V3(d, i, 0, k)] = 0.0;
    v[V3(d, i, d.ny, k)] = 0.0;
  }
  if (t < (long)d.nx * d.ny) {
    w[t] = 0.0;
    w[(long)d.nz * d.nx * d.ny + t] = 0.0;
  }
}

// Inactive interior faces (precomputed lists) set to zero.
__global__ void k_bc_zero(double *u, const int *lu, int nu_, double *v, const int *lv, int nv_, double *w,
                          const int *lw, int nw_) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nu_) u[lu[t]] = 0.0;
  if (t < nv_) v[lv[t]] = 0.0;
  if (t < nw_) w[lw[t]] = 0.0;
}

// ------------------------------------------------------------------ RHS
struct RhsArgs {
  Dims d;
  const double *u, *v, *w, *p;
  const uint8_t *fu, *fv, *fw, *fc;
  const double *Gu, *Gv, *Gw;
  const double *sc[3], *bc[3];
  double *b[3], *x0[3];
  long nb[3];
  double a, rho;
  KnownDiv tdx, tdy, tdz;  // 2 dx, 2 dy, 2 dz
  DF da, drho, drx, dry, drz;  // double-float a, rho, 1 / (2 dx), 1 / (2 dy), 1 / (2 dz)
  const float2 *u2, *v2, *w2, *p2;  // double-float copies of u, v, w, p (RhsDF; k_split_fields)
  int zero_guess;
};

// Arithmetic of the right-hand side. RhsF64: the reference's operations,
// each rounded in FP64 as above (bitwise the reference kernel). RhsDF: the
// same expressions in double-float on the FP32 and integer pipes (every
// input split from its FP64 bits, divisions by 2h as products with the
// double-float reciprocal), widened to FP64 once per row; about 2^-44 of
// the row's largest term, for the mixed-precision forms, where GB300's FP64
// rate bounds the FP64 kernel.
struct RhsF64 {
  using T = double;
  __device__ static T in(double x) { return x; }
  __device__ static T fld(const double *a, const float2 *, long i) { return a[i]; }
  __device__ static T zero() { return 0.0; }
  __device__ static T avg(T a, T b, T c, T d) { return avg4(a, b, c, d); }
  __device__ static T adv(const RhsArgs &A, T c, T dm, T dp, T a2, T em, T ep, T a3, T fm, T fp) {
    return advect(c, dm, dp, A.tdx, a2, em, ep, A.tdy, a3, fm, fp, A.tdz);
  }
  __device__ static T grad(T gl, T pl, T gr, T pr) { return grad_face(gl, pl, gr, pr); }
  __device__ static double rhs(const RhsArgs &A, T uc, T conv, T gp, double bc, double sc) {
    return mom_rhs(A.a, A.rho, uc, conv, gp, bc, sc);
  }
};
struct RhsDF {
  using T = DF;
  __device__ static T in(double x) { return df_of(x); }
  // a field value from the field's double-float copy (split once per step)
  __device__ static T fld(const double *, const float2 *a2, long i) {
    const float2 v = a2[i];
    return DF{v.x, v.y};
  }
  __device__ static T zero() { return DF{0.0f, 0.0f}; }
  __device__ static T avg(T a, T b, T c, T d) { return df_scale(df_add(df_add(df_add(a, b), c), d), 0.25f); }
  __device__ static T adv(const RhsArgs &A, T c, T dm, T dp, T a2, T em, T ep, T a3, T fm, T fp) {
    const T t1 = df_mul(df_mul(c, df_sub(dp, dm)), A.drx);
    const T t2 = df_mul(df_mul(a2, df_sub(ep, em)), A.dry);
    const T t3 = df_mul(df_mul(a3, df_sub(fp, fm)), A.drz);
    return df_add(df_add(t1, t2), t3);
  }
  __device__ static T grad(T gl, T pl, T gr, T pr) { return df_add(df_mul(gl, pl), df_mul(gr, pr)); }
  __device__ static double rhs(const RhsArgs &A, T uc, T conv, T gp, double bc, double sc) {
    T t = df_sub(df_mul(A.da, uc), df_mul(A.drho, conv));
    t = df_add(df_sub(t, gp), df_of(bc));
    return df_to_double(df_mul(t, df_of(sc)));
  }
};

// One thread per solve-box row of u, v and w (flat index over the three boxes).
// The loads are those of the reference's bounds-guarded loads
// (gpu_dense_ops.hpp:1-3) with the guards that a solve-box row can never fail
// dropped: on a u row (1 <= i <= nx-1) the x neighbours of u and the four v
// and w points of the averages always lie inside their arrays, only the y
// and z neighbours of u can fall back to the centre value; likewise for v
// (x and z neighbours guarded) and w (x and y neighbours guarded).
template <class M>
__global__ void __launch_bounds__(kThreads, 4) k_momentum_rhs(RhsArgs A) {
  using T = typename M::T;
  const Dims &d = A.d;
  const long total = A.nb[0] + A.nb[1] + A.nb[2];
  const long NU = (long)(d.nx + 1) * d.ny * d.nz, NV = (long)d.nx * (d.ny + 1) * d.nz,
             NW = (long)d.nx * d.ny * (d.nz + 1);
  const long su = d.nx + 1, pu = (long)(d.nx + 1) * d.ny;  // u strides along y and z
  const long sv = d.nx, pv = (long)d.nx * (d.ny + 1);     // v
  const long sw = d.nx, pw = (long)d.nx * d.ny;           // w and cells
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    if (t < A.nb[0]) {  // u row: face (i+1, j, k) with i in [0, nx-2]
      const long r = t;
      long q;
      const int i = udivmod(r, d.dnxm, q) + 1;
      long kq;
      const int j = udivmod(q, d.dny, kq), k = (int)kq;
      const long f = U3(d, i, j, k);
      const uint8_t fl = A.fu[f];
      double rhs = 0.0;
      if (fl & kRhsRow) {
        const T uc = M::fld(A.u, A.u2, f);
        T conv = M::zero();
        if (fl & kActive) {
          const long vb = V3(d, i - 1, j, k), wb = W3(d, i - 1, j, k);
          const T va = M::avg(M::fld(A.v, A.v2, vb), M::fld(A.v, A.v2, vb + sv),
                              M::fld(A.v, A.v2, vb + 1), M::fld(A.v, A.v2, vb + 1 + sv));
          const T wa = M::avg(M::fld(A.w, A.w2, wb), M::fld(A.w, A.w2, wb + pw),
                              M::fld(A.w, A.w2, wb + 1), M::fld(A.w, A.w2, wb + 1 + pw));
          conv = M::adv(A, uc, M::fld(A.u, A.u2, f - 1), M::fld(A.u, A.u2, f + 1), va,
                        (j > 0 ? M::fld(A.u, A.u2, f - su) : uc), (j < d.ny - 1 ? M::fld(A.u, A.u2, f + su) : uc), wa,
                        (k > 0 ? M::fld(A.u, A.u2, f - pu) : uc), (k < d.nz - 1 ? M::fld(A.u, A.u2, f + pu) : uc));
        }
        T gp = M::zero();
        if (fl & kQFace) {
          const long c = P3(d, i - 1, j, k);
          const T pl = (A.fc[c] & kFluid) ? M::fld(A.p, A.p2, c) : M::zero();
          const T pr = (A.fc[c + 1] & kFluid) ? M::fld(A.p, A.p2, c + 1) : M::zero();
          gp = M::grad(M::in(A.Gu[f]), pl, M::in(A.Gu[NU + f]), pr);
        }
        rhs = M::rhs(A, uc, conv, gp, A.bc[0][r], A.sc[0][r]);
      }
      A.b[0][r] = rhs;
      A.x0[0][r] = A.zero_guess ? 0.0 : A.u[f];
    } else if (t < A.nb[0] + A.nb[1]) {  // v row: face (i, j+1, k)
      const long r = t - A.nb[0];
      long q;
      const int i = udivmod(r, d.dnx, q);
      long kq;
      const int j = udivmod(q, d.dnym, kq) + 1, k = (int)kq;
      const long f = V3(d, i, j, k);
      const uint8_t fl = A.fv[f];
      double rhs = 0.0;
      if (fl & kRhsRow) {
        const T vc = M::fld(A.v, A.v2, f);
        T conv = M::zero();
        if (fl & kActive) {
          const long ub = U3(d, i, j - 1, k), wb = W3(d, i, j - 1, k);
          const T ua = M::avg(M::fld(A.u, A.u2, ub), M::fld(A.u, A.u2, ub + 1),
                              M::fld(A.u, A.u2, ub + su), M::fld(A.u, A.u2, ub + su + 1));
          const T wa = M::avg(M::fld(A.w, A.w2, wb), M::fld(A.w, A.w2, wb + sw),
                              M::fld(A.w, A.w2, wb + pw), M::fld(A.w, A.w2, wb + pw + sw));
          conv = M::adv(A, ua, (i > 0 ? M::fld(A.v, A.v2, f - 1) : vc),
                        (i < d.nx - 1 ? M::fld(A.v, A.v2, f + 1) : vc), vc,
                        M::fld(A.v, A.v2, f - sv), M::fld(A.v, A.v2, f + sv), wa,
                        (k > 0 ? M::fld(A.v, A.v2, f - pv) : vc), (k < d.nz - 1 ? M::fld(A.v, A.v2, f + pv) : vc));
        }
        T gp = M::zero();
        if (fl & kQFace) {
          const long c = P3(d, i, j - 1, k);
          const T pl = (A.fc[c] & kFluid) ? M::fld(A.p, A.p2, c) : M::zero();
          const T pr = (A.fc[c + sw] & kFluid) ? M::fld(A.p, A.p2, c + sw) : M::zero();
          gp = M::grad(M::in(A.Gv[f]), pl, M::in(A.Gv[NV + f]), pr);
        }
        rhs = M::rhs(A, vc, conv, gp, A.bc[1][r], A.sc[1][r]);
      }
      A.b[1][r] = rhs;
      A.x0[1][r] = A.zero_guess ? 0.0 : A.v[f];
    } else {  // w row: face (i, j, k+1)
      const long r = t - A.nb[0] - A.nb[1];
      long q;
      const int i = udivmod(r, d.dnx, q);
      long kq;
      const int j = udivmod(q, d.dny, kq), k = (int)kq + 1;
      const long f = W3(d, i, j, k);
      const uint8_t fl = A.fw[f];
      double rhs = 0.0;
      if (fl & kRhsRow) {
        const T wc = M::fld(A.w, A.w2, f);
        T conv = M::zero();
        // the convection of w uses the mask one plane below (gpu_dense_ops.hpp:14)
        if (A.fw[f - pw] & kActive) {
          const long ub = U3(d, i, j, k - 1), vb = V3(d, i, j, k - 1);
          const T ua = M::avg(M::fld(A.u, A.u2, ub), M::fld(A.u, A.u2, ub + 1),
                              M::fld(A.u, A.u2, ub + pu), M::fld(A.u, A.u2, ub + pu + 1));
          const T va = M::avg(M::fld(A.v, A.v2, vb), M::fld(A.v, A.v2, vb + sv),
                              M::fld(A.v, A.v2, vb + pv), M::fld(A.v, A.v2, vb + pv + sv));
          conv = M::adv(A, ua, (i > 0 ? M::fld(A.w, A.w2, f - 1) : wc),
                        (i < d.nx - 1 ? M::fld(A.w, A.w2, f + 1) : wc), va,
                        (j > 0 ? M::fld(A.w, A.w2, f - sw) : wc), (j < d.ny - 1 ? M::fld(A.w, A.w2, f + sw) : wc), wc,
                        M::fld(A.w, A.w2, f - pw), M::fld(A.w, A.w2, f + pw));
        }
        T gp = M::zero();
        if (fl & kQFace) {
          const long c = P3(d, i, j, k - 1);
          const T pl = (A.fc[c] & kFluid) ? M::fld(A.p, A.p2, c) : M::zero();
          const T pr = (A.fc[c + pw] & kFluid) ? M::fld(A.p, A.p2, c + pw) : M::zero();
          gp = M::grad(M::in(A.Gw[f]), pl, M::in(A.Gw[NW + f]), pr);
        }
        rhs = M::rhs(A, wc, conv, gp, A.bc[2][r], A.sc[2][r]);
      }
      A.b[2][r] = rhs;
      A.x0[2][r] = A.zero_guess ? 0.0 : A.w[f];
    }
  }
}

// Double-float copies of u, v, w and p for RhsDF: each value is split once
// per step instead of at each of its (about seven) uses by the right-hand
// side. Block row y takes field y.
struct SplitArgs {
  const double *src[4];
  float2 *dst[4];
  long n[4];
};
__global__ void __launch_bounds__(kThreads) k_split_fields(SplitArgs A) {
  const int a = blockIdx.y;
  const double *src = a == 0 ? A.src[0] : a == 1 ? A.src[1] : a == 2 ? A.src[2] : A.src[3];
  float2 *dst = a == 0 ? A.dst[0] : a == 1 ? A.dst[1] : a == 2 ? A.dst[2] : A.dst[3];
  const long n = a == 0 ? A.n[0] : a == 1 ? A.n[1] : a == 2 ? A.n[2] : A.n[3];
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float h, l;
    df_split_fast(src[i], h, l);
    dst[i] = make_float2(h, l);
  }
}

// ------------------------------------------------------------------ tilde
// ut = u, interior faces <- solve-box x (gpu_dense_ops.hpp:20-22); flags non-finite x.
__global__ void k_scatter(const double *u, const double *v, const double *w, const double *xu, const double *xv,
                          const double *xw, double *ut, double *vt, double *wt, Dims d, StepDiag *dg) {
  const long NU = (long)(d.nx + 1) * d.ny * d.nz, NV = (long)d.nx * (d.ny + 1) * d.nz,
             NW = (long)d.nx * d.ny * (d.nz + 1);
  int bad = 0;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < NU + NV + NW; t += (long)gridDim.x * blockDim.x) {
    if (t < NU) {
      const long f = t;
      long q;
      const int i = udivmod(f, d.dnx1, q);
      double val = u[f];
      if (i >= 1 && i <= d.nx - 1) { val = xu[q * (d.nx - 1) + (i - 1)]; bad |= !isfinite(val); }
      ut[f] = val;
    } else if (t < NU + NV) {
      const long f = t - NU;
      long q;
      const int i = udivmod(f, d.dnx, q);
      long kq;
      const int j = udivmod(q, d.dny1, kq), k = (int)kq;
      double val = v[f];
      if (j >= 1 && j <= d.ny - 1) { val = xv[((long)k * (d.ny - 1) + (j - 1)) * d.nx + i]; bad |= !isfinite(val); }
      vt[f] = val;
    } else {
      const long f = t - NU - NV;
      const long plane = (long)d.nx * d.ny;
      const int k = (int)(f / plane);
      double val = w[f];
      if (k >= 1 && k <= d.nz - 1) { val = xw[f - plane]; bad |= !isfinite(val); }
      wt[f] = val;
    }
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&dg->nonfinite_mom, 1);
}

// ------------------------------------------------------------------ pressure RHS
struct DivArgs {
  Dims d;
  const double *ut, *vt, *wt;
  const uint8_t *fu, *fv, *fw, *fc;
  const double *Dc;
  const double *div_bc;
  double *b, *x0;
  double neg_a;
  const double *ramp;
};

// D applied to the q-faces of a cell, as the reference's CSR row: fused
// multiply-add chain in column order u_w, u_e, v_s, v_n, w_b, w_t.
__device__ __forceinline__ double div_cell(const double *Dc, long NPc, long c, double qw, double qe, double qs,
                                           double qn, double qb, double qt) {
  double s = 0.0;
  s = fma(Dc[c], qw, s);
  s = fma(Dc[NPc + c], qe, s);
  s = fma(Dc[2 * NPc + c], qs, s);
  s = fma(Dc[3 * NPc + c], qn, s);
  s = fma(Dc[4 * NPc + c], qb, s);
  s = fma(Dc[5 * NPc + c], qt, s);
  return s;
}

__global__ void __launch_bounds__(kThreads) k_pressure_rhs(DivArgs A) {
  const Dims &d = A.d;
  const long NP = (long)d.nx * d.ny * d.nz;
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < NP; c += (long)gridDim.x * blockDim.x) {
    double rhs = 0.0;
    if (A.fc[c] & kFluid) {
      long q;
      const int i = udivmod(c, d.dnx, q);
      long kq;
      const int j = udivmod(q, d.dny, kq), k = (int)kq;
      const long fw_ = U3(d, i, j, k), fe = U3(d, i + 1, j, k);
      const long fs = V3(d, i, j, k), fn = V3(d, i, j + 1, k);
      const long fb = W3(d, i, j, k), ft = W3(d, i, j, k + 1);
      const double s = div_cell(A.Dc, NP, c, (A.fu[fw_] & kQFace) ? A.ut[fw_] : 0.0,
                                (A.fu[fe] & kQFace) ? A.ut[fe] : 0.0, (A.fv[fs] & kQFace) ? A.vt[fs] : 0.0,
                                (A.fv[fn] & kQFace) ? A.vt[fn] : 0.0, (A.fw[fb] & kQFace) ? A.wt[fb] : 0.0,
                                (A.fw[ft] & kQFace) ? A.wt[ft] : 0.0);
      rhs = __dmul_rn(A.neg_a, fma(*A.ramp, A.div_bc[c], s));
    }
    A.b[c] = rhs;
    A.x0[c] = 0.0;
  }
}

// ------------------------------------------------------------------ projection
struct ProjArgs {
  Dims d;
  const double *ut, *vt, *wt, *phi;
  double *u, *v, *w, *p;
  const uint8_t *fu, *fv, *fw, *fc;
  const double *Gu, *Gv, *Gw;
  double factor;
  StepDiag *dg;
};

__device__ __forceinline__ double phi_at(const ProjArgs &A, long c) { return (A.fc[c] & kFluid) ? A.phi[c] : 0.0; }

// q = q~ - (dt/rho) G phi on q-faces, other faces keep q~; p += phi on fluid cells.
__global__ void __launch_bounds__(kThreads, 4) k_project(ProjArgs A) {
  const Dims &d = A.d;
  const long NU = (long)(d.nx + 1) * d.ny * d.nz, NV = (long)d.nx * (d.ny + 1) * d.nz,
             NW = (long)d.nx * d.ny * (d.nz + 1), NP = (long)d.nx * d.ny * d.nz;
  const double nf = -A.factor;
  int bad = 0;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < NU + NV + NW + NP; t += (long)gridDim.x * blockDim.x) {
    if (t < NU) {
      const long f = t;
      double val = A.ut[f];
      if (A.fu[f] & kQFace) {
        long q;
        const int i = udivmod(f, d.dnx1, q);
        long kq;
      const int j = udivmod(q, d.dny, kq), k = (int)kq;
        const double pl = i > 0 ? phi_at(A, P3(d, i - 1, j, k)) : 0.0;
        const double pr = i < d.nx ? phi_at(A, P3(d, i, j, k)) : 0.0;
        val = fma(nf, grad_face(A.Gu[f], pl, A.Gu[NU + f], pr), val);
      }
      A.u[f] = val;
    } else if (t < NU + NV) {
      const long f = t - NU;
      double val = A.vt[f];
      if (A.fv[f] & kQFace) {
        long q;
        const int i = udivmod(f, d.dnx, q);
        long kq;
      const int j = udivmod(q, d.dny1, kq), k = (int)kq;
        const double pl = j > 0 ? phi_at(A, P3(d, i, j - 1, k)) : 0.0;
        const double pr = j < d.ny ? phi_at(A, P3(d, i, j, k)) : 0.0;
        val = fma(nf, grad_face(A.Gv[f], pl, A.Gv[NV + f], pr), val);
      }
      A.v[f] = val;
    } else if (t < NU + NV + NW) {
      const long f = t - NU - NV;
      double val = A.wt[f];
      if (A.fw[f] & kQFace) {
        const long plane = (long)d.nx * d.ny;
        const int k = (int)(f / plane);
        const long c = f - (long)k * plane;
        const double pl = k > 0 ? phi_at(A, c + (long)(k - 1) * plane) : 0.0;
        const double pr = k < d.nz ? phi_at(A, c + (long)k * plane) : 0.0;
        val = fma(nf, grad_face(A.Gw[f], pl, A.Gw[NW + f], pr), val);
      }
      A.w[f] = val;
    } else {
      const long c = t - NU - NV - NW;
      bad |= !isfinite(A.phi[c]);
      if (A.fc[c] & kFluid) A.p[c] = __dadd_rn(A.p[c], A.phi[c]);
    }
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&A.dg->nonfinite_p, 1);
}

// ------------------------------------------------------------------ diagnostics
struct DiagArgs {
  Dims d;
  const double *ut, *vt, *wt, *phi;
  const double *u, *v, *w;
  const uint8_t *fu, *fv, *fw, *fc;
  const double *Gu, *Gv, *Gw, *Dc, *div_bc;
  double factor;
  const double *ramp;
  double *part;
  StepDiag *dg;
  int np_active;
};

// Corrected q value of a face: the projected field holds it (k_project
// writes exactly this value), except on the faces the BC cleanup rewrote
// afterwards, where it is recomputed the same way.
__device__ __forceinline__ double q_face(const DiagArgs &A, const double *qt, const double *qn, const uint8_t *fl,
                                         const double *G, long NF, long f, double pl, double pr) {
  const uint8_t m = fl[f];
  if (!(m & kQFace)) return 0.0;
  if (!(m & kBcSet)) return qn[f];
  return fma(-A.factor, grad_face(G[f], pl, G[NF + f], pr), qt[f]);
}

// |x| as an ordered integer key: for non-NaN doubles the bit pattern without
// its sign orders like the magnitude, so the maxima run on the integer pipe
// (the FP64 pipe is the scarce one). NaN counts as 0, as fmax would ignore it.
__device__ __forceinline__ unsigned long long mag_key(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
  return b > 0x7FF0000000000000ull ? 0ull : b;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// The six corrected values of a cell next to a face the BC rewrote (rare:
// kept out of line so the common path keeps few registers).
__device__ __noinline__ void boundary_q(const DiagArgs &A, long c, int i, int j, int k, double &qw, double &qe,
                                        double &qs, double &qn, double &qb, double &qt) {
  const Dims &d = A.d;
  const long NU = (long)(d.nx + 1) * d.ny * d.nz, NV = (long)d.nx * (d.ny + 1) * d.nz,
             NW = (long)d.nx * d.ny * (d.nz + 1);
  const long plane = (long)d.nx * d.ny;
  auto ph = [&](long cc) { return (A.fc[cc] & kFluid) ? A.phi[cc] : 0.0; };
  const double pc = ph(c);
  const double pxm = i > 0 ? ph(c - 1) : 0.0, pxp = i < d.nx - 1 ? ph(c + 1) : 0.0;
  const double pym = j > 0 ? ph(c - d.nx) : 0.0, pyp = j < d.ny - 1 ? ph(c + d.nx) : 0.0;
  const double pzm = k > 0 ? ph(c - plane) : 0.0, pzp = k < d.nz - 1 ? ph(c + plane) : 0.0;
  qw = q_face(A, A.ut, A.u, A.fu, A.Gu, NU, U3(d, i, j, k), pxm, pc);
  qe = q_face(A, A.ut, A.u, A.fu, A.Gu, NU, U3(d, i + 1, j, k), pc, pxp);
  qs = q_face(A, A.vt, A.v, A.fv, A.Gv, NV, V3(d, i, j, k), pym, pc);
  qn = q_face(A, A.vt, A.v, A.fv, A.Gv, NV, V3(d, i, j + 1, k), pc, pyp);
  qb = q_face(A, A.wt, A.w, A.fw, A.Gw, NW, W3(d, i, j, k), pzm, pc);
  qt = q_face(A, A.wt, A.w, A.fw, A.Gw, NW, W3(d, i, j, k + 1), pc, pzp);
}

__global__ void __launch_bounds__(kThreads, 4) k_diagnostics(DiagArgs A) {
  const Dims &d = A.d;
  const long NU = (long)(d.nx + 1) * d.ny * d.nz, NV = (long)d.nx * (d.ny + 1) * d.nz,
             NW = (long)d.nx * d.ny * (d.nz + 1), NP = (long)d.nx * d.ny * d.nz;
  double div2 = 0.0;
  unsigned long long um = 0, vm = 0, wm = 0;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < NP + NU + NV + NW; t += (long)gridDim.x * blockDim.x) {
    if (t < NP) {
      const long c = t;
      if (!(A.fc[c] & kFluid)) continue;
      long q;
      const int i = udivmod(c, d.dnx, q);
      long kq;
      const int j = udivmod(q, d.dny, kq), k = (int)kq;
      const long fw_ = U3(d, i, j, k), fe = U3(d, i + 1, j, k), fs = V3(d, i, j, k), fn = V3(d, i, j + 1, k),
                 fb = W3(d, i, j, k), ft = W3(d, i, j, k + 1);
      double qw, qe, qs, qn, qb, qt;
      if (!((A.fu[fw_] | A.fu[fe] | A.fv[fs] | A.fv[fn] | A.fw[fb] | A.fw[ft]) & kBcSet)) {
        // interior cell: the six corrected values are the projected field
        qw = (A.fu[fw_] & kQFace) ? A.u[fw_] : 0.0;
        qe = (A.fu[fe] & kQFace) ? A.u[fe] : 0.0;
        qs = (A.fv[fs] & kQFace) ? A.v[fs] : 0.0;
        qn = (A.fv[fn] & kQFace) ? A.v[fn] : 0.0;
        qb = (A.fw[fb] & kQFace) ? A.w[fb] : 0.0;
        qt = (A.fw[ft] & kQFace) ? A.w[ft] : 0.0;
      } else {
        boundary_q(A, c, i, j, k, qw, qe, qs, qn, qb, qt);
      }
      const double s = div_cell(A.Dc, NP, c, qw, qe, qs, qn, qb, qt);
      const double dv = __dadd_rn(s, __dmul_rn(*A.ramp, A.div_bc[c]));
      div2 = __dadd_rn(div2, __dmul_rn(dv, dv));
    } else if (t < NP + NU) {
      const unsigned long long m = mag_key(A.u[t - NP]);
      um = m > um ? m : um;
    } else if (t < NP + NU + NV) {
      const unsigned long long m = mag_key(A.v[t - NP - NU]);
      vm = m > vm ? m : vm;
    } else {
      const unsigned long long m = mag_key(A.w[t - NP - NU - NV]);
      wm = m > wm ? m : wm;
    }
  }
  __shared__ double s_div[kWarps];
  __shared__ unsigned long long s_max[3][kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  div2 = warp_sum(div2);
  um = warp_max_u64(um); vm = warp_max_u64(vm); wm = warp_max_u64(wm);
  if (lane == 0) { s_div[warp] = div2; s_max[0][warp] = um; s_max[1][warp] = vm; s_max[2][warp] = wm; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    unsigned long long b = 0, c = 0, e = 0;
    for (int q = 0; q < kWarps; ++q) {
      a += s_div[q];
      b = s_max[0][q] > b ? s_max[0][q] : b;
      c = s_max[1][q] > c ? s_max[1][q] : c;
      e = s_max[2][q] > e ? s_max[2][q] : e;
    }
    A.part[4 * blockIdx.x + 0] = a;
    A.part[4 * blockIdx.x + 1] = __longlong_as_double((long long)b);
    A.part[4 * blockIdx.x + 2] = __longlong_as_double((long long)c);
    A.part[4 * blockIdx.x + 3] = __longlong_as_double((long long)e);
  }
  __threadfence();
  __syncthreads();
  __shared__ int last;
  if (threadIdx.x == 0) last = (atomicAdd(&A.dg->ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0, c = 0.0, e = 0.0;
    for (int q = 0; q < (int)gridDim.x; ++q) {
      a += A.part[4 * q]; b = fmax(b, A.part[4 * q + 1]); c = fmax(c, A.part[4 * q + 2]); e = fmax(e, A.part[4 * q + 3]);
    }
    A.dg->div2 = a; A.dg->umax = b; A.dg->vmax = c; A.dg->wmax = e;
    A.dg->ticket = 0;
  }
}

Dims dims_of(const ibm_ctx *c) {
  Dims d;
  d.nx = c->g.nx; d.ny = c->g.ny; d.nz = c->g.nz;
  d.dnx = make_idiv(d.nx); d.dnx1 = make_idiv(d.nx + 1); d.dnxm = make_idiv(std::max(1, d.nx - 1));
  d.dny = make_idiv(d.ny); d.dny1 = make_idiv(d.ny + 1); d.dnym = make_idiv(std::max(1, d.ny - 1));
  return d;
}

int blocks_for(long n) {
  long b = (n + kThreads - 1) / kThreads;
  const long cap = (long)sm_count() * 8;
  return (int)std::max(1L, std::min(b, cap));
}

// The same, capped at the blocks that stay resident (one wave of the
// grid-stride loop).
template <class K>
int wave_blocks(K kernel, long n) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
  const long b = (n + kThreads - 1) / kThreads;
  return (int)std::max(1L, std::min(b, (long)std::max(1, per_sm) * sm_count()));
}

}  // namespace

// Algorithmic bytes of each launch count every array element the kernel must
// touch once (stencil neighbours are reuse, not extra traffic).
void launch_bc(ibm_ctx *c, double *u, double *v, double *w) {
  const Dims d = dims_of(c);
  const long n = std::max((long)d.ny * d.nz, std::max((long)d.nx * d.nz, (long)d.nx * d.ny));
  {
    LaunchScope ls(K_BC, c->st, 32.0 * d.ny * d.nz + 16.0 * d.nx * d.nz + 16.0 * d.nx * d.ny);
    k_bc_planes<<<(int)((n + kThreads - 1) / kThreads), kThreads, 0, c->st>>>(u, v, w, c->uin.p, c->dramp.p, d);
  }
  const long m = std::max((long)c->zl_u.n, std::max((long)c->zl_v.n, (long)c->zl_w.n));
  if (m > 0) {
    LaunchScope ls(K_BC, c->st, 12.0 * (double)(c->zl_u.n + c->zl_v.n + c->zl_w.n));
    k_bc_zero<<<(int)((m + kThreads - 1) / kThreads), kThreads, 0, c->st>>>(u, c->zl_u.p, (int)c->zl_u.n, v, c->zl_v.p,
                                                                            (int)c->zl_v.n, w, c->zl_w.p, (int)c->zl_w.n);
  }
}

bool momentum_rhs_df(const ibm_solver_params &p) {
  const int vp = p.vel_precision >= 0 ? p.vel_precision : p.precision;
  return p.df_rhs != 0 && vp >= 1;
}

void ensure_rhs_df(ibm_ctx *c) {
  if (!momentum_rhs_df(c->prm) || c->df_u.p) return;
  c->df_u.alloc(c->g.NU); c->df_v.alloc(c->g.NV); c->df_w.alloc(c->g.NW); c->df_p.alloc(c->g.NP);
}

void launch_momentum_rhs(ibm_ctx *c) {
  RhsArgs A;
  A.d = dims_of(c);
  A.u = c->u.p; A.v = c->v.p; A.w = c->w.p; A.p = c->p.p;
  A.fu = c->fu.p; A.fv = c->fv.p; A.fw = c->fw.p; A.fc = c->fc.p;
  A.Gu = c->Gu.p; A.Gv = c->Gv.p; A.Gw = c->Gw.p;
  for (int f = 0; f < 3; ++f) {
    A.sc[f] = c->scale_box[f].p; A.bc[f] = c->bc_box[f].p;
    A.b[f] = c->bb[f].p; A.x0[f] = c->xb[f].p;
  }
  A.nb[0] = c->g.bu.n; A.nb[1] = c->g.bv.n; A.nb[2] = c->g.bw.n;
  A.a = c->g.rho / c->g.dt;
  A.rho = c->g.rho;
  A.tdx = make_known_div(2 * c->g.dx);
  A.tdy = make_known_div(2 * c->g.dy);
  A.tdz = make_known_div(2 * c->g.dz);
  A.zero_guess = c->prm.use_zero_initial_guess != 0;
  // host split of a constant: RN to FP32 and the rounded remainder (2^-48)
  auto split = [](double x) {
    const float h = (float)x;
    return DF{h, (float)(x - (double)h)};
  };
  A.da = split(A.a); A.drho = split(A.rho);
  A.drx = split(1.0 / (2 * c->g.dx)); A.dry = split(1.0 / (2 * c->g.dy)); A.drz = split(1.0 / (2 * c->g.dz));
  const double faces = (double)(c->g.NU + c->g.NV + c->g.NW), nbox = (double)(A.nb[0] + A.nb[1] + A.nb[2]);
  const long rows = A.nb[0] + A.nb[1] + A.nb[2];
  if (momentum_rhs_df(c->prm)) {
    if (!c->df_u.p || !c->df_v.p || !c->df_w.p || !c->df_p.p)
      throw Error(IBM_ERR_STATE, "double-float field copies not allocated");
    SplitArgs S;
    S.src[0] = c->u.p; S.src[1] = c->v.p; S.src[2] = c->w.p; S.src[3] = c->p.p;
    S.dst[0] = c->df_u.p; S.dst[1] = c->df_v.p; S.dst[2] = c->df_w.p; S.dst[3] = c->df_p.p;
    S.n[0] = c->g.NU; S.n[1] = c->g.NV; S.n[2] = c->g.NW; S.n[3] = c->g.NP;
    {
      LaunchScope ls(K_RHS, c->st, 16.0 * (faces + c->g.NP));
      const long nmax = std::max(std::max(S.n[0], S.n[1]), std::max(S.n[2], S.n[3]));
      const dim3 grid(std::max(1, wave_blocks(k_split_fields, nmax) / 4), 4);
      k_split_fields<<<grid, kThreads, 0, c->st>>>(S);
    }
    A.u2 = c->df_u.p; A.v2 = c->df_v.p; A.w2 = c->df_w.p; A.p2 = c->df_p.p;
    LaunchScope ls(K_RHS, c->st, 8.0 * faces + 9.0 * c->g.NP + nbox * (1 + 16 + 32));
    k_momentum_rhs<RhsDF><<<wave_blocks(k_momentum_rhs<RhsDF>, rows), kThreads, 0, c->st>>>(A);
  } else {
    A.u2 = A.v2 = A.w2 = A.p2 = nullptr;
    LaunchScope ls(K_RHS, c->st, 8.0 * faces + 9.0 * c->g.NP + nbox * (1 + 16 + 32));
    k_momentum_rhs<RhsF64><<<wave_blocks(k_momentum_rhs<RhsF64>, rows), kThreads, 0, c->st>>>(A);
  }
}

void launch_tilde(ibm_ctx *c) {
  const Dims d = dims_of(c);
  {
    const double faces = (double)(c->g.NU + c->g.NV + c->g.NW);
    LaunchScope ls(K_SCATTER, c->st, 16.0 * faces + 8.0 * (c->g.bu.n + c->g.bv.n + c->g.bw.n));
    k_scatter<<<wave_blocks(k_scatter, c->g.NU + c->g.NV + c->g.NW), kThreads, 0, c->st>>>(
        c->u.p, c->v.p, c->w.p, c->xb[0].p, c->xb[1].p, c->xb[2].p, c->ut.p, c->vt.p, c->wt.p, d, c->diag.p);
  }
  launch_bc(c, c->ut.p, c->vt.p, c->wt.p);
}

void launch_pressure_rhs(ibm_ctx *c) {
  DivArgs A;
  A.d = dims_of(c);
  A.ut = c->ut.p; A.vt = c->vt.p; A.wt = c->wt.p;
  A.fu = c->fu.p; A.fv = c->fv.p; A.fw = c->fw.p; A.fc = c->fc.p;
  A.Dc = c->Dc.p; A.div_bc = c->div_bc_cell.p;
  A.b = c->bb[3].p; A.x0 = c->xb[3].p;
  A.neg_a = -(c->g.rho / c->g.dt);
  A.ramp = c->dramp.p;
  const double faces = (double)(c->g.NU + c->g.NV + c->g.NW);
  LaunchScope ls(K_PRHS, c->st, 9.0 * faces + 73.0 * c->g.NP);
  k_pressure_rhs<<<wave_blocks(k_pressure_rhs, c->g.NP), kThreads, 0, c->st>>>(A);
}

// ------------------------------------------------------------------ forces
// Force of the fluid on the body (the reference computes none), from the
// end-of-step fields on the staircase of solid cells (non-fluid cells):
//  - pressure: a fluid cell next to a solid cell pushes the body with p times
//    the shared face's area, along the direction from the fluid cell into it;
//  - shear: a face velocity between two fluid cells whose two neighbours
//    across a coordinate direction are solid sees a no-slip wall half a cell
//    away: stress 2 rho nu u / h on the face's area in that direction.
// Each cell adds its own terms in a fixed order (pressure x, y, z; then the
// u, v, w faces on its lower side); blocks sum in a fixed order.
struct ForceArgs {
  Dims d;
  const double *u, *v, *w, *p;
  const uint8_t *fc;
  double dx, dy, dz, rho_nu2;   // rho_nu2 = 2 rho nu
  double *part;
  StepDiag *dg;
};

__device__ __forceinline__ void cell_force(const ForceArgs &A, long c, double f[3]) {
  const Dims &d = A.d;
  long q;
  const int i = udivmod(c, d.dnx, q);
  long kq;
      const int j = udivmod(q, d.dny, kq), k = (int)kq;
  const long sy = d.nx, sz = (long)d.nx * d.ny;
  auto solid = [&](int ii, int jj, int kk) {
    return ii >= 0 && ii < d.nx && jj >= 0 && jj < d.ny && kk >= 0 && kk < d.nz &&
           !(A.fc[((long)kk * d.ny + jj) * d.nx + ii] & kFluid);
  };
  auto fluid = [&](int ii, int jj, int kk) { return (A.fc[((long)kk * d.ny + jj) * d.nx + ii] & kFluid) != 0; };
  const double ax = A.dy * A.dz, ay = A.dx * A.dz, az = A.dx * A.dy;
  const double pc = A.p[c];
  if (solid(i + 1, j, k)) f[0] += pc * ax;
  if (solid(i - 1, j, k)) f[0] -= pc * ax;
  if (solid(i, j + 1, k)) f[1] += pc * ay;
  if (solid(i, j - 1, k)) f[1] -= pc * ay;
  if (solid(i, j, k + 1)) f[2] += pc * az;
  if (solid(i, j, k - 1)) f[2] -= pc * az;
  (void)sy; (void)sz;
  // u face on the lower x side, between cells i-1 and i
  if (i > 0 && fluid(i - 1, j, k)) {
    const double uf = A.u[U3(d, i, j, k)];
    const double t = A.rho_nu2 * uf;
    if (solid(i - 1, j + 1, k) && solid(i, j + 1, k)) f[0] += t * A.dx * A.dz / A.dy;
    if (solid(i - 1, j - 1, k) && solid(i, j - 1, k)) f[0] += t * A.dx * A.dz / A.dy;
    if (solid(i - 1, j, k + 1) && solid(i, j, k + 1)) f[0] += t * A.dx * A.dy / A.dz;
    if (solid(i - 1, j, k - 1) && solid(i, j, k - 1)) f[0] += t * A.dx * A.dy / A.dz;
  }
  if (j > 0 && fluid(i, j - 1, k)) {
    const double vf = A.v[V3(d, i, j, k)];
    const double t = A.rho_nu2 * vf;
    if (solid(i + 1, j - 1, k) && solid(i + 1, j, k)) f[1] += t * A.dy * A.dz / A.dx;
    if (solid(i - 1, j - 1, k) && solid(i - 1, j, k)) f[1] += t * A.dy * A.dz / A.dx;
    if (solid(i, j - 1, k + 1) && solid(i, j, k + 1)) f[1] += t * A.dx * A.dy / A.dz;
    if (solid(i, j - 1, k - 1) && solid(i, j, k - 1)) f[1] += t * A.dx * A.dy / A.dz;
  }
  if (k > 0 && fluid(i, j, k - 1)) {
    const double wf = A.w[W3(d, i, j, k)];
    const double t = A.rho_nu2 * wf;
    if (solid(i + 1, j, k - 1) && solid(i + 1, j, k)) f[2] += t * A.dz * A.dy / A.dx;
    if (solid(i - 1, j, k - 1) && solid(i - 1, j, k)) f[2] += t * A.dz * A.dy / A.dx;
    if (solid(i, j + 1, k - 1) && solid(i, j + 1, k)) f[2] += t * A.dz * A.dx / A.dy;
    if (solid(i, j - 1, k - 1) && solid(i, j - 1, k)) f[2] += t * A.dz * A.dx / A.dy;
  }
}

__global__ void __launch_bounds__(kThreads) k_forces(ForceArgs A) {
  const long NP = (long)A.d.nx * A.d.ny * A.d.nz;
  double f[3] = {0.0, 0.0, 0.0};
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < NP; c += (long)gridDim.x * blockDim.x)
    if (A.fc[c] & kFluid) cell_force(A, c, f);
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
      for (int w = 0; w < kWarps; ++w) a += s[q][w];
      A.part[3 * blockIdx.x + q] = a;
    }
  }
  __threadfence();
  __syncthreads();
  __shared__ int last;
  if (threadIdx.x == 0) last = (atomicAdd(&A.dg->fticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    for (int q = 0; q < 3; ++q) {
      double a = 0.0;
      for (int b = 0; b < (int)gridDim.x; ++b) a += A.part[3 * b + q];
      A.dg->force[q] = a;
    }
    A.dg->fticket = 0;
  }
}

void launch_forces(ibm_ctx *c) {
  if (c->prm.compute_forces == 2) {
    launch_forces_cut(c);
    return;
  }
  ForceArgs A;
  A.d = dims_of(c);
  A.u = c->u.p; A.v = c->v.p; A.w = c->w.p; A.p = c->p.p;
  A.fc = c->fc.p;
  A.dx = c->g.dx; A.dy = c->g.dy; A.dz = c->g.dz;
  A.rho_nu2 = 2.0 * c->g.rho * c->g.nu;
  A.part = c->part.p;
  A.dg = c->diag.p;
  const int nb = std::min(blocks_for(c->g.NP), 1024);
  LaunchScope ls(K_DIAG, c->st, 4.0 * 8.0 * c->g.NP + 7.0 * c->g.NP);
  k_forces<<<nb, kThreads, 0, c->st>>>(A);
}

void launch_projection(ibm_ctx *c) {
  ProjArgs A;
  A.d = dims_of(c);
  A.ut = c->ut.p; A.vt = c->vt.p; A.wt = c->wt.p; A.phi = c->xb[3].p;
  A.u = c->u.p; A.v = c->v.p; A.w = c->w.p; A.p = c->p.p;
  A.fu = c->fu.p; A.fv = c->fv.p; A.fw = c->fw.p; A.fc = c->fc.p;
  A.Gu = c->Gu.p; A.Gv = c->Gv.p; A.Gw = c->Gw.p;
  A.factor = c->g.dt / c->g.rho;
  A.dg = c->diag.p;
  const double faces = (double)(c->g.NU + c->g.NV + c->g.NW);
  {
    LaunchScope ls(K_PROJECT, c->st, 33.0 * faces + 25.0 * c->g.NP);
    k_project<<<wave_blocks(k_project, c->g.NU + c->g.NV + c->g.NW + c->g.NP), kThreads, 0, c->st>>>(A);
  }
  launch_bc(c, c->u.p, c->v.p, c->w.p);
  DiagArgs D;
  D.d = A.d;
  D.ut = c->ut.p; D.vt = c->vt.p; D.wt = c->wt.p; D.phi = c->xb[3].p;
  D.u = c->u.p; D.v = c->v.p; D.w = c->w.p;
  D.fu = c->fu.p; D.fv = c->fv.p; D.fw = c->fw.p; D.fc = c->fc.p;
  D.Gu = c->Gu.p; D.Gv = c->Gv.p; D.Gw = c->Gw.p; D.Dc = c->Dc.p; D.div_bc = c->div_bc_cell.p;
  D.factor = A.factor;
  D.ramp = c->dramp.p;
  // one wave: four resident blocks per SM (launch bounds), at most the 1024 partials of c->part
  const int nb = std::min(std::min(blocks_for(c->g.NP + c->g.NU + c->g.NV + c->g.NW), 4 * sm_count()), 1024);
  D.part = c->part.p;
  D.dg = c->diag.p;
  D.np_active = c->np_active;
  {
    LaunchScope ls(K_DIAG, c->st, 33.0 * faces + 65.0 * c->g.NP);
    k_diagnostics<<<nb, kThreads, 0, c->st>>>(D);
  }
  if (c->prm.compute_forces) launch_forces(c);
}

}  // namespace ibm

// Semicoarsening multigrid V-cycle used as the pressure preconditioner.
//
// Restates the published design of HYPRE's PFMG (third-party; configured by
// the reference at main.cu:207-221): each level is coarsened by two in one
// direction (the one with the smallest current spacing), interpolation is
// operator dependent along that direction (weights -sum(lower plane) /
// sum(own plane) and -sum(upper plane) / sum(own plane)), restriction is its
// transpose, coarse operators are Galerkin R A P (27-point), optionally
// collapsed to 7 points, the smoother is weighted Jacobi or a two-colour
// relaxation, and the coarsest level is solved with an explicit inverse.
//
// The hierarchy is built on the device once per pressure operator; the same
// kernels run in FP64 (plain form) and FP32 (mixed form, coefficients
// rounded from the FP64 hierarchy).
#include <algorithm>
#include <cmath>
#include <cstring>

#include <mutex>
#include <unordered_map>

#include "ibm_common.cuh"
#include "ibm_mg.cuh"

namespace ibm {

namespace {

__constant__ int c_slot7[7] = {13, 12, 14, 10, 16, 4, 22};  // Struct slot -> 27-point slot

__host__ __device__ inline int s27(int ox, int oy, int oz) { return (ox + 1) + 3 * (oy + 1) + 9 * (oz + 1); }
__host__ __device__ inline int s27_off(int s, int d) { return d == 0 ? s % 3 - 1 : d == 1 ? (s / 3) % 3 - 1 : s / 9 - 1; }

// Position of 27-point slot s among the stored slots (-1 when not stored).
__device__ inline int stored_slot(int ns, int s) {
  if (ns == 27) return s;
  switch (s) {
    case 13: return 0; case 12: return 1; case 14: return 2; case 10: return 3;
    case 16: return 4; case 4: return 5; case 22: return 6; default: return -1;
  }
}

__device__ inline bool gate_off(const int *gate) { return gate != nullptr && *gate == 0; }

template <class T>
__device__ inline T fmat(T a, T b, T c);
template <>
__device__ inline double fmat<double>(double a, double b, double c) { return fma(a, b, c); }
template <>
__device__ inline float fmat<float>(float a, float b, float c) { return fmaf(a, b, c); }

// (A x)_r for a stored 7- or 27-point level operator.
template <class T, int NS>
__device__ inline T apply_row(const T *__restrict__ A, long n, const T *__restrict__ x, int r, int i, int j, int k,
                              int nx, int ny, int nz) {
  T acc = T(0);
  if (NS == 7) {
    const long sy = nx, sz = (long)nx * ny;
    acc = fmat<T>(A[r], x[r], acc);
    acc = fmat<T>(A[n + r], i > 0 ? x[r - 1] : T(0), acc);
    acc = fmat<T>(A[2 * n + r], i < nx - 1 ? x[r + 1] : T(0), acc);
    acc = fmat<T>(A[3 * n + r], j > 0 ? x[r - sy] : T(0), acc);
    acc = fmat<T>(A[4 * n + r], j < ny - 1 ? x[r + sy] : T(0), acc);
    acc = fmat<T>(A[5 * n + r], k > 0 ? x[r - sz] : T(0), acc);
    acc = fmat<T>(A[6 * n + r], k < nz - 1 ? x[r + sz] : T(0), acc);
  } else {
#pragma unroll
    for (int s = 0; s < 27; ++s) {
      const int ii = i + s % 3 - 1, jj = j + (s / 3) % 3 - 1, kk = k + s / 9 - 1;
      const bool in = ii >= 0 && ii < nx && jj >= 0 && jj < ny && kk >= 0 && kk < nz;
      const T xv = in ? x[((long)kk * ny + jj) * nx + ii] : T(0);
      acc = fmat<T>(A[(long)s * n + r], xv, acc);
    }
  }
  return acc;
}

// ---------------------------------------------------------------- setup
__global__ void k_diag(const double *A, long n, double omega, double *invd, double *wd) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    const double d = A[r];  // slot 0 of either layout is... (27-point: centre at plane 13, see caller)
    const double id = d != 0.0 ? 1.0 / d : 0.0;
    invd[r] = id;
    wd[r] = omega * id;
  }
}

// 1 where a row has any off-diagonal coupling (0: an uncoupled point, e.g. a
// solid cell kept as an identity row).
__global__ void k_coupled(const double *A, int ns, long n, unsigned char *coupled) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    unsigned char c = 0;
    for (int q = 0; q < ns; ++q)
      if (q != (ns == 27 ? 13 : 0) && A[(long)q * n + r] != 0.0) c = 1;
    coupled[r] = c;
  }
}

// PFMG's operator-dependent weights. With `aware`, a coupled point that has no
// coupling along d (0/0 otherwise, e.g. a cut cell between the cylinder and a
// closed face) takes the constant from those of its two coarse neighbours that
// are coupled, so interpolation keeps reproducing constants there.
__global__ void k_interp_weights(const double *A, int ns, Box b, int d, const unsigned char *coupled, int aware,
                                 double *pm, double *pp) {
  const long n = b.n;
  const long stride = d == 0 ? 1 : d == 1 ? (long)b.nx : (long)b.nx * b.ny;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    double c0 = 0.0, cm = 0.0, cp = 0.0;
    for (int s = 0; s < 27; ++s) {
      const int q = stored_slot(ns, s);
      if (q < 0) continue;
      const double a = A[(long)q * n + r];
      const int od = s27_off(s, d);
      if (od == 0) c0 += a; else if (od < 0) cm += a; else cp += a;
    }
    double wm = 0.0, wp = 0.0;
    if (aware && coupled[r] && cm == 0.0 && cp == 0.0) {
      int idx[3];
      box_ijk(r, b, idx[0], idx[1], idx[2]);
      const int nd = d == 0 ? b.nx : d == 1 ? b.ny : b.nz;
      const int lo = idx[d] > 0 && coupled[r - stride];
      const int hi = idx[d] < nd - 1 && coupled[r + stride];
      if (lo + hi > 0) {
        wm = lo ? 1.0 / (lo + hi) : 0.0;
        wp = hi ? 1.0 / (lo + hi) : 0.0;
      }
    } else if (c0 != 0.0) {
      wm = -cm / c0;
      wp = -cp / c0;
    }
    pm[r] = wm;
    pp[r] = wp;
  }
}

// Level-0 operator of the symmetrized hierarchy: row r scaled by winv[r].
__global__ void k_scale_rows(const double *A7, const double *winv, long n, double *S7) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < 7 * n; t += (long)gridDim.x * blockDim.x)
    S7[t] = A7[t] * winv[t % n];
}

// Galerkin coarse operator, same summation order as the oracle (for each of
// the three restricting fine points, each fine stencil entry in slot order,
// each interpolating coarse point).
__global__ void k_rap(const double *Af, int ns, Box fb, const double *pm, const double *pp, int d, Box cb,
                      double *Ac) {
  for (long I = (long)blockIdx.x * blockDim.x + threadIdx.x; I < cb.n; I += (long)gridDim.x * blockDim.x) {
    int ci[3];
    box_ijk(I, cb, ci[0], ci[1], ci[2]);
    double ac[27];
#pragma unroll
    for (int s = 0; s < 27; ++s) ac[s] = 0.0;
    const int fn[3] = {fb.nx, fb.ny, fb.nz};
    const int cn[3] = {cb.nx, cb.ny, cb.nz};
    for (int fo = -1; fo <= 1; ++fo) {
      int f[3] = {ci[0], ci[1], ci[2]};
      f[d] = 2 * ci[d] + fo;
      if (f[d] < 0 || f[d] >= fn[d]) continue;
      const long fr = ((long)f[2] * fb.ny + f[1]) * fb.nx + f[0];
      const double rw = fo == 0 ? 1.0 : (fo < 0 ? pp[fr] : pm[fr]);
      if (rw == 0.0) continue;
      for (int s = 0; s < 27; ++s) {
        const int q = stored_slot(ns, s);
        if (q < 0) continue;
        const double a = Af[(long)q * fb.n + fr];
        if (a == 0.0) continue;
        const int o3[3] = {s27_off(s, 0), s27_off(s, 1), s27_off(s, 2)};
        const int g[3] = {f[0] + o3[0], f[1] + o3[1], f[2] + o3[2]};
        if (g[0] < 0 || g[0] >= fn[0] || g[1] < 0 || g[1] >= fn[1] || g[2] < 0 || g[2] >= fn[2]) continue;
        const long gr = ((long)g[2] * fb.ny + g[1]) * fb.nx + g[0];
        const double ra = rw * a;
        int jc[2];
        double pw[2];
        int nt;
        if ((g[d] & 1) == 0) { jc[0] = g[d] / 2; pw[0] = 1.0; nt = 1; }
        else {
          jc[0] = (g[d] - 1) / 2; pw[0] = pm[gr]; nt = 1;
          if ((g[d] + 1) / 2 < cn[d]) { jc[1] = (g[d] + 1) / 2; pw[1] = pp[gr]; nt = 2; }
        }
        for (int t = 0; t < nt; ++t) {
          if (pw[t] == 0.0) continue;
          int oc[3] = {o3[0], o3[1], o3[2]};
          oc[d] = jc[t] - ci[d];
          const int sc = s27(oc[0], oc[1], oc[2]);
#pragma unroll
          for (int u = 0; u < 27; ++u)
            if (u == sc) ac[u] = ac[u] + ra * pw[t];
        }
      }
    }
#pragma unroll
    for (int s = 0; s < 27; ++s) Ac[(long)s * cb.n + I] = ac[s];
  }
}

// 27 -> 7 point collapse preserving constants and linear functions (same order as the oracle).
// 27 -> 7 points: each off-axis entry moves to the axis neighbours it spans,
// the centre keeping the row sum. With `aware`, only coupled axis neighbours
// receive it (a coupling moved onto an uncoupled point, such as a solid cell,
// would make a Neumann wall act as a Dirichlet one on the coarse grid); with
// none the entry is lumped into the centre.
__global__ void k_collapse7(const double *A27, Box b, const unsigned char *coupled, int aware, double *A7) {
  const long n = b.n;
  const long st[3] = {1, (long)b.nx, (long)b.nx * b.ny};
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    double a[27];
#pragma unroll
    for (int s = 0; s < 27; ++s) a[s] = A27[(long)s * n + r];
    for (int s = 0; s < 27; ++s) {
      const int o3[3] = {s27_off(s, 0), s27_off(s, 1), s27_off(s, 2)};
      const int m = (o3[0] != 0) + (o3[1] != 0) + (o3[2] != 0);
      if (m < 2 || a[s] == 0.0) continue;
      const double e = a[s];
      a[s] = 0.0;
      int t = 0;
      for (int dd = 0; dd < 3; ++dd) {
        if (!o3[dd]) continue;
        if (aware && !coupled[r + o3[dd] * st[dd]]) continue;
        int q[3] = {0, 0, 0};
        q[dd] = o3[dd];
        const int sq = s27(q[0], q[1], q[2]);
        a[sq] = a[sq] + e;
        ++t;
      }
      a[13] = a[13] - (double)(t - 1) * e;
    }
    for (int q = 0; q < 7; ++q) A7[(long)q * n + r] = a[c_slot7[q]];
  }
}

template <class T>
__global__ void k_convert(const double *src, T *dst, long n) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    dst[r] = (T)src[r];
}

// ---------------------------------------------------------------- V-cycle
template <class T>
__global__ void k_load_input(T *bv, long n, VecRef in, const double *winv, const int *gate) {
  if (gate_off(gate)) return;
  const long off = in.idx ? (long)(*in.idx) * in.ld : 0;
  const double sc = in.nu ? 1.0 / in.nu[in.idx ? *in.idx : 0] : 1.0;
  const double *src = in.base + off;
  const float *srcf = in.basef ? in.basef + off : nullptr;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    const double a = srcf ? (double)srcf[r] : src[r];
    double v = in.nu ? a * sc : a;
    if (winv) v = v * winv[r];
    bv[r] = (T)v;
  }
}

// FP32 hierarchy fed from an FP32 basis: four rows per thread, scale and
// symmetrizer applied in FP32 (n % 4 == 0, 16-byte aligned source).
__global__ void k_load_input_f4(float *bv, long n, VecRef in, const float *winvf, const int *gate) {
  if (gate_off(gate)) return;
  const long off = in.idx ? (long)(*in.idx) * in.ld : 0;
  const float sc = in.nu ? (float)(1.0 / in.nu[in.idx ? *in.idx : 0]) : 1.0f;
  const float *srcf = in.basef + off;
  for (long r0 = 4 * ((long)blockIdx.x * blockDim.x + threadIdx.x); r0 < n; r0 += 4L * gridDim.x * blockDim.x) {
    float4 a = *reinterpret_cast<const float4 *>(srcf + r0);
    a.x *= sc; a.y *= sc; a.z *= sc; a.w *= sc;
    if (winvf) {
      const float4 w = *reinterpret_cast<const float4 *>(winvf + r0);
      a.x *= w.x; a.y *= w.y; a.z *= w.z; a.w *= w.w;
    }
    *reinterpret_cast<float4 *>(bv + r0) = a;
  }
}

template <class T>
__global__ void k_store_output(const T *x, long n, OutRef out, const int *gate) {
  if (gate_off(gate)) return;
  const long off = out.idx ? (long)(*out.idx) * out.ld : 0;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    if (out.d) out.d[off + r] = (double)x[r];
    else out.f[off + r] = (float)x[r];
  }
}

template <class T>
__global__ void k_relax_zero(const T *wd, const T *b, T *x, long n, const int *gate) {
  if (gate_off(gate)) return;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    x[r] = wd[r] * b[r];
}

// Weighted Jacobi: t = x + wd (b - A x).
template <class T, int NS>
__global__ void k_relax_jacobi(const T *A, const T *wd, const T *b, const T *x, T *t, Box bx, const int *gate) {
  if (gate_off(gate)) return;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < bx.n; r += (long)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(r, bx, i, j, k);
    const T ax = apply_row<T, NS>(A, bx.n, x, (int)r, i, j, k, bx.nx, bx.ny, bx.nz);
    t[r] = fmat<T>(wd[r], b[r] - ax, x[r]);
  }
}

// One colour phase of the two-colour relaxation: points of `color` take
// x + invd (b - A x) from the phase's input; the others are copied.
// zero_x treats the input as all zeros (first phase of a zero-guess sweep).
template <class T, int NS>
__global__ void k_relax_color(const T *A, const T *invd, const T *b, const T *x, T *t, Box bx, int color,
                              int zero_x, const int *gate) {
  if (gate_off(gate)) return;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < bx.n; r += (long)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(r, bx, i, j, k);
    if (((i + j + k) & 1) != color) { t[r] = zero_x ? T(0) : x[r]; continue; }
    if (zero_x) { t[r] = invd[r] * b[r]; continue; }
    const T ax = apply_row<T, NS>(A, bx.n, x, (int)r, i, j, k, bx.nx, bx.ny, bx.nz);
    t[r] = fmat<T>(invd[r], b[r] - ax, x[r]);
  }
}

// Colour-split coefficients of levels with an even nx. Rows 2m and 2m+1 lie on
// one x line and have opposite colours (parity of i+j+k), so the pair index m
// numbers the points of either colour. Each point keeps one contiguous record
// (array of structures, so a warp reads one contiguous block per phase and a
// thread loads its record with 16-byte vector loads):
//   7-point levels:  [c][m][8]  = inverse diagonal, couplings -x,+x,-y,+y,-z,+z, diagonal
//   27-point levels: [c][m][28] = the 27 coefficients (27-point slot order), inverse diagonal
__device__ __forceinline__ long rb_row(long m, int color, const Box &b, int &i, int &j, int &k) {
  const unsigned q = 2u * (unsigned)m;
  const unsigned line = fast_div(q, b.dx);
  const unsigned kk = fast_div(line, b.dy);
  j = (int)(line - kk * (unsigned)b.ny);
  k = (int)kk;
  const unsigned r = q + ((j + k + color) & 1);
  i = (int)(r - line * (unsigned)b.nx);
  return (long)r;
}

// Vector loads of a record of N values of T (N * sizeof(T) a multiple of 16).
template <class T, int N>
__device__ __forceinline__ void load_rec(const T *__restrict__ p, T (&v)[N]) {
  static_assert((N * sizeof(T)) % 16 == 0, "records are whole 16-byte units");
  const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
  for (int u = 0; u < (int)(N * sizeof(T) / 16); ++u) {
    // streamed once per phase: evict-first, so the solution and right-hand
    // side of the level stay in L2 across the phases
    const float4 f = __ldcs(q + u);
    memcpy(reinterpret_cast<char *>(v) + 16 * u, &f, 16);
  }
}

// Where a level's colour-split records live: the records themselves, or a
// 2-byte class per record and the table of distinct records (record classes,
// ibm_classes.cu). The table is small and read through the read-only cache;
// the per-record data streams.
template <class T, int W>
struct Recs {
  const T *R = nullptr;            // [c][m][W]
  const uint16_t *code = nullptr;  // [c][m] when classed
  const T *tab = nullptr;          // [K][W]
};
template <class T, int W>
__device__ __forceinline__ void load_recs(const Recs<T, W> &s, long idx, T (&v)[W]) {
  if (s.code) {
    const float4 *q = reinterpret_cast<const float4 *>(s.tab + (long)__ldcs(s.code + idx) * W);
#pragma unroll
    for (int u = 0; u < (int)(W * sizeof(T) / 16); ++u) {
      const float4 f = __ldg(q + u);
      memcpy(reinterpret_cast<char *>(v) + 16 * u, &f, 16);
    }
  } else {
    load_rec<T, W>(s.R + idx * W, v);
  }
}
template <class T, int W>
__device__ __forceinline__ const T *rec_ptr(const Recs<T, W> &s, long idx) {
  return s.code ? s.tab + (long)__ldcs(s.code + idx) * W : s.R + idx * W;
}

template <class T>
__global__ void k_split_colors(const T *A, const T *invd, Box bx, T *R) {
  const long h = bx.n / 2;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < 2 * h; t += (long)gridDim.x * blockDim.x) {
    const int c = (int)(t / h);
    const long m = t - c * h;
    int i, j, k;
    const long r = rb_row(m, c, bx, i, j, k);
    T *o = R + ((long)c * h + m) * 8;
    o[0] = invd[r];
    for (int s = 1; s < 7; ++s) o[s] = A[(long)s * bx.n + r];
    o[7] = A[r];
  }
}

// One colour phase in place: x_r = invd_r (b_r - sum of the couplings to the
// other colour's points). Points of one colour are not coupled to each other
// in a 7-point stencil, so the phase reads only values it does not write.
template <class T>
__global__ void __launch_bounds__(kThreads) k_relax_rb(Recs<T, 8> R, const T *__restrict__ b, T *x,
                                                       Box bx, int color, const int *gate) {
  if (gate_off(gate)) return;
  const long h = bx.n / 2;
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const long sy = nx, sz = (long)nx * ny;
  for (long m = (long)blockIdx.x * blockDim.x + threadIdx.x; m < h; m += (long)gridDim.x * blockDim.x) {
    int i, j, k;
    const long r = rb_row(m, color, bx, i, j, k);
    T c[8];
    load_recs<T, 8>(R, (long)color * h + m, c);
    const T xw = i > 0 ? x[r - 1] : T(0);
    const T xe = i < nx - 1 ? x[r + 1] : T(0);
    const T xs = j > 0 ? x[r - sy] : T(0);
    const T xn = j < ny - 1 ? x[r + sy] : T(0);
    const T xb = k > 0 ? x[r - sz] : T(0);
    const T xt = k < nz - 1 ? x[r + sz] : T(0);
    T acc = T(0);
    acc = fmat<T>(c[1], xw, acc);
    acc = fmat<T>(c[2], xe, acc);
    acc = fmat<T>(c[3], xs, acc);
    acc = fmat<T>(c[4], xn, acc);
    acc = fmat<T>(c[5], xb, acc);
    acc = fmat<T>(c[6], xt, acc);
    x[r] = c[0] * (b[r] - acc);
  }
}

// 27-point levels: diagonal neighbours share a colour, so a phase cannot
// update in place: it writes every point of the pair to the other buffer (the
// own-colour point relaxed, the other copied), with the same arithmetic as
// k_relax_color.
template <class T>
__global__ void k_split_colors27(const T *A, const T *invd, Box bx, T *R) {
  const long h = bx.n / 2;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < 2 * h; t += (long)gridDim.x * blockDim.x) {
    const int c = (int)(t / h);
    const long m = t - c * h;
    int i, j, k;
    const long r = rb_row(m, c, bx, i, j, k);
    T *o = R + ((long)c * h + m) * 28;
    for (int s = 0; s < 27; ++s) o[s] = A[(long)s * bx.n + r];
    o[27] = invd[r];
  }
}

// Kernel bodies below take their first item and stride (t0, ts) so that the
// stand-alone kernels and the fused coarse-level kernel (k_mg_tail) run the
// same per-point arithmetic.
template <class T>
__device__ __forceinline__ void relax_rb27_body(const Recs<T, 28> &R, const T *b, const T *x, T *t, const Box &bx,
                                                int color, int zero_x, long t0, long ts) {
  const long h = bx.n / 2;
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  for (long m = t0; m < h; m += ts) {
    int i, j, k;
    const long r = rb_row(m, color, bx, i, j, k);
    const long idx = (long)color * h + m;
    if (zero_x) {
      t[r] = rec_ptr<T, 28>(R, idx)[27] * b[r];
      t[r ^ 1] = T(0);
      continue;
    }
    // FP32 records come in with vector loads; FP64 ones (twice the registers)
    // are read one value at a time
    T c[sizeof(T) == 4 ? 28 : 1];
    if constexpr (sizeof(T) == 4) load_recs<T, 28>(R, idx, c);
    const T *__restrict__ pr = sizeof(T) == 4 ? nullptr : rec_ptr<T, 28>(R, idx);
    T acc = T(0);
#pragma unroll
    for (int s = 0; s < 27; ++s) {
      const int ii = i + s % 3 - 1, jj = j + (s / 3) % 3 - 1, kk = k + s / 9 - 1;
      const bool in = ii >= 0 && ii < nx && jj >= 0 && jj < ny && kk >= 0 && kk < nz;
      const T xv = in ? x[((long)kk * ny + jj) * nx + ii] : T(0);
      T cs;
      if constexpr (sizeof(T) == 4) cs = c[s];
      else cs = pr[s];
      acc = fmat<T>(cs, xv, acc);
    }
    T cd;
    if constexpr (sizeof(T) == 4) cd = c[27];
    else cd = pr[27];
    t[r] = fmat<T>(cd, b[r] - acc, x[r]);
    t[r ^ 1] = x[r ^ 1];
  }
}
template <class T>
__global__ void __launch_bounds__(kThreads, 4) k_relax_rb27(Recs<T, 28> R, const T *__restrict__ b,
                                                         const T *__restrict__ x, T *__restrict__ t, Box bx,
                                                         int color, int zero_x, const int *gate) {
  if (gate_off(gate)) return;
  relax_rb27_body<T>(R, b, x, t, bx, color, zero_x, (long)blockIdx.x * blockDim.x + threadIdx.x,
                     (long)gridDim.x * blockDim.x);
}

// Quartet form of the FP32 27-point phase (nx a multiple of 4): a thread
// takes four consecutive points of a line, loads the 9 x 6 window of x values
// their stencils touch (16-byte loads plus the two edge values per line, 0
// outside the box) and writes the pair's four outputs with one 16-byte store:
// the phase colour's points relaxed, the others copied. Per point the
// arithmetic is k_relax_rb27's, in the same slot order.
__device__ __forceinline__ void relax_rb27_quad_body(const Recs<float, 28> &R, const float *b, const float *x,
                                                     float *t, const Box &bx, int color, int zero_x, long t0,
                                                     long ts) {
  const long h = bx.n / 2, n4 = bx.n / 4;
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  for (long q = t0; q < n4; q += ts) {
    const long r0 = 4 * q;
    const unsigned line = fast_div((unsigned)r0, bx.dx);
    const int i0 = (int)((unsigned)r0 - line * (unsigned)nx);
    const unsigned kk = fast_div(line, bx.dy);
    const int j = (int)(line - kk * (unsigned)ny), k = (int)kk;
    const int p = (j + k + color) & 1;  // the phase's points are l = p, p + 2
    const long m0 = (long)color * h + r0 / 2;
    const float4 bq = *reinterpret_cast<const float4 *>(b + r0);
    const float bb[4] = {bq.x, bq.y, bq.z, bq.w};
    if (zero_x) {
      float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int u = 0; u < 2; ++u) o[p + 2 * u] = rec_ptr<float, 28>(R, m0 + u)[27] * bb[p + 2 * u];
      *reinterpret_cast<float4 *>(t + r0) = make_float4(o[0], o[1], o[2], o[3]);
      continue;
    }
    // w[L][c]: line L = (dj + 1) + 3 (dk + 1), column i0 - 1 + c
    float w[9][6];
#pragma unroll
    for (int L = 0; L < 9; ++L) {
      const int jj = j + L % 3 - 1, kz = k + L / 3 - 1;
      if (jj >= 0 && jj < ny && kz >= 0 && kz < nz) {
        const float *xr = x + ((long)kz * ny + jj) * nx + i0;
        const float4 v = *reinterpret_cast<const float4 *>(xr);
        w[L][0] = i0 > 0 ? xr[-1] : 0.0f;
        w[L][1] = v.x; w[L][2] = v.y; w[L][3] = v.z; w[L][4] = v.w;
        w[L][5] = i0 + 4 < nx ? xr[4] : 0.0f;
      } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) w[L][c] = 0.0f;
      }
    }
    float o[4] = {w[4][1], w[4][2], w[4][3], w[4][4]};
    auto relax_at = [&](int l, const float (&c)[28]) {
      float acc = 0.0f;
#pragma unroll
      for (int s = 0; s < 27; ++s) acc = fmaf(c[s], w[s / 3][l + s % 3], acc);
      return fmaf(c[27], bb[l] - acc, w[4][l + 1]);
    };
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      float c[28];
      load_recs<float, 28>(R, m0 + u, c);
      if (p == 0) o[2 * u] = relax_at(2 * u, c);
      else o[2 * u + 1] = relax_at(2 * u + 1, c);
    }
    *reinterpret_cast<float4 *>(t + r0) = make_float4(o[0], o[1], o[2], o[3]);
  }
}
__global__ void __launch_bounds__(kThreads) k_relax_rb27_quad(Recs<float, 28> R, const float *__restrict__ b,
                                                              const float *__restrict__ x, float *__restrict__ t,
                                                              Box bx, int color, int zero_x, const int *gate) {
  if (gate_off(gate)) return;
  relax_rb27_quad_body(R, b, x, t, bx, color, zero_x, (long)blockIdx.x * blockDim.x + threadIdx.x,
                       (long)gridDim.x * blockDim.x);
}

// Quartet form of the FP32 27-point residual (nx a multiple of 4): the 9 x 6
// window of x as in k_relax_rb27_quad, all four points b - A x in
// k_residual_rb27's slot order, one 16-byte store.
__device__ __forceinline__ void residual_rb27_quad_body(const Recs<float, 28> &R, const float *b, const float *x,
                                                        float *res, const Box &bx, long t0, long ts) {
  const long h = bx.n / 2, n4 = bx.n / 4;
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  for (long q = t0; q < n4; q += ts) {
    const long r0 = 4 * q;
    const unsigned line = fast_div((unsigned)r0, bx.dx);
    const int i0 = (int)((unsigned)r0 - line * (unsigned)nx);
    const unsigned kk = fast_div(line, bx.dy);
    const int j = (int)(line - kk * (unsigned)ny), k = (int)kk;
    const int p0 = (j + k) & 1;  // colour of the quad's even points (l = 0, 2)
    float w[9][6];
#pragma unroll
    for (int L = 0; L < 9; ++L) {
      const int jj = j + L % 3 - 1, kz = k + L / 3 - 1;
      if (jj >= 0 && jj < ny && kz >= 0 && kz < nz) {
        const float *xr = x + ((long)kz * ny + jj) * nx + i0;
        const float4 v = *reinterpret_cast<const float4 *>(xr);
        w[L][0] = i0 > 0 ? xr[-1] : 0.0f;
        w[L][1] = v.x; w[L][2] = v.y; w[L][3] = v.z; w[L][4] = v.w;
        w[L][5] = i0 + 4 < nx ? xr[4] : 0.0f;
      } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) w[L][c] = 0.0f;
      }
    }
    const float4 bq = *reinterpret_cast<const float4 *>(b + r0);
    const float bb[4] = {bq.x, bq.y, bq.z, bq.w};
    float o[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      // point l has colour p0 ^ (l & 1); its record is m = (r0 + l) / 2 of that colour
      const int col = p0 ^ (l & 1);
      float c[28];
      load_recs<float, 28>(R, (long)col * h + r0 / 2 + l / 2, c);
      float acc = 0.0f;
#pragma unroll
      for (int s = 0; s < 27; ++s) acc = fmaf(c[s], w[s / 3][l + s % 3], acc);
      o[l] = bb[l] - acc;
    }
    *reinterpret_cast<float4 *>(res + r0) = make_float4(o[0], o[1], o[2], o[3]);
  }
}
__global__ void __launch_bounds__(kThreads) k_residual_rb27_quad(Recs<float, 28> R, const float *__restrict__ b,
                                                                 const float *__restrict__ x,
                                                                 float *__restrict__ res, Box bx, const int *gate) {
  if (gate_off(gate)) return;
  residual_rb27_quad_body(R, b, x, res, bx, (long)blockIdx.x * blockDim.x + threadIdx.x,
                          (long)gridDim.x * blockDim.x);
}

// Residual of a 27-point level from its colour-split records: every point
// (both colours; same-colour points are coupled), b - A x in apply_row's slot
// order, so the result equals k_residual<T, 27> bit for bit.
template <class T>
__device__ __forceinline__ void residual_rb27_body(const Recs<T, 28> &R, const T *b, const T *x, T *res,
                                                   const Box &bx, long t0, long ts) {
  const long h = bx.n / 2;
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  for (long t = t0; t < 2 * h; t += ts) {
    const int color = t >= h;
    const long m = t - color * h;
    int i, j, k;
    const long r = rb_row(m, color, bx, i, j, k);
    T c[sizeof(T) == 4 ? 28 : 1];
    if constexpr (sizeof(T) == 4) load_recs<T, 28>(R, t, c);
    const T *__restrict__ pr = sizeof(T) == 4 ? nullptr : rec_ptr<T, 28>(R, t);
    T acc = T(0);
#pragma unroll
    for (int s = 0; s < 27; ++s) {
      const int ii = i + s % 3 - 1, jj = j + (s / 3) % 3 - 1, kk = k + s / 9 - 1;
      const bool in = ii >= 0 && ii < nx && jj >= 0 && jj < ny && kk >= 0 && kk < nz;
      const T xv = in ? x[((long)kk * ny + jj) * nx + ii] : T(0);
      T cs;
      if constexpr (sizeof(T) == 4) cs = c[s];
      else cs = pr[s];
      acc = fmat<T>(cs, xv, acc);
    }
    res[r] = b[r] - acc;
  }
}
template <class T>
__global__ void __launch_bounds__(kThreads, 4) k_residual_rb27(Recs<T, 28> R, const T *__restrict__ b,
                                                            const T *__restrict__ x, T *__restrict__ res, Box bx,
                                                            const int *gate) {
  if (gate_off(gate)) return;
  residual_rb27_body<T>(R, b, x, res, bx, (long)blockIdx.x * blockDim.x + threadIdx.x,
                        (long)gridDim.x * blockDim.x);
}

// Residual after a two-colour sweep that ended with colour 1: the colour-1
// points were just solved exactly against their colour-0 neighbours, so their
// residual is zero up to rounding and is written as 0; colour-0 points take
// b - A x with the colour-split coefficients (centre first, as apply_row).
template <class T>
__global__ void __launch_bounds__(kThreads) k_residual_rb(Recs<T, 8> R, const T *__restrict__ b,
                                                          const T *__restrict__ x, T *__restrict__ res, Box bx,
                                                          const int *gate) {
  if (gate_off(gate)) return;
  const long h = bx.n / 2;
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const long sy = nx, sz = (long)nx * ny;
  for (long m = (long)blockIdx.x * blockDim.x + threadIdx.x; m < h; m += (long)gridDim.x * blockDim.x) {
    int i, j, k;
    const long r = rb_row(m, 0, bx, i, j, k);
    T c[8];
    load_recs<T, 8>(R, m, c);
    const T xc = x[r];
    const T xw = i > 0 ? x[r - 1] : T(0);
    const T xe = i < nx - 1 ? x[r + 1] : T(0);
    const T xs = j > 0 ? x[r - sy] : T(0);
    const T xn = j < ny - 1 ? x[r + sy] : T(0);
    const T xb = k > 0 ? x[r - sz] : T(0);
    const T xt = k < nz - 1 ? x[r + sz] : T(0);
    T acc = T(0);
    acc = fmat<T>(c[7], xc, acc);
    acc = fmat<T>(c[1], xw, acc);
    acc = fmat<T>(c[2], xe, acc);
    acc = fmat<T>(c[3], xs, acc);
    acc = fmat<T>(c[4], xn, acc);
    acc = fmat<T>(c[5], xb, acc);
    acc = fmat<T>(c[6], xt, acc);
    res[r] = b[r] - acc;
    res[r ^ 1] = T(0);
  }
}

// Quartet form of the FP32 in-place phases (nx a multiple of 4): a thread
// takes four consecutive points of a line, two of each colour, and issues its
// loads (two records, b and the x values of its own and the four neighbouring
// lines as 16-byte vectors) before it computes. One point per thread leaves a
// phase latency-bound on its dependent loads; the quad puts about a dozen
// independent loads in flight per thread at 60 registers (four blocks per SM).
// Per point the arithmetic is k_relax_rb's, in the same order.
// The two records of a quad's points of one colour (record indices m0, m0+1).
__device__ __forceinline__ void load_quad_recs(const Recs<float, 8> &R, long m0, float (&c)[2][8]) {
  if (R.code) {
    const ushort2 k2 = __ldcs(reinterpret_cast<const ushort2 *>(R.code + m0));
    const unsigned short ks[2] = {k2.x, k2.y};
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const float4 *qq = reinterpret_cast<const float4 *>(R.tab + 8 * (long)ks[t]);
      const float4 u = __ldg(qq), w = __ldg(qq + 1);
      c[t][0] = u.x; c[t][1] = u.y; c[t][2] = u.z; c[t][3] = u.w;
      c[t][4] = w.x; c[t][5] = w.y; c[t][6] = w.z; c[t][7] = w.w;
    }
  } else {
#pragma unroll
    for (int t = 0; t < 2; ++t) load_rec<float, 8>(R.R + (m0 + t) * 8, c[t]);
  }
}

template <int P>
__device__ __forceinline__ void relax_quad(const float (&c)[2][8], const float4 &bq, const float4 &xc,
                                           const float4 &xs, const float4 &xn, const float4 &xb, const float4 &xt,
                                           float xl, float xr, float (&out)[2]) {
  const float cc[4] = {xc.x, xc.y, xc.z, xc.w}, ss[4] = {xs.x, xs.y, xs.z, xs.w}, nn[4] = {xn.x, xn.y, xn.z, xn.w};
  const float bo[4] = {xb.x, xb.y, xb.z, xb.w}, tt[4] = {xt.x, xt.y, xt.z, xt.w}, bb[4] = {bq.x, bq.y, bq.z, bq.w};
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const int l = P + 2 * t;
    const float xw = l == 0 ? xl : cc[l == 0 ? 0 : l - 1];
    const float xe = l == 3 ? xr : cc[l == 3 ? 3 : l + 1];
    float acc = 0.0f;
    acc = fmaf(c[t][1], xw, acc);
    acc = fmaf(c[t][2], xe, acc);
    acc = fmaf(c[t][3], ss[l], acc);
    acc = fmaf(c[t][4], nn[l], acc);
    acc = fmaf(c[t][5], bo[l], acc);
    acc = fmaf(c[t][6], tt[l], acc);
    out[t] = c[t][0] * (bb[l] - acc);
  }
}

// One quad of an FP32 in-place phase: the four points r0 .. r0+3 of line
// (j, k) from column i0.
__device__ __forceinline__ void relax_quad_at(const Recs<float, 8> &R, const float *__restrict__ b, float *x,
                                              const Box &bx, int color, int zero_x, long r0, int i0, int j, int k,
                                              float *zout = nullptr) {
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const long sy = nx, sz = (long)nx * ny;
  const int p = (j + k + color) & 1;
  const long m0 = (long)color * (bx.n / 2) + r0 / 2;
  float c[2][8];
  load_quad_recs(R, m0, c);
  const float4 bq = *reinterpret_cast<const float4 *>(b + r0);
  if (zero_x) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p == 0) { v.x = c[0][0] * bq.x; v.z = c[1][0] * bq.z; }
    else { v.y = c[0][0] * bq.y; v.w = c[1][0] * bq.w; }
    *reinterpret_cast<float4 *>(x + r0) = v;
    return;
  }
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 xc = *reinterpret_cast<const float4 *>(x + r0);
  const float4 xs = j > 0 ? *reinterpret_cast<const float4 *>(x + r0 - sy) : z4;
  const float4 xn = j < ny - 1 ? *reinterpret_cast<const float4 *>(x + r0 + sy) : z4;
  const float4 xb = k > 0 ? *reinterpret_cast<const float4 *>(x + r0 - sz) : z4;
  const float4 xt = k < nz - 1 ? *reinterpret_cast<const float4 *>(x + r0 + sz) : z4;
  const float xl = i0 > 0 ? x[r0 - 1] : 0.0f;
  const float xr = i0 + 4 < nx ? x[r0 + 4] : 0.0f;
  float out[2];
  float4 q = xc;  // the quad after the phase
  if (p == 0) {
    relax_quad<0>(c, bq, xc, xs, xn, xb, xt, xl, xr, out);
    x[r0] = out[0];
    x[r0 + 2] = out[1];
    q.x = out[0];
    q.z = out[1];
  } else {
    relax_quad<1>(c, bq, xc, xs, xn, xb, xt, xl, xr, out);
    x[r0 + 1] = out[0];
    x[r0 + 3] = out[1];
    q.y = out[0];
    q.w = out[1];
  }
  if (zout) *reinterpret_cast<float4 *>(zout + r0) = q;
}

// The finest level's first phase from a zero guess with the V-cycle's input
// load fused in (k_load_input_f4's b = winv * in / nu, then k_relax_rb_quad's
// zero phase), and its last phase with the output store fused in (the whole
// quad also written to the preconditioned direction). Same values as the
// separate kernels.
__global__ void __launch_bounds__(kThreads) k_relax_rb_quad_in(Recs<float, 8> R, float *bv, float *x, Box bx,
                                                               VecRef in, const float *winvf, const int *gate) {
  if (gate_off(gate)) return;
  const long n4 = bx.n / 4;
  const long off = in.idx ? (long)(*in.idx) * in.ld : 0;
  const float sc = in.nu ? (float)(1.0 / in.nu[in.idx ? *in.idx : 0]) : 1.0f;
  const float *srcf = in.basef + off;
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long)gridDim.x * blockDim.x) {
    const long r0 = 4 * q;
    float4 a = *reinterpret_cast<const float4 *>(srcf + r0);
    a.x *= sc; a.y *= sc; a.z *= sc; a.w *= sc;
    if (winvf) {
      const float4 w = *reinterpret_cast<const float4 *>(winvf + r0);
      a.x *= w.x; a.y *= w.y; a.z *= w.z; a.w *= w.w;
    }
    *reinterpret_cast<float4 *>(bv + r0) = a;
    const unsigned line = fast_div((unsigned)r0, bx.dx);
    const unsigned kk = fast_div(line, bx.dy);
    const int j = (int)(line - kk * (unsigned)bx.ny), k = (int)kk;
    const int p = (j + k) & 1;  // colour-0 points of the quad
    float c[2][8];
    load_quad_recs(R, r0 / 2, c);
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p == 0) { v.x = c[0][0] * a.x; v.z = c[1][0] * a.z; }
    else { v.y = c[0][0] * a.y; v.w = c[1][0] * a.w; }
    *reinterpret_cast<float4 *>(x + r0) = v;
  }
}

__global__ void __launch_bounds__(kThreads) k_relax_rb_quad_out(Recs<float, 8> R, const float *__restrict__ b,
                                                                float *x, Box bx, int color, OutRef out,
                                                                const int *gate) {
  if (gate_off(gate)) return;
  const long n4 = bx.n / 4;
  float *z = out.f + (out.idx ? (long)(*out.idx) * out.ld : 0);
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long)gridDim.x * blockDim.x) {
    const long r0 = 4 * q;
    const unsigned line = fast_div((unsigned)r0, bx.dx);
    const int i0 = (int)((unsigned)r0 - line * (unsigned)bx.nx);
    const unsigned kk = fast_div(line, bx.dy);
    relax_quad_at(R, b, x, bx, color, 0, r0, i0, (int)(line - kk * (unsigned)bx.ny), (int)kk, z);
  }
}

__global__ void __launch_bounds__(kThreads) k_relax_rb_quad(Recs<float, 8> R, const float *__restrict__ b, float *x,
                                                            Box bx, int color, int zero_x, const int *gate) {
  if (gate_off(gate)) return;
  const long n4 = bx.n / 4;
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long)gridDim.x * blockDim.x) {
    const long r0 = 4 * q;
    const unsigned line = fast_div((unsigned)r0, bx.dx);
    const int i0 = (int)((unsigned)r0 - line * (unsigned)bx.nx);
    const unsigned kk = fast_div(line, bx.dy);
    relax_quad_at(R, b, x, bx, color, zero_x, r0, i0, (int)(line - kk * (unsigned)bx.ny), (int)kk);
  }
}

// One whole two-colour sweep of a 7-point FP32 level (colour 0, then colour
// 1) in one kernel, out of place: x_new = sweep(x_old). A block takes a tile
// of kSwJ x kSwK lines and kSwX points of each, loads x_old over the tile
// and a two-line (two-point) halo into shared memory, relaxes the colour-0
// points of the tile and of a one-line halo ring there, then the colour-1
// points of the tile from those, and writes the tile's points of both
// colours to x_new. The halo ring's colour-0 values are computed again by
// every tile that needs them, from the same old values, so every point gets
// exactly the value of the two in-place phases (k_relax_rb_quad with colour
// 0, then 1): same records, same operations, same order. Reading x_old and
// writing x_new keeps one tile's writes out of another tile's halo. With
// zero_x the sweep starts from x = 0 (the V-cycle's first sweep): x_old is
// not read. Each x value moves from L2 once per sweep instead of about five
// times per phase.
constexpr int kSwX = 64, kSwJ = 8, kSwK = 8;
constexpr int kSwXS = kSwX + 8;  // shared row: points i0 - 4 .. i0 + kSwX + 3 (16-byte loads)

// One colour phase of k_relax_rb_sweep on the shared tile: LINES lines of
// PER_LINE points of the colour, the lines starting FIRST lines into the
// tile's shared rows in j and k (1: the halo ring included; 2: the tile);
// colour 0 takes the records [0, h), colour 1 [h, 2h) (rec_base). A thread
// takes its points kSwChunk at a time: first the class codes and
// right-hand sides of the chunk (independent loads in flight together),
// then the relaxations from shared memory.
constexpr int kSwChunk = 4;
template <int LINES, int PER_LINE, int FIRST>
__device__ __forceinline__ void sweep_phase(const Recs<float, 8> &R, const float *__restrict__ b,
                                            float (*sx)[kSwJ + 4][kSwXS], const Box &bx, int i0, int j0, int k0,
                                            long rec_base) {
  constexpr int NI = (LINES * PER_LINE + kThreads - 1) / kThreads;
  constexpr int LW = kSwJ + 4 - 2 * FIRST;  // lines of the phase in j: kSwJ + 2 with the ring, kSwJ without
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const int colour = FIRST == 1 ? 0 : 1;
  const int istart = FIRST == 1 ? i0 - 1 : i0;
#pragma unroll 1
  for (int t0 = 0; t0 < NI; t0 += kSwChunk) {
    int rr[kSwChunk], li[kSwChunk], lj[kSwChunk], lk[kSwChunk];
    float bv[kSwChunk];
    unsigned short code[kSwChunk];
#pragma unroll
    for (int u = 0; u < kSwChunk; ++u) {
      const int e = threadIdx.x + (t0 + u) * kThreads;
      rr[u] = -1;
      if (t0 + u >= NI || e >= LINES * PER_LINE) continue;
      const int sidx = e % PER_LINE, line = e / PER_LINE;
      lj[u] = line % LW + FIRST;
      lk[u] = line / LW + FIRST;
      const int j = j0 - 2 + lj[u], k = k0 - 2 + lk[u];
      const int i = istart + ((istart + j + k + colour) & 1) + 2 * sidx;
      if (j < 0 || j >= ny || k < 0 || k >= nz || i < 0 || i >= nx || i > i0 + kSwX) continue;
      const int r = (k * ny + j) * nx + i;
      rr[u] = r;
      li[u] = i - i0 + 4;
      bv[u] = b[r];
      code[u] = R.code ? __ldcs(R.code + rec_base + (r >> 1)) : 0;
    }
#pragma unroll
    for (int u = 0; u < kSwChunk; ++u) {
      if (rr[u] < 0) continue;
      float c[8];
      if (R.code) {
        const float4 *qq = reinterpret_cast<const float4 *>(R.tab + 8 * (long)code[u]);
        const float4 p0 = __ldg(qq), p1 = __ldg(qq + 1);
        c[0] = p0.x; c[1] = p0.y; c[2] = p0.z; c[3] = p0.w; c[4] = p1.x; c[5] = p1.y; c[6] = p1.z; c[7] = p1.w;
      } else {
        load_rec<float, 8>(R.R + (rec_base + (rr[u] >> 1)) * 8, c);
      }
      const int a = lk[u], bj = lj[u], ci = li[u];
      float acc = 0.0f;
      acc = fmaf(c[1], sx[a][bj][ci - 1], acc);
      acc = fmaf(c[2], sx[a][bj][ci + 1], acc);
      acc = fmaf(c[3], sx[a][bj - 1][ci], acc);
      acc = fmaf(c[4], sx[a][bj + 1][ci], acc);
      acc = fmaf(c[5], sx[a - 1][bj][ci], acc);
      acc = fmaf(c[6], sx[a + 1][bj][ci], acc);
      sx[a][bj][ci] = c[0] * (bv[u] - acc);
    }
  }
}

__global__ void __launch_bounds__(kThreads, 3) k_relax_rb_sweep(Recs<float, 8> R, const float *__restrict__ b,
                                                             const float *__restrict__ xo, float *__restrict__ xn,
                                                             Box bx, int zero_x, const int *gate) {
  if (gate_off(gate)) return;
  __shared__ __align__(16) float sx[kSwK + 4][kSwJ + 4][kSwXS];
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const long h = bx.n / 2;
  const int tx = (nx + kSwX - 1) / kSwX, tyj = (ny + kSwJ - 1) / kSwJ, tzk = (nz + kSwK - 1) / kSwK;
  const long ntiles = (long)tx * tyj * tzk;
  for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int ti = (int)(tile % tx), tj = (int)((tile / tx) % tyj), tk = (int)(tile / ((long)tx * tyj));
    const int i0 = ti * kSwX, j0 = tj * kSwJ, k0 = tk * kSwK;
    // x_old over the tile and its halo; 0 outside the box (the stencil's zero)
    constexpr int nq = kSwXS / 4, nlines = (kSwK + 4) * (kSwJ + 4);
#pragma unroll 4
    for (int e = threadIdx.x; e < nlines * nq; e += blockDim.x) {
      const int q = e % nq, line = e / nq;
      const int lj = line % (kSwJ + 4), lk = line / (kSwJ + 4);
      const int j = j0 - 2 + lj, k = k0 - 2 + lk, gi = i0 - 4 + 4 * q;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (!zero_x && j >= 0 && j < ny && k >= 0 && k < nz && gi >= 0 && gi < nx)
        v = *reinterpret_cast<const float4 *>(xo + ((long)k * ny + j) * nx + gi);
      *reinterpret_cast<float4 *>(&sx[lk][lj][4 * q]) = v;
    }
    __syncthreads();
    // colour 0 over the tile and the one-line ring: lines j0-1 .. j0+kSwJ,
    // k0-1 .. k0+kSwK, points i0-1 .. i0+kSwX (kSwX/2 + 1 of each colour a
    // line); then colour 1 over the tile. Each thread first issues the class
    // codes and right-hand sides of all its points (independent loads in
    // flight together), then relaxes them from shared memory.
    sweep_phase<(kSwK + 2) * (kSwJ + 2), kSwX / 2 + 1, 1>(R, b, sx, bx, i0, j0, k0, 0L);
    __syncthreads();
    sweep_phase<kSwK * kSwJ, kSwX / 2, 2>(R, b, sx, bx, i0, j0, k0, h);
    __syncthreads();
    // the tile's points of both colours to x_new
    {
      constexpr int nq4 = kSwX / 4, lines = kSwK * kSwJ;
      for (int e = threadIdx.x; e < lines * nq4; e += blockDim.x) {
        const int q = e % nq4, line = e / nq4;
        const int lj = line % kSwJ + 2, lk = line / kSwJ + 2;
        const int j = j0 - 2 + lj, k = k0 - 2 + lk, gi = i0 + 4 * q;
        if (j >= ny || k >= nz || gi >= nx) continue;
        *reinterpret_cast<float4 *>(xn + ((long)k * ny + j) * nx + gi) =
            *reinterpret_cast<const float4 *>(&sx[lk][lj][4 + 4 * q]);
      }
    }
    __syncthreads();  // the shared tile is reused by the next tile
  }
}

// Residual after a sweep that ended with colour 1 (k_residual_rb), quartet
// form: colour-0 points b - A x in k_residual_rb's order, colour-1 points 0.
template <int P>
__device__ __forceinline__ void resid_quad(const float (&c)[2][8], const float4 &bq, const float4 &xc,
                                           const float4 &xs, const float4 &xn, const float4 &xb, const float4 &xt,
                                           float xl, float xr, float (&res)[4]) {
  const float cc[4] = {xc.x, xc.y, xc.z, xc.w}, ss[4] = {xs.x, xs.y, xs.z, xs.w}, nn[4] = {xn.x, xn.y, xn.z, xn.w};
  const float bo[4] = {xb.x, xb.y, xb.z, xb.w}, tt[4] = {xt.x, xt.y, xt.z, xt.w}, bb[4] = {bq.x, bq.y, bq.z, bq.w};
#pragma unroll
  for (int l = 0; l < 4; ++l) res[l] = 0.0f;
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const int l = P + 2 * t;
    const float xw = l == 0 ? xl : cc[l == 0 ? 0 : l - 1];
    const float xe = l == 3 ? xr : cc[l == 3 ? 3 : l + 1];
    float acc = 0.0f;
    acc = fmaf(c[t][7], cc[l], acc);
    acc = fmaf(c[t][1], xw, acc);
    acc = fmaf(c[t][2], xe, acc);
    acc = fmaf(c[t][3], ss[l], acc);
    acc = fmaf(c[t][4], nn[l], acc);
    acc = fmaf(c[t][5], bo[l], acc);
    acc = fmaf(c[t][6], tt[l], acc);
    res[l] = bb[l] - acc;
  }
}

__global__ void __launch_bounds__(kThreads) k_residual_rb_quad(Recs<float, 8> R, const float *__restrict__ b,
                                                               const float *__restrict__ x, float *__restrict__ res,
                                                               Box bx, const int *gate) {
  if (gate_off(gate)) return;
  const long n4 = bx.n / 4;
  const int nx = bx.nx, ny = bx.ny, nz = bx.nz;
  const long sy = nx, sz = (long)nx * ny;
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long)gridDim.x * blockDim.x) {
    const long r0 = 4 * q;
    const unsigned line = fast_div((unsigned)r0, bx.dx);
    const int i0 = (int)((unsigned)r0 - line * (unsigned)nx);
    const unsigned kk = fast_div(line, bx.dy);
    const int j = (int)(line - kk * (unsigned)ny), k = (int)kk;
    float c[2][8];
    load_quad_recs(R, r0 / 2, c);
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 bq = *reinterpret_cast<const float4 *>(b + r0);
    const float4 xc = *reinterpret_cast<const float4 *>(x + r0);
    const float4 xs = j > 0 ? *reinterpret_cast<const float4 *>(x + r0 - sy) : z4;
    const float4 xn = j < ny - 1 ? *reinterpret_cast<const float4 *>(x + r0 + sy) : z4;
    const float4 xb = k > 0 ? *reinterpret_cast<const float4 *>(x + r0 - sz) : z4;
    const float4 xt = k < nz - 1 ? *reinterpret_cast<const float4 *>(x + r0 + sz) : z4;
    const float xl = i0 > 0 ? x[r0 - 1] : 0.0f;
    const float xr = i0 + 4 < nx ? x[r0 + 4] : 0.0f;
    float rr[4];
    if (((j + k) & 1) == 0) resid_quad<0>(c, bq, xc, xs, xn, xb, xt, xl, xr, rr);
    else resid_quad<1>(c, bq, xc, xs, xn, xb, xt, xl, xr, rr);
    *reinterpret_cast<float4 *>(res + r0) = make_float4(rr[0], rr[1], rr[2], rr[3]);
  }
}

// First phase from a zero guess: colour-0 points take invd b, colour-1 points 0.
template <class T>
__global__ void k_relax_rb_zero(Recs<T, 8> R, const T *__restrict__ b, T *x, Box bx, const int *gate) {
  if (gate_off(gate)) return;
  const long h = bx.n / 2;
  for (long m = (long)blockIdx.x * blockDim.x + threadIdx.x; m < h; m += (long)gridDim.x * blockDim.x) {
    int i, j, k;
    const long r = rb_row(m, 0, bx, i, j, k);
    x[r] = rec_ptr<T, 8>(R, m)[0] * b[r];
    x[r ^ 1] = T(0);
  }
}

template <class T, int NS>
__global__ void k_residual(const T *A, const T *b, const T *x, T *res, Box bx, const int *gate) {
  if (gate_off(gate)) return;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < bx.n; r += (long)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(r, bx, i, j, k);
    res[r] = b[r] - apply_row<T, NS>(A, bx.n, x, (int)r, i, j, k, bx.nx, bx.ny, bx.nz);
  }
}

template <class T>
__device__ __forceinline__ void restrict_body(const T *res, const T *pm, const T *pp, const Box &fb, int d, T *bc,
                                              const Box &cb, long t0, long ts) {
  const int fn[3] = {fb.nx, fb.ny, fb.nz};
  for (long I = t0; I < cb.n; I += ts) {
    int ci[3];
    box_ijk(I, cb, ci[0], ci[1], ci[2]);
    T acc = T(0);
    for (int fo = -1; fo <= 1; ++fo) {
      int f[3] = {ci[0], ci[1], ci[2]};
      f[d] = 2 * ci[d] + fo;
      if (f[d] < 0 || f[d] >= fn[d]) continue;
      const long fr = ((long)f[2] * fb.ny + f[1]) * fb.nx + f[0];
      const T rw = fo == 0 ? T(1) : (fo < 0 ? pp[fr] : pm[fr]);
      acc = fmat<T>(rw, res[fr], acc);
    }
    bc[I] = acc;
  }
}
template <class T>
__global__ void k_restrict(const T *res, const T *pm, const T *pp, Box fb, int d, T *bc, Box cb, const int *gate) {
  if (gate_off(gate)) return;
  restrict_body<T>(res, pm, pp, fb, d, bc, cb, (long)blockIdx.x * blockDim.x + threadIdx.x,
                   (long)gridDim.x * blockDim.x);
}

// Restriction / interpolation along y or z on FP32 levels whose nx is a
// multiple of 4: four consecutive x points share everything but their x, so a
// thread moves them with 16-byte loads. Same operations as k_restrict /
// k_prolong, lane by lane.
__device__ __forceinline__ void restrict_yz4_body(const float *res, const float *pm, const float *pp, const Box &fb,
                                                  int d, float *bc, const Box &cb, long t0, long ts) {
  const long n4 = cb.n / 4;
  const long plane_f = (long)fb.nx * fb.ny;
  const int nfd = d == 1 ? fb.ny : fb.nz;
  for (long t = t0; t < n4; t += ts) {
    int i, J, k;
    box_ijk(4 * t, cb, i, J, k);
    const int cd = d == 1 ? J : k;
    // fine index of (i, 2cd + fo) along d
    auto fidx = [&](int fo) {
      const int y = d == 1 ? 2 * cd + fo : J, z = d == 2 ? 2 * cd + fo : k;
      return (long)z * plane_f + (long)y * fb.nx + i;
    };
    const bool lo = 2 * cd - 1 >= 0, hi = 2 * cd + 1 < nfd;
    const float4 rm = *reinterpret_cast<const float4 *>(res + fidx(0));
    float4 rl = make_float4(0.f, 0.f, 0.f, 0.f), rh = rl, wl = rl, wh = rl;
    if (lo) {
      rl = *reinterpret_cast<const float4 *>(res + fidx(-1));
      wl = *reinterpret_cast<const float4 *>(pp + fidx(-1));
    }
    if (hi) {
      rh = *reinterpret_cast<const float4 *>(res + fidx(1));
      wh = *reinterpret_cast<const float4 *>(pm + fidx(1));
    }
    auto one = [&](float a_rl, float a_wl, float a_rm, float a_rh, float a_wh) {
      float acc = 0.0f;
      if (lo) acc = fmaf(a_wl, a_rl, acc);
      acc = fmaf(1.0f, a_rm, acc);
      if (hi) acc = fmaf(a_wh, a_rh, acc);
      return acc;
    };
    float4 o;
    o.x = one(rl.x, wl.x, rm.x, rh.x, wh.x);
    o.y = one(rl.y, wl.y, rm.y, rh.y, wh.y);
    o.z = one(rl.z, wl.z, rm.z, rh.z, wh.z);
    o.w = one(rl.w, wl.w, rm.w, rh.w, wh.w);
    *reinterpret_cast<float4 *>(bc + 4 * t) = o;
  }
}
__global__ void k_restrict_yz4(const float *__restrict__ res, const float *__restrict__ pm,
                               const float *__restrict__ pp, Box fb, int d, float *__restrict__ bc, Box cb,
                               const int *gate) {
  if (gate_off(gate)) return;
  restrict_yz4_body(res, pm, pp, fb, d, bc, cb, (long)blockIdx.x * blockDim.x + threadIdx.x,
                    (long)gridDim.x * blockDim.x);
}

__device__ __forceinline__ void prolong_yz4_body(const float *xc, const Box &cb, const float *pm, const float *pp,
                                                 const Box &fb, int d, float *x, int accumulate, long t0, long ts) {
  const long n4 = fb.n / 4;
  const long plane_c = (long)cb.nx * cb.ny;
  const int ncd = d == 1 ? cb.ny : cb.nz;
  for (long t = t0; t < n4; t += ts) {
    int i, y, k;
    box_ijk(4 * t, fb, i, y, k);
    const int fd = d == 1 ? y : k;
    auto cidx = [&](int c) {
      const int yy = d == 1 ? c : y, zz = d == 2 ? c : k;
      return (long)zz * plane_c + (long)yy * cb.nx + i;
    };
    float4 corr;
    if ((fd & 1) == 0) {
      corr = *reinterpret_cast<const float4 *>(xc + cidx(fd / 2));
    } else {
      const float4 x0 = *reinterpret_cast<const float4 *>(xc + cidx((fd - 1) / 2));
      float4 x1 = make_float4(0.f, 0.f, 0.f, 0.f);
      if ((fd + 1) / 2 < ncd) x1 = *reinterpret_cast<const float4 *>(xc + cidx((fd + 1) / 2));
      const float4 a = *reinterpret_cast<const float4 *>(pp + 4 * t);
      const float4 b = *reinterpret_cast<const float4 *>(pm + 4 * t);
      corr.x = fmaf(a.x, x1.x, b.x * x0.x);
      corr.y = fmaf(a.y, x1.y, b.y * x0.y);
      corr.z = fmaf(a.z, x1.z, b.z * x0.z);
      corr.w = fmaf(a.w, x1.w, b.w * x0.w);
    }
    float4 *xo = reinterpret_cast<float4 *>(x + 4 * t);
    if (accumulate) {
      const float4 xv = *xo;
      corr.x = xv.x + corr.x; corr.y = xv.y + corr.y; corr.z = xv.z + corr.z; corr.w = xv.w + corr.w;
    }
    *xo = corr;
  }
}
__global__ void k_prolong_yz4(const float *__restrict__ xc, Box cb, const float *__restrict__ pm,
                              const float *__restrict__ pp, Box fb, int d, float *x, int accumulate,
                              const int *gate) {
  if (gate_off(gate)) return;
  prolong_yz4_body(xc, cb, pm, pp, fb, d, x, accumulate, (long)blockIdx.x * blockDim.x + threadIdx.x,
                   (long)gridDim.x * blockDim.x);
}

// Restriction / interpolation along x on FP32 levels with fine nx = 2 coarse
// nx and coarse nx a multiple of 4: a thread makes four coarse points from
// fine points 2i0 - 1 .. 2i0 + 7 (restriction), or four fine points from
// coarse points i0/2 .. i0/2 + 2 (interpolation), with 16-byte loads. Same
// operations as k_restrict / k_prolong, point by point.
__device__ __forceinline__ void restrict_x4_body(const float *res, const float *pm, const float *pp, const Box &fb,
                                                 float *bc, const Box &cb, long t0, long ts) {
  const long n4 = cb.n / 4;
  for (long t = t0; t < n4; t += ts) {
    const long c0 = 4 * t;
    const unsigned cline = fast_div((unsigned)c0, cb.dx);
    const int ci0 = (int)((unsigned)c0 - cline * (unsigned)cb.nx);
    const long f0 = (long)cline * fb.nx + 2 * ci0;  // fine point 2 ci0 of the same line
    float rv[9], wl[9], wh[9];  // fine points 2ci0 - 1 + e, e = 0..8
    {
      const float4 a = *reinterpret_cast<const float4 *>(res + f0), b4 = *reinterpret_cast<const float4 *>(res + f0 + 4);
      rv[1] = a.x; rv[2] = a.y; rv[3] = a.z; rv[4] = a.w; rv[5] = b4.x; rv[6] = b4.y; rv[7] = b4.z; rv[8] = b4.w;
      const float4 p1 = *reinterpret_cast<const float4 *>(pp + f0), p2 = *reinterpret_cast<const float4 *>(pp + f0 + 4);
      wl[1] = p1.x; wl[2] = p1.y; wl[3] = p1.z; wl[4] = p1.w; wl[5] = p2.x; wl[6] = p2.y; wl[7] = p2.z; wl[8] = p2.w;
      const float4 m1 = *reinterpret_cast<const float4 *>(pm + f0), m2 = *reinterpret_cast<const float4 *>(pm + f0 + 4);
      wh[1] = m1.x; wh[2] = m1.y; wh[3] = m1.z; wh[4] = m1.w; wh[5] = m2.x; wh[6] = m2.y; wh[7] = m2.z; wh[8] = m2.w;
      const bool lo = ci0 > 0;
      rv[0] = lo ? res[f0 - 1] : 0.0f;
      wl[0] = lo ? pp[f0 - 1] : 0.0f;
      wh[0] = 0.0f;
    }
    float o[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      // coarse point ci0 + u: fine 2(ci0 + u) - 1, 2(ci0 + u), 2(ci0 + u) + 1 = rv[2u], rv[2u + 1], rv[2u + 2]
      float acc = 0.0f;
      if (ci0 + u > 0) acc = fmaf(wl[2 * u], rv[2 * u], acc);
      acc = fmaf(1.0f, rv[2 * u + 1], acc);
      acc = fmaf(wh[2 * u + 2], rv[2 * u + 2], acc);  // 2(ci0 + u) + 1 < fine nx always
      o[u] = acc;
    }
    *reinterpret_cast<float4 *>(bc + c0) = make_float4(o[0], o[1], o[2], o[3]);
  }
}
__global__ void k_restrict_x4(const float *__restrict__ res, const float *__restrict__ pm,
                              const float *__restrict__ pp, Box fb, float *__restrict__ bc, Box cb, const int *gate) {
  if (gate_off(gate)) return;
  restrict_x4_body(res, pm, pp, fb, bc, cb, (long)blockIdx.x * blockDim.x + threadIdx.x,
                   (long)gridDim.x * blockDim.x);
}

__device__ __forceinline__ void prolong_x4_body(const float *xc, const Box &cb, const float *pm, const float *pp,
                                                const Box &fb, float *x, int accumulate, long t0, long ts) {
  const long n4 = fb.n / 4;
  for (long t = t0; t < n4; t += ts) {
    const long r0 = 4 * t;
    const unsigned line = fast_div((unsigned)r0, fb.dx);
    const int i0 = (int)((unsigned)r0 - line * (unsigned)fb.nx);
    const long cc = (long)line * cb.nx + i0 / 2;  // coarse point i0 / 2 of the same line
    const float2 c01 = *reinterpret_cast<const float2 *>(xc + cc);
    const float c2 = i0 / 2 + 2 < cb.nx ? xc[cc + 2] : 0.0f;
    const float4 a = *reinterpret_cast<const float4 *>(pp + r0), m = *reinterpret_cast<const float4 *>(pm + r0);
    // fine i0 + 0: even -> c0; i0 + 1: odd between c0, c1; i0 + 2: c1; i0 + 3: between c1, c2
    float4 corr;
    corr.x = c01.x;
    corr.y = fmaf(a.y, c01.y, m.y * c01.x);
    corr.z = c01.y;
    corr.w = fmaf(a.w, c2, m.w * c01.y);
    float4 *xo = reinterpret_cast<float4 *>(x + r0);
    if (accumulate) {
      const float4 xv = *xo;
      corr.x = xv.x + corr.x; corr.y = xv.y + corr.y; corr.z = xv.z + corr.z; corr.w = xv.w + corr.w;
    }
    *xo = corr;
  }
}
__global__ void k_prolong_x4(const float *__restrict__ xc, Box cb, const float *__restrict__ pm,
                             const float *__restrict__ pp, Box fb, float *x, int accumulate, const int *gate) {
  if (gate_off(gate)) return;
  prolong_x4_body(xc, cb, pm, pp, fb, x, accumulate, (long)blockIdx.x * blockDim.x + threadIdx.x,
                  (long)gridDim.x * blockDim.x);
}

template <class T>
__device__ __forceinline__ void prolong_body(const T *xc, const Box &cb, const T *pm, const T *pp, const Box &fb,
                                             int d, T *x, int accumulate, long t0, long ts) {
  const int cn[3] = {cb.nx, cb.ny, cb.nz};
  for (long r = t0; r < fb.n; r += ts) {
    int f[3];
    box_ijk(r, fb, f[0], f[1], f[2]);
    T corr;
    if ((f[d] & 1) == 0) {
      int c[3] = {f[0], f[1], f[2]};
      c[d] = f[d] / 2;
      corr = xc[((long)c[2] * cb.ny + c[1]) * cb.nx + c[0]];
    } else {
      int c0[3] = {f[0], f[1], f[2]};
      c0[d] = (f[d] - 1) / 2;
      const T x0 = xc[((long)c0[2] * cb.ny + c0[1]) * cb.nx + c0[0]];
      T x1 = T(0);
      if ((f[d] + 1) / 2 < cn[d]) {
        int c1[3] = {f[0], f[1], f[2]};
        c1[d] = (f[d] + 1) / 2;
        x1 = xc[((long)c1[2] * cb.ny + c1[1]) * cb.nx + c1[0]];
      }
      corr = fmat<T>(pp[r], x1, pm[r] * x0);
    }
    x[r] = accumulate ? x[r] + corr : corr;
  }
}
template <class T>
__global__ void k_prolong(const T *xc, Box cb, const T *pm, const T *pp, Box fb, int d, T *x, int accumulate,
                          const int *gate) {
  if (gate_off(gate)) return;
  prolong_body<T>(xc, cb, pm, pp, fb, d, x, accumulate, (long)blockIdx.x * blockDim.x + threadIdx.x,
                  (long)gridDim.x * blockDim.x);
}

// Coarsest level: x = Ainv b (one warp per row).
// Coarsest level: x = A^-1 b, one warp per row. FP64 hierarchies accumulate
// in FP64; FP32 ones in FP32 per lane (n / 32 products each) and FP64 across
// the warp, so a dense level of a few thousand points does not wait on the
// FP64 pipe.
template <class T>
__device__ __forceinline__ void dense_body(const T *Ainv, const T *b, T *x, int n, long t0, long ts) {
  const int warp = (int)(t0 >> 5), lane = threadIdx.x & 31;
  const int nw = (int)(ts >> 5);
  for (int r = warp; r < n; r += nw) {
    double acc;
    if constexpr (sizeof(T) == 4) {
      float a = 0.0f;
      if (n % 128 == 0) {
        // 16-byte loads: lane l takes columns 4l .. 4l+3 of every 128
        const float4 *row = reinterpret_cast<const float4 *>(Ainv + (long)r * n);
        const float4 *bb = reinterpret_cast<const float4 *>(b);
        for (int c = lane; c < n / 4; c += 32) {
          const float4 m = row[c], v = bb[c];
          a = fmaf(m.x, v.x, a);
          a = fmaf(m.y, v.y, a);
          a = fmaf(m.z, v.z, a);
          a = fmaf(m.w, v.w, a);
        }
      } else {
        for (int c = lane; c < n; c += 32) a = fmaf(Ainv[(long)r * n + c], b[c], a);
      }
      acc = (double)a;
    } else {
      acc = 0.0;
      for (int c = lane; c < n; c += 32) acc = fma(Ainv[(long)r * n + c], b[c], acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) x[r] = (T)acc;
  }
}
template <class T>
__global__ void k_dense(const T *Ainv, const T *b, T *x, int n, const int *gate) {
  if (gate_off(gate)) return;
  dense_body<T>(Ainv, b, x, n, (long)blockIdx.x * blockDim.x + threadIdx.x, (long)gridDim.x * blockDim.x);
}

// ---------------------------------------------------------------------------
// Fused coarse levels. Below the finest level every phase of the V-cycle
// (restrictions, two-colour 27-point sweeps, residuals, the dense coarsest
// solve, interpolations) runs in one persistent cooperative kernel: its blocks
// run the phases of a precomputed list in order, each over all its points
// (the same per-point arithmetic as the stand-alone kernels, through the
// shared bodies above), with a grid-wide barrier between phases. On the
// 640x128x128 channel that replaces about 50 launches per V-cycle whose work
// is a few microseconds each. Data written by one phase is read by the next
// with ordinary (coherent) loads: the phase list is the only read-only input.
// ---------------------------------------------------------------------------
enum TailKind : int {
  TK_RELAX27Q = 0, TK_RELAX27, TK_RESID27Q, TK_RESID27, TK_RESTRICT, TK_RESTRICT_YZ4, TK_RESTRICT_X4, TK_PROLONG,
  TK_PROLONG_YZ4, TK_PROLONG_X4, TK_DENSE
};

struct TailOp {
  int kind = 0, color = 0, zero = 0, d = 0, accumulate = 0, n = 0;
  Box fb, cb;               // the level (fine box) and, for transfers, the coarse box
  Recs<float, 28> R;        // colour-split records of a relaxed level
  const float *a = nullptr;   // right-hand side (sweeps, residuals) or the dense inverse
  const float *src = nullptr; // x read (sweeps, residuals), residual (restriction), coarse x (interpolation)
  const float *pm = nullptr, *pp = nullptr;  // interpolation weights
  float *dst = nullptr;
};

// Barrier state, cleared before every launch: blocks arrived at the current
// barrier, the barrier's generation, and an error flag set when a block gave
// up waiting.
struct TailBar {
  unsigned arrived, gen, err, pad;
};

// A cooperative launch keeps every block resident, so each barrier completes
// once all blocks reach it; the bound only keeps a fault elsewhere from
// turning into an endless wait (about a second of polling).
constexpr unsigned kTailSpin = 1u << 21;

// Grid-wide barrier; returns true when the error flag is set (a block timed
// out), after which the blocks stop.
__device__ __forceinline__ bool tail_sync(TailBar *tb, unsigned &gen) {
  __shared__ int s_err;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned g = gen;
    __threadfence();  // this block's writes before the arrival
    if (atomicAdd(&tb->arrived, 1u) == gridDim.x - 1) {
      atomicExch(&tb->arrived, 0u);
      __threadfence();
      atomicExch(&tb->gen, g + 1);
    } else {
      unsigned it = 0;
      while (*reinterpret_cast<volatile unsigned *>(&tb->gen) == g) {
        if (++it > kTailSpin) {
          atomicExch(&tb->err, 1u);
          break;
        }
        __nanosleep(40);
      }
    }
    gen = g + 1;
    __threadfence();  // the other blocks' writes after the barrier
    s_err = *reinterpret_cast<volatile unsigned *>(&tb->err) != 0u;
  }
  __syncthreads();
  return s_err != 0;
}

__global__ void __launch_bounds__(kThreads) k_mg_tail(const TailOp *__restrict__ ops, int nops, TailBar *tb,
                                                      float *out, const int *gate) {
  if (gate_off(gate)) return;
  const long t0 = (long)blockIdx.x * blockDim.x + threadIdx.x, ts = (long)gridDim.x * blockDim.x;
  unsigned gen = 0;
  for (int o = 0; o < nops; ++o) {
    const TailOp op = ops[o];
    switch (op.kind) {
      case TK_RELAX27Q: relax_rb27_quad_body(op.R, op.a, op.src, op.dst, op.fb, op.color, op.zero, t0, ts); break;
      case TK_RELAX27: relax_rb27_body<float>(op.R, op.a, op.src, op.dst, op.fb, op.color, op.zero, t0, ts); break;
      case TK_RESID27Q: residual_rb27_quad_body(op.R, op.a, op.src, op.dst, op.fb, t0, ts); break;
      case TK_RESID27: residual_rb27_body<float>(op.R, op.a, op.src, op.dst, op.fb, t0, ts); break;
      case TK_RESTRICT: restrict_body<float>(op.src, op.pm, op.pp, op.fb, op.d, op.dst, op.cb, t0, ts); break;
      case TK_RESTRICT_YZ4: restrict_yz4_body(op.src, op.pm, op.pp, op.fb, op.d, op.dst, op.cb, t0, ts); break;
      case TK_RESTRICT_X4: restrict_x4_body(op.src, op.pm, op.pp, op.fb, op.dst, op.cb, t0, ts); break;
      case TK_PROLONG:
        prolong_body<float>(op.src, op.cb, op.pm, op.pp, op.fb, op.d, op.dst, op.accumulate, t0, ts);
        break;
      case TK_PROLONG_YZ4:
        prolong_yz4_body(op.src, op.cb, op.pm, op.pp, op.fb, op.d, op.dst, op.accumulate, t0, ts);
        break;
      case TK_PROLONG_X4: prolong_x4_body(op.src, op.cb, op.pm, op.pp, op.fb, op.dst, op.accumulate, t0, ts); break;
      case TK_DENSE: dense_body<float>(op.a, op.src, op.dst, op.n, t0, ts); break;
      default: break;
    }
    if (o + 1 < nops && tail_sync(tb, gen)) {
      // a block timed out: stop, and make the result non-finite so the
      // solver reports it (IBM_ERR_NONFINITE) instead of using it
      if (blockIdx.x == 0 && threadIdx.x == 0) out[0] = __int_as_float(0x7fc00000);
      return;
    }
  }
}

int grid_for(long n) {
  long b = (n + kThreads - 1) / kThreads;
  const long cap = (long)sm_count() * 8;
  if (b > cap) b = cap;
  return (int)std::max(1L, b);
}

// One thread per element for the V-cycle's streaming kernels: every block
// retires after one element per thread, so the GPU keeps many independent
// loads in flight without a serial loop per thread.
int grid_all(long n) { return (int)std::max(1L, std::min((n + kThreads - 1) / kThreads, 1L << 30)); }

// Blocks for a grid-stride kernel over n items: one per kThreads items, at
// most as many as stay resident (one wave). A resident grid loops over its
// items instead of launching a block per kThreads of them: measured on the
// finest phase at 640x128x128, 35 us with a block per item group, 29 us with
// four blocks per SM.
template <class K>
int resident_grid(K kernel, long n) {
  static std::mutex mu;
  static std::unordered_map<const void *, int> cache;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find((const void *)kernel);
    if (it != cache.end()) per_sm = it->second;
  }
  if (per_sm == 0) {
    IBM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0));
    per_sm = std::max(1, per_sm);
    std::lock_guard<std::mutex> lock(mu);
    cache[(const void *)kernel] = per_sm;
  }
  return (int)std::min<long>(grid_all(n), (long)per_sm * sm_count());
}

// Blocks of k_relax_rb_sweep: one tile each, at most as many as stay resident.
int sweep_grid(const Box &b) {
  static int per_sm = 0;
  if (per_sm == 0) {
    IBM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_relax_rb_sweep, kThreads, 0));
    per_sm = std::max(1, per_sm);
  }
  const long tiles = (long)((b.nx + kSwX - 1) / kSwX) * ((b.ny + kSwJ - 1) / kSwJ) * ((b.nz + kSwK - 1) / kSwK);
  return (int)std::max(1L, std::min(tiles, (long)per_sm * sm_count()));
}

// Gauss-Jordan inverse with partial pivoting of the assembled coarsest operator.
void dense_inverse(const std::vector<double> &A, int ns, const Box &b, std::vector<double> &inv) {
  const long n = b.n;
  std::vector<double> M((size_t)(n * n), 0.0);
  for (long r = 0; r < n; ++r) {
    const int i = (int)(r % b.nx), j = (int)((r / b.nx) % b.ny), k = (int)(r / ((long)b.nx * b.ny));
    for (int s = 0; s < 27; ++s) {
      int q = -1;
      if (ns == 27) q = s;
      else {
        static const int map[27] = {-1, -1, -1, -1, 5, -1, -1, -1, -1, -1, 3, -1, 1, 0, 2, -1, 4, -1,
                                    -1, -1, -1, -1, 6, -1, -1, -1, -1};
        q = map[s];
      }
      if (q < 0) continue;
      const int ii = i + s27_off(s, 0), jj = j + s27_off(s, 1), kk = k + s27_off(s, 2);
      if (ii < 0 || ii >= b.nx || jj < 0 || jj >= b.ny || kk < 0 || kk >= b.nz) continue;
      M[(size_t)(r * n + ((long)kk * b.ny + jj) * b.nx + ii)] += A[(size_t)q * n + r];
    }
  }
  inv.assign((size_t)(n * n), 0.0);
  for (long r = 0; r < n; ++r) inv[(size_t)(r * n + r)] = 1.0;
  for (long c = 0; c < n; ++c) {
    long piv = c;
    for (long r = c + 1; r < n; ++r)
      if (std::fabs(M[(size_t)(r * n + c)]) > std::fabs(M[(size_t)(piv * n + c)])) piv = r;
    if (piv != c)
      for (long t = 0; t < n; ++t) {
        std::swap(M[(size_t)(c * n + t)], M[(size_t)(piv * n + t)]);
        std::swap(inv[(size_t)(c * n + t)], inv[(size_t)(piv * n + t)]);
      }
    const double pv = M[(size_t)(c * n + c)];
    if (pv == 0.0) continue;
    const double ip = 1.0 / pv;
    for (long t = 0; t < n; ++t) { M[(size_t)(c * n + t)] *= ip; inv[(size_t)(c * n + t)] *= ip; }
    for (long r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = M[(size_t)(r * n + c)];
      if (f == 0.0) continue;
      for (long t = 0; t < n; ++t) {
        M[(size_t)(r * n + t)] -= f * M[(size_t)(c * n + t)];
        inv[(size_t)(r * n + t)] -= f * inv[(size_t)(c * n + t)];
      }
    }
  }
}

}  // namespace

// ---------------------------------------------------------------- host side
// Colour-split copy of a relaxed 7-point level with an even nx (the fine
// level), used by the in-place two-colour relaxation.
// With record classes on, the records are replaced by their classes when
// there are at most kMaxClasses distinct ones.
template <class T>
static void split_colors(cudaStream_t st, MgLevelT<T> &F, const MgParams &prm) {
  if (prm.relax != 2 || (F.b.nx & 1) || F.b.n < 2) return;
  DBuf<T> &R = F.ns == 7 ? F.rb : F.rb27;
  const int W = F.ns == 7 ? 8 : 28;
  R.alloc((size_t)W * F.b.n);
  {
    LaunchScope ls(K_SETUP, st, 0.0);
    if (F.ns == 7) k_split_colors<T><<<grid_for(F.b.n), kThreads, 0, st>>>(F.A, F.invd.p, F.b, R.p);
    else k_split_colors27<T><<<grid_for(F.b.n), kThreads, 0, st>>>(F.A, F.invd.p, F.b, R.p);
  }
  if (prm.classes && build_classes<T>(st, R.p, W, F.b.n, F.rbc)) R.release();
}

template <class T, int W>
static Recs<T, W> recs_of(const DBuf<T> &plain, const Classes<T> &c) {
  Recs<T, W> r;
  if (c.ok() && c.W == W) { r.code = c.code.p; r.tab = c.tab.p; }
  else r.R = plain.p;
  return r;
}

template <>
void Multigrid::build<double>(cudaStream_t st, std::vector<MgLevelT<double>> &L, const Box &b0, const double *A7,
                              const double h0[3]) {
  L.clear();
  L.reserve(64);
  L.emplace_back();
  L[0].b = b0;
  L[0].ns = 7;
  L[0].A = A7;
  if (winv_) {
    L[0].Aown.alloc((size_t)7 * b0.n);
    {
      LaunchScope ls(K_SETUP, st, 0.0);
      k_scale_rows<<<grid_for(7 * b0.n), kThreads, 0, st>>>(A7, winv_, b0.n, L[0].Aown.p);
    }
    L[0].A = L[0].Aown.p;
  }
  const int aware = prm.options & 1;
  DBuf<unsigned char> coupled;
  double h[3] = {h0[0], h0[1], h0[2]};
  int queue[3], nq = 0;  // directions still to coarsen in the current group
  for (int l = 0;; ++l) {
    MgLevelT<double> &F = L[l];
    const long n = F.b.n;
    F.wd.alloc(n); F.invd.alloc(n); F.x.alloc(n); F.bv.alloc(n); F.r.alloc(n); F.t.alloc(n);
    // diagonal: plane 0 of a 7-point level, plane 13 of a 27-point level
    const double *diag = F.A + (F.ns == 27 ? 13L * n : 0L);
    {
      LaunchScope ls(K_SETUP, st, 0.0);
      k_diag<<<grid_for(n), kThreads, 0, st>>>(diag, n, prm.omega, F.invd.p, F.wd.p);
    }
    split_colors(st, F, prm);
    const int dims[3] = {F.b.nx, F.b.ny, F.b.nz};
    // A group starts at a relaxed level: every direction whose spacing is
    // within group_ratio of the smallest is coarsened once (smallest spacing
    // first); levels inside the group are not relaxed.
    F.relax = (nq == 0);
    if (nq == 0) {
      double hmin = 0.0;
      bool any = false;
      for (int dd = 0; dd < 3; ++dd)
        if (dims[dd] > 1 && (!any || h[dd] < hmin)) { hmin = h[dd]; any = true; }
      int cand[3], nc = 0;
      for (int dd = 0; dd < 3; ++dd)
        if (dims[dd] > 1 && (h[dd] == hmin || (prm.group_ratio > 0.0 && h[dd] <= prm.group_ratio * hmin)))
          cand[nc++] = dd;
      for (int a = 0; a < nc; ++a)
        for (int b2 = a + 1; b2 < nc; ++b2)
          if (h[cand[b2]] < h[cand[a]]) std::swap(cand[a], cand[b2]);
      if (prm.group_ratio <= 0.0 && nc > 1) nc = 1;
      for (int a = 0; a < nc; ++a) queue[a] = cand[nc - 1 - a];
      nq = nc;
    }
    int d = -1;
    while (nq > 0 && d < 0) {
      const int q = queue[--nq];
      if (dims[q] > 1) d = q;
    }
    if (n <= prm.coarse_max || l + 1 >= prm.max_levels || d < 0 || l + 1 >= 60) {
      F.cdir = -1;
      F.relax = 1;
      if (n > 4096) throw Error(IBM_ERR_ARG, "multigrid coarsest level too large for the dense solve");
      std::vector<double> hostA((size_t)F.ns * n), inv;
      IBM_CUDA_TRY(cudaMemcpyAsync(hostA.data(), F.A, sizeof(double) * hostA.size(), cudaMemcpyDeviceToHost, st));
      IBM_CUDA_TRY(cudaStreamSynchronize(st));
      dense_inverse(hostA, F.ns, F.b, inv);
      F.dense.alloc(inv.size());
      IBM_CUDA_TRY(cudaMemcpyAsync(F.dense.p, inv.data(), sizeof(double) * inv.size(), cudaMemcpyHostToDevice, st));
      IBM_CUDA_TRY(cudaStreamSynchronize(st));
      break;
    }
    F.cdir = d;
    h[d] *= 2.0;
    F.pm.alloc(n); F.pp.alloc(n);
    coupled.alloc(n);
    {
      LaunchScope ls(K_SETUP, st, 0.0);
      k_coupled<<<grid_for(n), kThreads, 0, st>>>(F.A, F.ns, n, coupled.p);
      k_interp_weights<<<grid_for(n), kThreads, 0, st>>>(F.A, F.ns, F.b, d, coupled.p, aware, F.pm.p, F.pp.p);
    }
    const Box cb = make_box(d == 0 ? (F.b.nx + 1) / 2 : F.b.nx, d == 1 ? (F.b.ny + 1) / 2 : F.b.ny,
                            d == 2 ? (F.b.nz + 1) / 2 : F.b.nz);
    L.emplace_back();
    MgLevelT<double> &Fr = L[l];  // re-fetch after emplace
    MgLevelT<double> &C = L[l + 1];
    C.b = cb;
    DBuf<double> a27;
    a27.alloc((size_t)27 * cb.n);
    {
      LaunchScope ls(K_SETUP, st, 0.0);
      k_rap<<<grid_for(cb.n), kThreads, 0, st>>>(Fr.A, Fr.ns, Fr.b, Fr.pm.p, Fr.pp.p, d, cb, a27.p);
    }
    if (prm.rap == 1) {
      C.Aown.alloc((size_t)7 * cb.n);
      DBuf<unsigned char> ccoupled;
      ccoupled.alloc(cb.n);
      {
        LaunchScope ls(K_SETUP, st, 0.0);
        k_coupled<<<grid_for(cb.n), kThreads, 0, st>>>(a27.p, 27, cb.n, ccoupled.p);
        k_collapse7<<<grid_for(cb.n), kThreads, 0, st>>>(a27.p, cb, ccoupled.p, aware, C.Aown.p);
      }
      IBM_CUDA_TRY(cudaStreamSynchronize(st));
      C.ns = 7;
    } else {
      C.Aown = std::move(a27);
      C.ns = 27;
    }
    C.A = C.Aown.p;
  }
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
  IBM_CUDA_TRY(cudaGetLastError());
}

static float *record_tail(std::vector<MgLevelT<float>> &L, int l, const MgParams &p, std::vector<TailOp> &ops,
                          double &bytes);

void Multigrid::setup(cudaStream_t st, const Box &b, const double *A7, const float *A7f, const double h[3],
                      const MgParams &p, bool fp64, bool fp32, const double *winv) {
  prm = p;
  winv_ = winv;
  winvf_.release();
  if (winv) {
    winvf_.alloc(b.n);
    LaunchScope ls(K_SETUP, st, 0.0);
    k_convert<float><<<grid_for(b.n), kThreads, 0, st>>>(winv, winvf_.p, b.n);
  }
  (void)fp64;
  build<double>(st, L64, b, A7, h);
  L32.clear();
  if (fp32) {
    L32.reserve(L64.size());
    for (size_t l = 0; l < L64.size(); ++l) {
      const MgLevelT<double> &D = L64[l];
      L32.emplace_back();
      MgLevelT<float> &F = L32.back();
      F.b = D.b; F.cdir = D.cdir; F.ns = D.ns; F.relax = D.relax;
      const long n = D.b.n;
      if (l == 0 && !winv_) F.A = A7f;
      else {
        F.Aown.alloc((size_t)D.ns * n);
        {
          LaunchScope ls(K_SETUP, st, 0.0);
          k_convert<float><<<grid_for((long)D.ns * n), kThreads, 0, st>>>(D.A, F.Aown.p, (long)D.ns * n);
        }
        F.A = F.Aown.p;
      }
      auto conv = [&](const DBuf<double> &src, DBuf<float> &dst) {
        if (!src.p) return;
        dst.alloc(src.n);
        {
          LaunchScope ls(K_SETUP, st, 0.0);
          k_convert<float><<<grid_for((long)src.n), kThreads, 0, st>>>(src.p, dst.p, (long)src.n);
        }
      };
      conv(D.wd, F.wd); conv(D.invd, F.invd); conv(D.pm, F.pm); conv(D.pp, F.pp); conv(D.dense, F.dense);
      split_colors(st, F, prm);
      F.x.alloc(n); F.bv.alloc(n); F.r.alloc(n); F.t.alloc(n);
    }
    IBM_CUDA_TRY(cudaStreamSynchronize(st));
  }
  build_tail(st);
}

void Multigrid::build_tail(cudaStream_t st) {
  tail_nops_ = 0;
  tail_ops_.release();
  tail_bar_.release();
  if (prm.fused_coarse <= 0 || prm.relax != 2 || L32.size() < 2 || L32[0].cdir < 0) return;
  // the first level below the finest that is small enough: its phases (and
  // the coarser ones') are bound by launch latency, not by their work
  int lt = 1;
  while (lt < (int)L32.size() && L32[lt].b.n > prm.fused_coarse) ++lt;
  if (lt >= (int)L32.size()) return;
  std::vector<TailOp> ops;
  double bytes = 0.0;
  float *out = record_tail(L32, lt, prm, ops, bytes);
  if (!out || ops.empty()) return;
  int per_sm = 0;
  IBM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mg_tail, kThreads, 0));
  if (per_sm < 1) return;
  tail_blocks_ = std::min(per_sm, 2) * sm_count();
  tail_ops_.alloc(sizeof(TailOp) * ops.size());
  IBM_CUDA_TRY(cudaMemcpyAsync(tail_ops_.p, ops.data(), sizeof(TailOp) * ops.size(), cudaMemcpyHostToDevice, st));
  tail_bar_.alloc(sizeof(TailBar) / sizeof(unsigned));
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
  tail_nops_ = (int)ops.size();
  tail_level_ = lt;
  tail_out_ = out;
  tail_bytes_ = bytes;
}

// Runs the V-cycle from level l with zero initial guess; returns (through the
// level's x buffer pointer swap-free scheme) the buffer holding the result.
// The fused coarse levels of an FP32 hierarchy, ready to launch.
struct TailLaunch {
  const TailOp *ops = nullptr;
  int nops = 0, blocks = 0, level = 1;  // the first fused level
  TailBar *bar = nullptr;
  float *out = nullptr;
  double bytes = 0.0;
};

// Records the V-cycle from level l (>= 1) of an FP32 hierarchy as phases of
// k_mg_tail, in the order and with the buffers vcycle() below would launch
// them, adding each phase's algorithmic bytes (vcycle's accounting) to
// `bytes`. Returns the buffer that holds level l's result, or nullptr when a
// level needs a phase the fused kernel does not have (7-point or Jacobi
// relaxation): the hierarchy then keeps one launch per phase.
static float *record_tail(std::vector<MgLevelT<float>> &L, int l, const MgParams &p, std::vector<TailOp> &ops,
                          double &bytes) {
  MgLevelT<float> &F = L[l];
  const long n = F.b.n;
  const double T_ = 4.0;
  if (F.cdir < 0) {
    TailOp op;
    op.kind = TK_DENSE;
    op.a = F.dense.p; op.src = F.bv.p; op.dst = F.x.p; op.n = (int)n; op.fb = F.b;
    ops.push_back(op);
    bytes += T_ * ((double)n * n + 2.0 * n);
    return F.x.p;
  }
  const int c1 = (l > 0 && p.nu_coarse > 0) ? p.nu_coarse : p.nu1, c2 = (l > 0 && p.nu_coarse > 0) ? p.nu_coarse : p.nu2;
  const int nu1 = F.relax ? c1 : 0, nu2 = F.relax ? c2 : 0;
  const Recs<float, 28> R27 = recs_of<float, 28>(F.rb27, F.rbc);
  const bool rb27 = R27.R || R27.code;
  if ((nu1 > 0 || nu2 > 0) && !(p.relax == 2 && rb27 && F.ns == 27)) return nullptr;
  const double rec27 = R27.code ? 2.0 : 28.0 * T_;
  const bool quad = p.quads && F.b.nx % 4 == 0;
  float *cur = F.x.p, *oth = F.t.p;
  auto relax = [&](bool zero) {
    for (int color = 0; color < 2; ++color) {
      const bool z = zero && color == 0;
      TailOp op;
      op.kind = quad ? TK_RELAX27Q : TK_RELAX27;
      op.R = R27; op.a = F.bv.p; op.src = cur; op.dst = oth; op.fb = F.b; op.color = color; op.zero = z;
      ops.push_back(op);
      bytes += z ? 0.5 * n * (R27.code ? 2.0 : T_) + 1.5 * T_ * n : 0.5 * n * rec27 + 2.5 * T_ * n;
      std::swap(cur, oth);
    }
  };
  for (int s = 0; s < nu1; ++s) relax(s == 0);
  const float *res = F.bv.p;
  if (nu1 > 0) {
    TailOp op;
    op.kind = quad ? TK_RESID27Q : TK_RESID27;
    op.R = R27; op.a = F.bv.p; op.src = cur; op.dst = F.r.p; op.fb = F.b;
    ops.push_back(op);
    bytes += n * rec27 + 3.0 * T_ * n;
    res = F.r.p;
  }
  MgLevelT<float> &C = L[l + 1];
  const bool yz4 = F.cdir != 0 && F.b.nx % 4 == 0;
  const bool x4 = !yz4 && p.quads && F.cdir == 0 && F.b.nx == 2 * C.b.nx && C.b.nx % 4 == 0;
  {
    TailOp op;
    op.kind = yz4 ? TK_RESTRICT_YZ4 : x4 ? TK_RESTRICT_X4 : TK_RESTRICT;
    op.src = res; op.pm = F.pm.p; op.pp = F.pp.p; op.fb = F.b; op.d = F.cdir; op.dst = C.bv.p; op.cb = C.b;
    ops.push_back(op);
    bytes += T_ * (3.0 * n + C.b.n);
  }
  float *xc = record_tail(L, l + 1, p, ops, bytes);
  if (!xc) return nullptr;
  {
    TailOp op;
    op.kind = yz4 ? TK_PROLONG_YZ4 : x4 ? TK_PROLONG_X4 : TK_PROLONG;
    op.src = xc; op.cb = C.b; op.pm = F.pm.p; op.pp = F.pp.p; op.fb = F.b; op.d = F.cdir; op.dst = cur;
    op.accumulate = nu1 > 0;
    ops.push_back(op);
    bytes += T_ * ((nu1 > 0 ? 4.0 : 3.0) * n + C.b.n);
  }
  for (int s = 0; s < nu2; ++s) relax(false);
  return cur;
}

// One cooperative launch of the fused coarse levels (a memset clears the
// barrier state first); returns the buffer holding the first fused level's
// correction.
static float *launch_tail(cudaStream_t st, const TailLaunch &t, const int *gate) {
  IBM_CUDA_TRY(cudaMemsetAsync(t.bar, 0, sizeof(TailBar), st));
  LaunchScope ls(K_MG_COARSE, st, t.bytes);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)t.blocks);
  cfg.blockDim = dim3(kThreads);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  IBM_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_mg_tail, t.ops, t.nops, t.bar, t.out, gate));
  return t.out;
}

template <class T>
// fin / fout (finest level only, may be null): the V-cycle's input load and
// output store, fused into the first and the last relaxation phases.
// tail (FP32 hierarchies, may be null): the levels from tail->level on run as
// the fused coarse kernel instead of one launch per phase.
static T *vcycle(cudaStream_t st, std::vector<MgLevelT<T>> &L, int l, const MgParams &p, const int *gate,
                 const VecRef *fin = nullptr, const OutRef *fout = nullptr, const float *winvf = nullptr,
                 const TailLaunch *tail = nullptr) {
  MgLevelT<T> &F = L[l];
  const long n = F.b.n;
  const double T_ = sizeof(T);
  const int g = grid_for(n);
  if (F.cdir < 0) {
    LaunchScope ls(K_MG_DENSE, st, T_ * ((double)n * n + 2.0 * n));
    k_dense<T><<<std::max(1, (int)std::min<long>((n + 7) / 8, (long)sm_count() * 4)), kThreads, 0, st>>>(
        F.dense.p, F.bv.p, F.x.p, (int)n, gate);
    return F.x.p;
  }
  T *cur = F.x.p, *oth = F.t.p;
  const double sweep_bytes = T_ * n * (F.ns + 4.0);
  const long h = n / 2;
  // Colour-split records, plain or classed. Algorithmic bytes of a phase: the
  // records of its colour, b of its colour, x of the other colour read and
  // the phase's writes of x.
  const Recs<T, 8> R7 = recs_of<T, 8>(F.rb, F.rbc);
  const Recs<T, 28> R27 = recs_of<T, 28>(F.rb27, F.rbc);
  const bool rb7 = R7.R || R7.code, rb27 = R27.R || R27.code;
  const bool quad = F.b.nx % 4 == 0 && p.quads;  // quartet kernels (FP32)
  const double rec7 = R7.code ? 2.0 : 8.0 * T_, rec27 = R27.code ? 2.0 : 28.0 * T_;
  auto relax = [&](bool zero, bool last) {
    if constexpr (sizeof(T) == 4) {
      if (p.relax == 2 && rb7 && quad && p.fused_sweep && !(zero && fin) && !(last && fout)) {
        // both colour phases in one kernel, out of place
        LaunchScope ls(K_MG_RELAX_FINE, st, (zero ? 0.5 * n * (R7.code ? 2.0 : T_) + 1.5 * T_ * n
                                                  : 0.5 * n * rec7 + 1.5 * T_ * n) +
                                                0.5 * n * rec7 + 1.5 * T_ * n);
        k_relax_rb_sweep<<<sweep_grid(F.b), kThreads, 0, st>>>(R7, F.bv.p, cur, oth, F.b, zero ? 1 : 0, gate);
        std::swap(cur, oth);
        return;
      }
      if (p.relax == 2 && rb7 && quad) {
        for (int color = 0; color < 2; ++color) {
          const bool z = zero && color == 0;
          if (z && fin) {
            LaunchScope ls(K_MG_RELAX_FINE, st, 0.5 * n * (R7.code ? 2.0 : T_) + (winvf ? 4.0 : 3.0) * T_ * n);
            k_relax_rb_quad_in<<<resident_grid(k_relax_rb_quad_in, n / 4), kThreads, 0, st>>>(R7, F.bv.p, cur, F.b, *fin, winvf, gate);
          } else if (color == 1 && last && fout) {
            LaunchScope ls(K_MG_RELAX_FINE, st, 0.5 * n * rec7 + 2.5 * T_ * n);
            k_relax_rb_quad_out<<<resident_grid(k_relax_rb_quad_out, n / 4), kThreads, 0, st>>>(R7, F.bv.p, cur, F.b, 1, *fout, gate);
          } else {
            LaunchScope ls(K_MG_RELAX_FINE, st, z ? 0.5 * n * (R7.code ? 2.0 : T_) + 1.5 * T_ * n
                                                  : 0.5 * n * rec7 + 1.5 * T_ * n);
            k_relax_rb_quad<<<resident_grid(k_relax_rb_quad, n / 4), kThreads, 0, st>>>(R7, F.bv.p, cur, F.b, color, z, gate);
          }
        }
        return;
      }
    }
    if (p.relax == 2 && rb7) {
      {
        LaunchScope ls(K_MG_RELAX_FINE, st, zero ? 0.5 * n * (R7.code ? 2.0 : T_) + 1.5 * T_ * n
                                                 : 0.5 * n * rec7 + 1.5 * T_ * n);
        if (zero) k_relax_rb_zero<T><<<grid_all(h), kThreads, 0, st>>>(R7, F.bv.p, cur, F.b, gate);
        else k_relax_rb<T><<<grid_all(h), kThreads, 0, st>>>(R7, F.bv.p, cur, F.b, 0, gate);
      }
      LaunchScope ls(K_MG_RELAX_FINE, st, 0.5 * n * rec7 + 1.5 * T_ * n);
      k_relax_rb<T><<<grid_all(h), kThreads, 0, st>>>(R7, F.bv.p, cur, F.b, 1, gate);
    } else if (p.relax == 2 && rb27) {
      for (int color = 0; color < 2; ++color) {
        const bool z = zero && color == 0;
        LaunchScope ls(K_MG_RELAX, st, z ? 0.5 * n * (R27.code ? 2.0 : T_) + 1.5 * T_ * n
                                         : 0.5 * n * rec27 + 2.5 * T_ * n);
        bool done = false;
        if constexpr (sizeof(T) == 4) {
          if (p.quads && F.b.nx % 4 == 0) {
            k_relax_rb27_quad<<<resident_grid(k_relax_rb27_quad, n / 4), kThreads, 0, st>>>(R27, F.bv.p, cur, oth, F.b, color, z, gate);
            done = true;
          }
        }
        if (!done) k_relax_rb27<T><<<grid_all(h), kThreads, 0, st>>>(R27, F.bv.p, cur, oth, F.b, color, z, gate);
        std::swap(cur, oth);
      }
    } else if (p.relax == 2) {
      for (int color = 0; color < 2; ++color) {
        const bool z = zero && color == 0;
        LaunchScope ls(K_MG_RELAX, st, z ? 3.0 * T_ * n : sweep_bytes);
        if (F.ns == 7) k_relax_color<T, 7><<<g, kThreads, 0, st>>>(F.A, F.invd.p, F.bv.p, cur, oth, F.b, color, z, gate);
        else k_relax_color<T, 27><<<g, kThreads, 0, st>>>(F.A, F.invd.p, F.bv.p, cur, oth, F.b, color, z, gate);
        std::swap(cur, oth);
      }
    } else if (zero) {
      LaunchScope ls(K_MG_RELAX, st, 3.0 * T_ * n);
      k_relax_zero<T><<<g, kThreads, 0, st>>>(F.wd.p, F.bv.p, cur, n, gate);
    } else {
      LaunchScope ls(K_MG_RELAX, st, sweep_bytes);
      if (F.ns == 7) k_relax_jacobi<T, 7><<<g, kThreads, 0, st>>>(F.A, F.wd.p, F.bv.p, cur, oth, F.b, gate);
      else k_relax_jacobi<T, 27><<<g, kThreads, 0, st>>>(F.A, F.wd.p, F.bv.p, cur, oth, F.b, gate);
      std::swap(cur, oth);
    }
  };
  // Inside a coarsening group (F.relax == 0) the level only passes the
  // right-hand side down and the correction up.
  // sweeps: the finest level takes nu1 / nu2, coarser relaxed levels nu_coarse
  // each way when it is set
  const int c1 = (l > 0 && p.nu_coarse > 0) ? p.nu_coarse : p.nu1, c2 = (l > 0 && p.nu_coarse > 0) ? p.nu_coarse : p.nu2;
  const int nu1 = F.relax ? c1 : 0, nu2 = F.relax ? c2 : 0;
  for (int s = 0; s < nu1; ++s) relax(s == 0, false);
  const T *res = F.bv.p;  // residual of a zero initial guess is b
  if (nu1 > 0 && p.relax == 2 && rb7) {
    LaunchScope ls(K_MG_RESID, st, 0.5 * n * rec7 + 2.5 * T_ * n);
    bool done = false;
    if constexpr (sizeof(T) == 4) {
      if (quad) {
        k_residual_rb_quad<<<resident_grid(k_residual_rb_quad, n / 4), kThreads, 0, st>>>(R7, F.bv.p, cur, F.r.p, F.b, gate);
        done = true;
      }
    }
    if (!done) k_residual_rb<T><<<grid_all(n / 2), kThreads, 0, st>>>(R7, F.bv.p, cur, F.r.p, F.b, gate);
    res = F.r.p;
  } else if (nu1 > 0 && p.relax == 2 && rb27) {
    LaunchScope ls(K_MG_RESID, st, n * rec27 + 3.0 * T_ * n);
    bool done = false;
    if constexpr (sizeof(T) == 4) {
      if (p.quads && F.b.nx % 4 == 0) {
        k_residual_rb27_quad<<<resident_grid(k_residual_rb27_quad, n / 4), kThreads, 0, st>>>(R27, F.bv.p, cur, F.r.p, F.b, gate);
        done = true;
      }
    }
    if (!done) k_residual_rb27<T><<<grid_all(n), kThreads, 0, st>>>(R27, F.bv.p, cur, F.r.p, F.b, gate);
    res = F.r.p;
  } else if (nu1 > 0) {
    LaunchScope ls(K_MG_RESID, st, T_ * n * (F.ns + 3.0));
    if (F.ns == 7) k_residual<T, 7><<<grid_all(n), kThreads, 0, st>>>(F.A, F.bv.p, cur, F.r.p, F.b, gate);
    else k_residual<T, 27><<<grid_all(n), kThreads, 0, st>>>(F.A, F.bv.p, cur, F.r.p, F.b, gate);
    res = F.r.p;
  }
  MgLevelT<T> &C = L[l + 1];
  {
    LaunchScope ls(K_MG_RESTRICT, st, T_ * (3.0 * n + C.b.n));
    if constexpr (sizeof(T) == 4) {
      if (F.cdir != 0 && F.b.nx % 4 == 0)
        k_restrict_yz4<<<resident_grid(k_restrict_yz4, C.b.n / 4), kThreads, 0, st>>>(res, F.pm.p, F.pp.p, F.b, F.cdir, C.bv.p, C.b, gate);
      else if (p.quads && F.cdir == 0 && F.b.nx == 2 * C.b.nx && C.b.nx % 4 == 0)
        k_restrict_x4<<<resident_grid(k_restrict_x4, C.b.n / 4), kThreads, 0, st>>>(res, F.pm.p, F.pp.p, F.b, C.bv.p, C.b, gate);
      else
        k_restrict<T><<<grid_all(C.b.n), kThreads, 0, st>>>(res, F.pm.p, F.pp.p, F.b, F.cdir, C.bv.p, C.b, gate);
    } else {
      k_restrict<T><<<grid_all(C.b.n), kThreads, 0, st>>>(res, F.pm.p, F.pp.p, F.b, F.cdir, C.bv.p, C.b, gate);
    }
  }
  T *xc = nullptr;
  if constexpr (sizeof(T) == 4) {
    if (tail && l + 1 == tail->level) xc = launch_tail(st, *tail, gate);
  }
  if (!xc) xc = vcycle<T>(st, L, l + 1, p, gate, nullptr, nullptr, nullptr, tail);
  {
    LaunchScope ls(K_MG_PROLONG, st, T_ * ((nu1 > 0 ? 4.0 : 3.0) * n + C.b.n));
    if constexpr (sizeof(T) == 4) {
      if (F.cdir != 0 && F.b.nx % 4 == 0)
        k_prolong_yz4<<<resident_grid(k_prolong_yz4, n / 4), kThreads, 0, st>>>(xc, C.b, F.pm.p, F.pp.p, F.b, F.cdir, cur, nu1 > 0, gate);
      else if (p.quads && F.cdir == 0 && F.b.nx == 2 * C.b.nx && C.b.nx % 4 == 0)
        k_prolong_x4<<<resident_grid(k_prolong_x4, n / 4), kThreads, 0, st>>>(xc, C.b, F.pm.p, F.pp.p, F.b, cur, nu1 > 0, gate);
      else
        k_prolong<T><<<grid_all(n), kThreads, 0, st>>>(xc, C.b, F.pm.p, F.pp.p, F.b, F.cdir, cur, nu1 > 0, gate);
    } else {
      k_prolong<T><<<grid_all(n), kThreads, 0, st>>>(xc, C.b, F.pm.p, F.pp.p, F.b, F.cdir, cur, nu1 > 0, gate);
    }
  }
  for (int s = 0; s < nu2; ++s) relax(false, s == nu2 - 1);
  return cur;
}

void Multigrid::apply(cudaStream_t st, const VecRef &in, const OutRef &out, const int *gate, bool use_fp32) {
  if (prm.cycles != 1) throw Error(IBM_ERR_UNSUPPORTED, "multigrid: only one V-cycle per application");
  const double ob = out.d ? 8.0 : 4.0;
  if (use_fp32) {
    if (L32.empty()) throw Error(IBM_ERR_STATE, "multigrid: FP32 hierarchy not built");
    MgLevelT<float> &F = L32[0];
    // input load and output store fused into the finest level's first and
    // last phases when that level relaxes with the quartet kernels
    const bool fuse = in.basef && out.f && !out.d && F.b.n % 4 == 0 && (in.ld % 4) == 0 && prm.quads &&
                      prm.relax == 2 && F.relax && F.cdir >= 0 && F.ns == 7 && (F.rb.p || F.rbc.ok()) &&
                      F.b.nx % 4 == 0 && prm.nu1 > 0 && prm.nu2 > 0;
    TailLaunch tl;
    if (tail_nops_ > 0) {
      tl.ops = reinterpret_cast<const TailOp *>(tail_ops_.p);
      tl.nops = tail_nops_; tl.blocks = tail_blocks_; tl.level = tail_level_;
      tl.bar = reinterpret_cast<TailBar *>(tail_bar_.p);
      tl.out = tail_out_; tl.bytes = tail_bytes_;
    }
    const TailLaunch *tp = tail_nops_ > 0 ? &tl : nullptr;
    if (fuse) {
      vcycle<float>(st, L32, 0, prm, gate, &in, &out, winvf_.p, tp);
      return;
    }
    {
      if (in.basef && F.b.n % 4 == 0 && (in.ld % 4) == 0) {
        LaunchScope ls(K_MG_LOAD, st, (winv_ ? 12.0 : 8.0) * F.b.n);
        k_load_input_f4<<<resident_grid(k_load_input_f4, F.b.n / 4), kThreads, 0, st>>>(F.bv.p, F.b.n, in, winvf_.p, gate);
      } else {
        LaunchScope ls(K_MG_LOAD, st, (winv_ ? 20.0 : 12.0) * F.b.n);
        k_load_input<float><<<grid_for(F.b.n), kThreads, 0, st>>>(F.bv.p, F.b.n, in, winv_, gate);
      }
    }
    float *x = vcycle<float>(st, L32, 0, prm, gate, nullptr, nullptr, nullptr, tp);
    LaunchScope ls(K_MG_STORE, st, (4.0 + ob) * F.b.n);
    k_store_output<float><<<grid_for(F.b.n), kThreads, 0, st>>>(x, F.b.n, out, gate);
  } else {
    MgLevelT<double> &F = L64[0];
    {
      LaunchScope ls(K_MG_LOAD, st, (winv_ ? 24.0 : 16.0) * F.b.n);
      k_load_input<double><<<grid_for(F.b.n), kThreads, 0, st>>>(F.bv.p, F.b.n, in, winv_, gate);
    }
    double *x = vcycle<double>(st, L64, 0, prm, gate);
    LaunchScope ls(K_MG_STORE, st, (8.0 + ob) * F.b.n);
    k_store_output<double><<<grid_for(F.b.n), kThreads, 0, st>>>(x, F.b.n, out, gate);
  }
}

void Multigrid::level_info(int l, int dims[3], int *cdir, int *ns) const {
  const auto &F = L64.at((size_t)l);
  dims[0] = F.b.nx; dims[1] = F.b.ny; dims[2] = F.b.nz;
  *cdir = F.cdir;
  *ns = F.ns;
}

void Multigrid::level_coef27(cudaStream_t st, int l, double *host_out) const {
  const auto &F = L64.at((size_t)l);
  const long n = F.b.n;
  std::vector<double> planes((size_t)F.ns * n);
  IBM_CUDA_TRY(cudaMemcpyAsync(planes.data(), F.A, sizeof(double) * planes.size(), cudaMemcpyDeviceToHost, st));
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
  static const int slot7[7] = {13, 12, 14, 10, 16, 4, 22};
  for (long r = 0; r < n; ++r) {
    for (int s = 0; s < 27; ++s) host_out[r * 27 + s] = 0.0;
    for (int q = 0; q < F.ns; ++q) host_out[r * 27 + (F.ns == 27 ? q : slot7[q])] = planes[(size_t)q * n + r];
  }
}

size_t Multigrid::bytes() const {
  size_t b = 0;
  for (const auto &F : L64) b += F.Aown.bytes() + F.wd.bytes() + F.invd.bytes() + F.pm.bytes() + F.pp.bytes() + F.x.bytes() + F.bv.bytes() + F.r.bytes() + F.t.bytes() + F.dense.bytes() + F.rb.bytes() + F.rb27.bytes() + F.rbc.bytes();
  for (const auto &F : L32) b += F.Aown.bytes() + F.wd.bytes() + F.invd.bytes() + F.pm.bytes() + F.pp.bytes() + F.x.bytes() + F.bv.bytes() + F.r.bytes() + F.t.bytes() + F.dense.bytes() + F.rb.bytes() + F.rb27.bytes() + F.rbc.bytes();
  return b;
}

}  // namespace ibm

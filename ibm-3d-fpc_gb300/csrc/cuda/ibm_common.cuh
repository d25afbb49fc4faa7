// Internal declarations shared by the CUDA translation units of libibmgpu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "ibm_gpu.h"

namespace ibm {

constexpr int kMaxKdim = 63;          // Krylov basis holds at most 64 vectors
constexpr int kThreads = 256;         // threads per block of the streaming kernels
constexpr int kWarps = kThreads / 32;
constexpr int kRowsPerThread = 4;     // rows per thread per tile in the reduction kernels
constexpr int kTile = kThreads * kRowsPerThread;
constexpr int kMaxSys = 4;            // systems solved together (u, v, w momentum batch)

// Error plumbing ------------------------------------------------------------
struct Status {
  int code = IBM_OK;
  std::string msg;
};

#define IBM_CUDA_TRY(expr)                                                                     \
  do {                                                                                         \
    cudaError_t e__ = (expr);                                                                  \
    if (e__ != cudaSuccess) {                                                                  \
      char b__[512];                                                                           \
      snprintf(b__, sizeof(b__), "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e__),      \
               __FILE__, __LINE__);                                                            \
      throw ::ibm::Error(IBM_ERR_CUDA, b__);                                                   \
    }                                                                                          \
  } while (0)

struct Error {
  int code;
  std::string msg;
  Error(int c, std::string m) : code(c), msg(std::move(m)) {}
};

// Device buffer -------------------------------------------------------------
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count == 0) return;
    cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      char b[256];
      snprintf(b, sizeof(b), "cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
      throw Error(IBM_ERR_NOMEM, b);
    }
    n = count;
  }
  void zero(cudaStream_t s) {
    if (p) IBM_CUDA_TRY(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Record classes (ibm_classes.cu) -------------------------------------------
// The distinct records of an array of nrec records of W values: record t
// equals tab[code[t]] bit for bit.
constexpr int kMaxClasses = 65535;
template <class T>
struct Classes {
  DBuf<uint16_t> code;  // class of each record
  DBuf<T> tab;          // [K][W] distinct records, first-seen order
  int K = 0, W = 0;
  bool ok() const { return code.p != nullptr; }
  size_t bytes() const { return code.bytes() + tab.bytes(); }
};
// Fills c for the records rec[t * W .. t * W + W) (device memory, t < nrec).
// Returns false and leaves c empty when there are more than kMaxClasses
// distinct records. Synchronises the stream.
template <class T>
bool build_classes(cudaStream_t st, const T *rec, int W, long nrec, Classes<T> &c);

// Division by an invariant divisor d >= 1 through a multiply-high (Granlund
// and Montgomery, "Division by invariant integers using multiplication",
// PLDI 1994): with s = ceil(log2 d) and m = floor(2^32 (2^s - d) / d) + 1,
// n / d = (mulhi(n, m) + n) >> s for every 32-bit n.
struct FastDiv {
  unsigned m = 1, s = 0;
};
inline FastDiv make_fastdiv(unsigned d) {
  FastDiv f;
  unsigned s = 0;
  while ((1ull << s) < d) ++s;
  f.s = s;
  f.m = (unsigned)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
  return f;
}

struct Box {
  int nx = 0, ny = 0, nz = 0, n = 0;
  FastDiv dx, dy;  // division by nx and by ny
};
inline Box make_box(int nx, int ny, int nz) {
  Box b;
  b.nx = nx; b.ny = ny; b.nz = nz; b.n = nx * ny * nz;
  b.dx = make_fastdiv((unsigned)(nx > 0 ? nx : 1));
  b.dy = make_fastdiv((unsigned)(ny > 0 ? ny : 1));
  return b;
}

// 7-point operator on a solve box: coefficient planes [7][n] (C,-x,+x,-y,+y,-z,+z).
struct Op7 {
  Box b;
  bool set = false;
  DBuf<double> c;      // as supplied
  DBuf<double> invd;   // 1 / C
  DBuf<double> cj;     // C * invd(neighbour): the right-Jacobi-preconditioned operator
  DBuf<float> cf;      // FP32 coefficients (mixed precision)
  DBuf<float> cjf;     // FP32 copy of cj (two Jacobi sweeps in one pass)
  DBuf<float> invdf;
  // Record classes of the rows (empty when there are too many distinct rows):
  Classes<double> cls;  // classes of the supplied rows (W 7)
  DBuf<double> tab;     // [K][8] the distinct rows, slot 7 zero
  DBuf<float> tabf;     // [K][8] their FP32 copies (the rows of cf)
  DBuf<float> tabdf;    // [K][16] the rows as double-float pairs: hi in slots 0-7, lo in 8-15
  Classes<float> clsj;  // classes of the FP32 Jacobi records {invdf, cjf_1..cjf_6, 0} (W 8)
  bool cls_tried = false;  // classes built (or found too many) for the current coefficients
};

// Per-system GMRES scalars kept on the device (no host round trip per iteration).
struct KScal {
  int kdim, maxit;
  double tol;
  int active;         // 1 while an Arnoldi cycle is running
  int cycle_end;      // 1 when the cycle stopped and the solution update is due
  int i;              // Arnoldi vectors built in this cycle
  int iters;
  int status;         // 0 running, 1 converged, 2 iteration limit, 3 stagnation
  int claimed;        // the Givens estimate reached the tolerance
  unsigned ticket;    // last-block-done counter of the reduction kernels
  int nonfinite;
  int use64;          // double-float residual too close to call: FP64 residuals for the rest of the solve
  double b_norm, r_norm, eps, real_old;
  double cyc_eps;     // the current cycle also ends when the estimate reaches this
  double cyc_rtol;    // cyc_eps = max(eps, cyc_rtol * true residual at the cycle start)
  double nu[kMaxKdim + 1];            // norms of the stored (unnormalised) basis vectors
  double H[(kMaxKdim + 1) * kMaxKdim];  // H(i,j) at [i*kMaxKdim + j]
  double cs[kMaxKdim], sn[kMaxKdim], g[kMaxKdim + 1], y[kMaxKdim];
  double coef[kMaxKdim + 1];          // coefficients of the next basis update
  double h1[kMaxKdim + 1];
};

// Device view of one linear system for the Krylov kernels.
struct KSys {
  int nx, ny, nz, n;
  FastDiv fdx, fdy;     // division by nx and by ny
  const double *A;      // operator applied in the Arnoldi step ([7][n])
  const double *Ar;     // operator of the true residual ([7][n])
  const double *invd;   // inverse diagonal (Jacobi solution update)
  const float *Af;      // FP32 operator (inner FP32 sweeps)
  const float *Ajf;     // FP32 right-Jacobi-scaled operator (cj)
  const float *invdf;
  double *V;            // basis, vector k at V + k*ldv
  long ldv;
  float *Z;             // flexible basis (FP32), vector k at Z + k*ldv
  double *w, *x, *z, *z2;
  const double *b;
  float *zf, *zf2;      // FP32 work for the inner sweeps
  double *part;         // block partial sums [nblk][kMaxKdim + 2]
  float *Vf, *wf;       // FP32 basis and work vector of the FP32 Arnoldi cycles (a32)
  int a32;              // Arnoldi cycles in FP32 (basis, operator, dots per thread), restarts in FP64
  int x_zero;           // the initial guess is zero: the first residual is b
  int vec4;             // n % 4 == 0: FP32 vectors and planes are 16-byte aligned in blocks of 4 rows
  int nblk;
  int pc;               // 0 Jacobi folded into A, 1 explicit z (multigrid), 2 flexible FP32 z
  int pc_cb;            // pc 2: preconditioner supplied by a callback (else FP32 Jacobi sweeps)
  KScal *s;
  // Record classes (null cls / clsj: the planes above are read instead)
  const uint16_t *cls;  // class of each row of Ar (and of Af, its FP32 copy)
  const double *tab;    // [K][8] rows of Ar
  const float *tabf;    // [K][8] rows of Af
  const uint16_t *clsj; // class of each FP32 Jacobi record
  const float *tabj;    // [K][8] {invdf, Ajf_1..Ajf_6, 0}
  const float *tabdf;   // [K][16] rows of Ar as double-float pairs
  int df_resid;         // FP32 cycles with classes: true residuals in double-float (FP32 pipe)
  float2 *xs;           // df_resid: x as double-float pairs, written with every update of x
  int df_spmv;          // pc 2, FP64 cycles, classes: A z_j in double-float (tabdf) on the FP32 pipe
  int cgs1;             // pc 2, FP64 cycles: one classical Gram-Schmidt pass (no k_arnoldi_orth)
  float *vcur;          // pc 2 with FP32 Jacobi and an FP64 basis: (float) V_j of the current j, written
                        // by the kernel that forms V_j, read by the Jacobi sweeps (null: read V_j)
};

// Host-side mirror of what the loop needs from each system after a step.
struct KFlags {
  int active, cycle_end, status, iters, i, nonfinite;
  double rel;
};

// ---------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Flat row -> (i, j, k) on a box.
__device__ __forceinline__ unsigned fast_div(unsigned n, FastDiv f) {
  return (unsigned)(((unsigned long long)__umulhi(n, f.m) + n) >> f.s);
}
// Flat row -> (i, j, k) on a box without hardware-emulated divisions.
__device__ __forceinline__ void box_ijk(long r, const Box &b, int &i, int &j, int &k) {
  const unsigned q = fast_div((unsigned)r, b.dx);
  i = (int)((unsigned)r - q * (unsigned)b.nx);
  const unsigned kk = fast_div(q, b.dy);
  j = (int)(q - kk * (unsigned)b.ny);
  k = (int)kk;
}
__device__ __forceinline__ void row_ijk(int r, int nx, int ny, int &i, int &j, int &k) {
  const unsigned plane = (unsigned)nx * (unsigned)ny;
  k = (int)((unsigned)r / plane);
  const unsigned rem = (unsigned)r - (unsigned)k * plane;
  j = (int)(rem / (unsigned)nx);
  i = (int)(rem - (unsigned)j * (unsigned)nx);
}

// y_r = sum_s c_s x_{r+off_s}, fused multiply-add chain in slot order
// C,-x,+x,-y,+y,-z,+z; neighbours outside the box contribute 0. Slot s of the
// row is c0[s * cs]: planes [7][n] give c0 = c + r, cs = n; a class table
// row gives cs = 1.
template <class T, class X>
__device__ __forceinline__ double stencil7_at(const T *__restrict__ c0, long cs, const X *__restrict__ x, int r,
                                              int i, int j, int k, int nx, int ny, int nz) {
  const long sy = nx, sz = (long)nx * ny;
  double acc = 0.0;
  acc = fma((double)c0[0], (double)x[r], acc);
  acc = fma((double)c0[cs], i > 0 ? (double)x[r - 1] : 0.0, acc);
  acc = fma((double)c0[2 * cs], i < nx - 1 ? (double)x[r + 1] : 0.0, acc);
  acc = fma((double)c0[3 * cs], j > 0 ? (double)x[r - sy] : 0.0, acc);
  acc = fma((double)c0[4 * cs], j < ny - 1 ? (double)x[r + sy] : 0.0, acc);
  acc = fma((double)c0[5 * cs], k > 0 ? (double)x[r - sz] : 0.0, acc);
  acc = fma((double)c0[6 * cs], k < nz - 1 ? (double)x[r + sz] : 0.0, acc);
  return acc;
}
template <class T, class X>
__device__ __forceinline__ double stencil7_row(const T *__restrict__ c, long n, const X *__restrict__ x, int r,
                                               int i, int j, int k, int nx, int ny, int nz) {
  return stencil7_at(c + r, n, x, r, i, j, k, nx, ny, nz);
}

// FP32 variant.
__device__ __forceinline__ float stencil7_at_f(const float *__restrict__ c0, long cs, const float *__restrict__ x,
                                               int r, int i, int j, int k, int nx, int ny, int nz) {
  const long sy = nx, sz = (long)nx * ny;
  float acc = 0.0f;
  acc = fmaf(c0[0], x[r], acc);
  acc = fmaf(c0[cs], i > 0 ? x[r - 1] : 0.0f, acc);
  acc = fmaf(c0[2 * cs], i < nx - 1 ? x[r + 1] : 0.0f, acc);
  acc = fmaf(c0[3 * cs], j > 0 ? x[r - sy] : 0.0f, acc);
  acc = fmaf(c0[4 * cs], j < ny - 1 ? x[r + sy] : 0.0f, acc);
  acc = fmaf(c0[5 * cs], k > 0 ? x[r - sz] : 0.0f, acc);
  acc = fmaf(c0[6 * cs], k < nz - 1 ? x[r + sz] : 0.0f, acc);
  return acc;
}
__device__ __forceinline__ float stencil7_row_f(const float *__restrict__ c, long n, const float *__restrict__ x,
                                                int r, int i, int j, int k, int nx, int ny, int nz) {
  return stencil7_at_f(c + r, n, x, r, i, j, k, nx, ny, nz);
}

// Grid size for persistent grid-stride kernels: a multiple of the SM count.
int persistent_blocks(int rows, int blocks_per_sm = 4);
int sm_count();

// Launch counter (all kernels of the library go through this).
void count_launch(long long n = 1);
long long launches();

// Kernel classes for accounting (ibm_profile in include/ibm_gpu.h).
enum KernelId {
  K_BC = 0, K_RHS, K_SCATTER, K_PRHS, K_PROJECT, K_DIAG,
  K_GM_INIT, K_GM_SPMV, K_GM_ORTH, K_GM_NEXT, K_GM_UPDATE, K_GM_RESID, K_GM_ADDZ, K_GM_JAC32,
  K_MG_LOAD, K_MG_RELAX, K_MG_RESID, K_MG_RESTRICT, K_MG_PROLONG, K_MG_DENSE, K_MG_STORE,
  K_MG_RELAX_FINE,  // in-place two-colour phases of 7-point levels (the finest)
  K_MG_COARSE,      // all levels below the finest fused into one persistent kernel per V-cycle
  K_ADJOINT,        // reverse sweep of the adjoint step (dense transposes)
  K_SETUP, K_COUNT
};
const char *kernel_name(int k);

// Records one launch of kernel class k moving `bytes` algorithmic bytes; when
// k is the context's timed class, the launch is bracketed by CUDA events on
// stream st. Construct immediately before the launch, destroy after it.
struct LaunchScope {
  LaunchScope(KernelId k, cudaStream_t st, double bytes, long long n = 1);
  ~LaunchScope();
  KernelId k;
  cudaStream_t st;
  int slot = -1;
};

// Per-context accounting state (one per ibm_ctx; current one is thread-local).
enum Phase { PH_RHS = 0, PH_MOM, PH_P, PH_PROJ, PH_OTHER, PH_COUNT };
struct Prof {
  long long launches[K_COUNT] = {};
  double bytes[K_COUNT] = {};
  double ms[K_COUNT] = {};
  long long timed[K_COUNT] = {};
  double phase_bytes[PH_COUNT] = {};
  int phase = PH_OTHER;
  int timed_kernel = -1;
  std::vector<cudaEvent_t> pool;
  struct Pending { int k; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  void reset();
  void drain();  // call after the stream is synchronised
  ~Prof();
};
Prof *&current_prof();
struct PhaseScope {
  int prev;
  explicit PhaseScope(int ph) {
    Prof *p = current_prof();
    prev = p ? p->phase : PH_OTHER;
    if (p) p->phase = ph;
  }
  ~PhaseScope() {
    if (Prof *p = current_prof()) p->phase = prev;
  }
};

}  // namespace ibm

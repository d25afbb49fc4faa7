// Restarted, right-preconditioned GMRES for up to kMaxSys independent 7-point
// systems at once, with every scalar kept on the device.
//
// Restates the algorithm of HYPRE_StructGMRESSolve (third-party, called by
// the reference at main.cu:284-286 and 327): Arnoldi with Givens rotations,
// stop when the estimated ||r||/||b|| <= tol, confirm with the true residual
// and restart from it; a cycle whose estimate claimed convergence but whose
// true residual did not decrease stops (stagnation), as HYPRE does.
// Orthogonalisation is classical Gram-Schmidt applied twice, so each pass is
// one sweep over the basis with all dot products batched.
//
// Per Arnoldi step, three streaming kernels:
//   k_arnoldi_spmv : w = A z_j and d1_k = (v_k, w)         (last block: h1, coefficients)
//   k_arnoldi_orth : w -= V c1, d2_k = (v_k, w)              (last block: h2, Hessenberg column)
//   k_arnoldi_next : v_{j+1} = w - V c2, |v_{j+1}|^2          (last block: Givens, stop test)
// Basis vectors are stored unnormalised with their exact norms in nu[].
// Reductions are deterministic: fixed per-warp order inside a block, block
// partials summed in block order by the last block to finish.
#include "ibm_common.cuh"
#include "ibm_krylov.cuh"
#include "ibm_df.cuh"

namespace ibm {

namespace {

constexpr int kLd = kMaxKdim + 2;  // stride of block partials
constexpr int kChunk32 = 8;  // basis vectors whose dot products a thread keeps in registers

// Flat row -> (i, j, k) of a system's box (invariant-divisor division).
__device__ __forceinline__ void sys_ijk(long r, const KSys &S, int &i, int &j, int &k) {
  const unsigned q = fast_div((unsigned)r, S.fdx);
  i = (int)((unsigned)r - q * (unsigned)S.nx);
  const unsigned kk = fast_div(q, S.fdy);
  j = (int)(q - kk * (unsigned)S.ny);
  k = (int)kk;
}

// Slot 0 of row r of Ar and the distance between its slots: the row of the
// row's class, or the planes.
__device__ __forceinline__ const double *ar_row(const KSys &S, long r, long &cs) {
  if (S.cls) { cs = 1; return S.tab + 8 * (long)S.cls[r]; }
  cs = S.n;
  return S.Ar + r;
}
// The same for the Arnoldi operator A (classed only when A is Ar).
__device__ __forceinline__ const double *a_row(const KSys &S, long r, long &cs) {
  if (S.cls && S.A == S.Ar) { cs = 1; return S.tab + 8 * (long)S.cls[r]; }
  cs = S.n;
  return S.A + r;
}
// ... and for Af, the FP32 copy of Ar.
__device__ __forceinline__ const float *af_row(const KSys &S, long r, long &cs) {
  if (S.cls) { cs = 1; return S.tabf + 8 * (long)S.cls[r]; }
  cs = S.n;
  return S.Af + r;
}

// Four class-table rows (8 floats each) as four 16-byte pairs, transposed so
// that cp[s] holds slot s of the four rows.
__device__ __forceinline__ void load_rows4(const float *__restrict__ tab, ushort4 c4, float4 (&cp)[7]) {
  const unsigned short ks[4] = {c4.x, c4.y, c4.z, c4.w};
  float v[4][8];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float4 *p = reinterpret_cast<const float4 *>(tab + 8 * (long)ks[q]);
    const float4 a = __ldg(p), b = __ldg(p + 1);
    v[q][0] = a.x; v[q][1] = a.y; v[q][2] = a.z; v[q][3] = a.w;
    v[q][4] = b.x; v[q][5] = b.y; v[q][6] = b.z; v[q][7] = b.w;
  }
#pragma unroll
  for (int s = 0; s < 7; ++s) cp[s] = make_float4(v[0][s], v[1][s], v[2][s], v[3][s]);
}

// Sum block partials of `nd` dot products in block order; one warp per dot.
__device__ void reduce_partials(const double *part, int nblk, int nd, double *out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int k = warp; k < nd; k += kWarps) {
    double s = 0.0;
    for (int b = lane; b < nblk; b += 32) s += part[(long)b * kLd + k];
    s = warp_sum(s);
    if (lane == 0) out[k] = s;
  }
}

// Common tail of the reduction kernels: write this block's sums, and return
// true in the block that finishes last (after all partials are visible).
__device__ bool block_partials_and_last(double *sacc, int nd, double *part, unsigned *ticket) {
  __syncthreads();
  for (int k = threadIdx.x; k < nd; k += blockDim.x) {
    double s = 0.0;
    for (int w = 0; w < kWarps; ++w) s += sacc[k * kWarps + w];
    part[(long)blockIdx.x * kLd + k] = s;
  }
  __threadfence();
  __syncthreads();
  __shared__ int last;
  if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (last) __threadfence();
  return last != 0;
}

// r = b - Ar x; V_0 = r; |b|^2, |r|^2. Last block: norms, tolerance, state.
__global__ void __launch_bounds__(kThreads) k_init(KSys *sys, int nsys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  __shared__ double sacc[2 * kWarps];
  if (threadIdx.x < 2 * kWarps) sacc[threadIdx.x] = 0.0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // per-thread sums over all of the thread's rows, one warp reduction at the
  // end (GB300's FP64 pipe is the bound here: no FP64 work per tile)
  double pb = 0.0, pr = 0.0;
  if (S.a32 && S.x_zero) {
    // r = b: the FP32 basis vector from the bits of b (integer split, one FP32
    // add: b rounded to FP32), |b|^2 in FP32 per thread; no FP64 instruction
    float pf = 0.0f;
    for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
#pragma unroll
      for (int t = 0; t < kRowsPerThread; ++t) {
        const long r = t0 + t * kThreads + threadIdx.x;
        if (r < S.n) {
          float bh, bl;
          df_split(S.b[r], bh, bl);
          const float v = __fadd_rn(bh, bl);
          S.Vf[r] = v;
          pf = fmaf(v, v, pf);
        }
      }
    }
    pb = pr = (double)pf;
  } else {
    for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
#pragma unroll
      for (int t = 0; t < kRowsPerThread; ++t) {
        const long r = t0 + t * kThreads + threadIdx.x;
        if (r < S.n) {
          int i, j, k;
          sys_ijk(r, S, i, j, k);
          // with finite coefficients A 0 is +0 in every row, so b - 0 equals b - A x
          // bit for bit: a zero guess takes r = b and |r| = |b|
          const double bv = S.b[r];
          double rv = bv;
          if (!S.x_zero) {
            long cs;
            const double *c0 = ar_row(S, r, cs);
            rv = bv - stencil7_at(c0, cs, S.x, (int)r, i, j, k, S.nx, S.ny, S.nz);
            pr = fma(rv, rv, pr);
          }
          if (S.a32) S.Vf[r] = (float)rv;
          else S.V[r] = rv;
          if (S.vcur) S.vcur[r] = (float)rv;
          pb = fma(bv, bv, pb);
        }
      }
    }
    if (S.x_zero) pr = pb;
  }
  pb = warp_sum(pb);
  pr = warp_sum(pr);
  if (lane == 0) { sacc[warp] = pb; sacc[kWarps + warp] = pr; }
  if (!block_partials_and_last(sacc, 2, S.part, &sc->ticket)) return;
  __shared__ double tot[2];
  reduce_partials(S.part, gridDim.x, 2, tot);
  __syncthreads();
  if (threadIdx.x == 0) {
    sc->ticket = 0;
    const double bn = sqrt(tot[0]), rn = sqrt(tot[1]);
    sc->b_norm = bn;
    sc->r_norm = rn;
    sc->eps = sc->tol * (bn > 0.0 ? bn : rn);
    sc->cyc_eps = fmax(sc->eps, sc->cyc_rtol * rn);
    sc->real_old = bn;
    sc->iters = 0;
    sc->i = 0;
    sc->claimed = 0;
    sc->cycle_end = 0;
    sc->nonfinite = !isfinite(rn);
    sc->use64 = 0;
    if (!isfinite(rn)) { sc->status = 2; sc->active = 0; }
    else if (rn == 0.0 || rn <= sc->eps) { sc->status = 1; sc->active = 0; }
    else if (sc->maxit <= 0) { sc->status = 2; sc->active = 0; }
    else { sc->status = 0; sc->active = 1; }
    sc->nu[0] = rn;
    sc->g[0] = rn;
  }
}

// w = A z_j (z_j = M v_j by the system's preconditioner mode), d1_k = (V_k, w).
// Closes Arnoldi step j (one thread): h(j+1,j) = |v_{j+1}| = hn, the previous
// rotations applied to the new Hessenberg column, a new Givens rotation, the
// residual estimate and the stop tests; at the end of a cycle the
// back-substitution H y = g and the update coefficients y / nu.
__device__ void arnoldi_finalize(KScal *sc, int j, double hn) {
  const int K = kMaxKdim;
  sc->nu[j + 1] = hn;
  sc->H[(j + 1) * K + j] = hn;
  // apply previous rotations to the new column, then a new rotation
  for (int q = 0; q < j; ++q) {
    const double t = sc->H[q * K + j];
    sc->H[q * K + j] = sc->sn[q] * sc->H[(q + 1) * K + j] + sc->cs[q] * t;
    sc->H[(q + 1) * K + j] = -sc->sn[q] * t + sc->cs[q] * sc->H[(q + 1) * K + j];
  }
  const double a = sc->H[j * K + j], b = sc->H[(j + 1) * K + j];
  double gam = sqrt(b * b + a * a);
  if (gam == 0.0) gam = 2.220446049250313e-16;
  sc->cs[j] = a / gam;
  sc->sn[j] = b / gam;
  sc->g[j + 1] = -sc->sn[j] * sc->g[j];
  sc->g[j] = sc->cs[j] * sc->g[j];
  sc->H[j * K + j] = sc->sn[j] * b + sc->cs[j] * a;
  sc->i = j + 1;
  sc->iters += 1;
  sc->r_norm = fabs(sc->g[j + 1]);
  const bool claimed = sc->r_norm <= sc->eps || hn == 0.0;
  const bool cycle_done = sc->r_norm <= sc->cyc_eps;
  if (!isfinite(sc->r_norm)) sc->nonfinite = 1;
  if (claimed || cycle_done || sc->i >= sc->kdim || sc->iters >= sc->maxit || !isfinite(sc->r_norm)) {
    sc->claimed = claimed;
    sc->active = 0;
    sc->cycle_end = 1;
    // back substitution H y = g for the i x i upper triangle
    const int m = sc->i;
    for (int q = m - 1; q >= 0; --q) {
      double t = sc->g[q];
      for (int c = q + 1; c < m; ++c) t -= sc->H[q * K + c] * sc->y[c];
      sc->y[q] = t / sc->H[q * K + q];
    }
    for (int q = 0; q < m; ++q) sc->coef[q] = sc->y[q] / sc->nu[q];
  }
}

// FP64 Arnoldi kernels with a short basis (at most kDots64 vectors) keep each
// dot product as a per-thread sum over all the thread's rows and reduce it
// across the warp once per kernel; a reduction per tile of rows cost about as
// much FP64 issue as the products themselves.
constexpr int kDots64 = 8;
__device__ __forceinline__ void flush_dots64(const double (&pd)[kDots64], int nd, double *sacc, int warp,
                                             int lane) {
#pragma unroll
  for (int kk = 0; kk < kDots64; ++kk) {
    if (kk >= nd) break;
    const double p = warp_sum(pd[kk]);
    if (lane == 0) sacc[kk * kWarps + warp] += p;
  }
}

__global__ void __launch_bounds__(kThreads) k_arnoldi_spmv(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->active || S.a32) return;
  const int j = sc->i, nd = j + 1;
  __shared__ double sacc[(kMaxKdim + 1) * kWarps];
  for (int t = threadIdx.x; t < nd * kWarps; t += blockDim.x) sacc[t] = 0.0;
  __shared__ double inv_nu;
  if (threadIdx.x == 0) inv_nu = 1.0 / sc->nu[j];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double *vj = S.V + (long)j * S.ldv;
  double pd[kDots64];
#pragma unroll
  for (int kk = 0; kk < kDots64; ++kk) pd[kk] = 0.0;
  for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
    double wv[kRowsPerThread];
#pragma unroll
    for (int t = 0; t < kRowsPerThread; ++t) {
      const long r = t0 + t * kThreads + threadIdx.x;
      wv[t] = 0.0;
      if (r < S.n) {
        int i, jj, k;
        sys_ijk(r, S, i, jj, k);
        double w;
        long cs;
        const double *c0 = a_row(S, r, cs);
        if (S.df_spmv) {
          // A z_j with z_j exact in FP32: the seven products and their sum in
          // double-float, widened once (two conversions and one FP64 add)
          // (a neighbour outside the box reads as 0: its product and sum are
          // exact no-ops, so all seven loads issue together)
          const float4 *c4 = reinterpret_cast<const float4 *>(S.tabdf + 16 * (long)S.cls[r]);
          const float *zj = S.Z + (long)j * S.ldv;
          const long sy = S.nx, sz = (long)S.nx * S.ny;
          const float z0 = zj[r], zxm = i > 0 ? zj[r - 1] : 0.0f, zxp = i < S.nx - 1 ? zj[r + 1] : 0.0f,
                      zym = jj > 0 ? zj[r - sy] : 0.0f, zyp = jj < S.ny - 1 ? zj[r + sy] : 0.0f,
                      zzm = k > 0 ? zj[r - sz] : 0.0f, zzp = k < S.nz - 1 ? zj[r + sz] : 0.0f;
          const float4 h0 = __ldg(c4), h1 = __ldg(c4 + 1), l0 = __ldg(c4 + 2), l1 = __ldg(c4 + 3);
          float ah = 0.0f, al = 0.0f;
          df_fma1(ah, al, h0.x, l0.x, z0);
          df_fma1(ah, al, h0.y, l0.y, zxm);
          df_fma1(ah, al, h0.z, l0.z, zxp);
          df_fma1(ah, al, h0.w, l0.w, zym);
          df_fma1(ah, al, h1.x, l1.x, zyp);
          df_fma1(ah, al, h1.y, l1.y, zzm);
          df_fma1(ah, al, h1.z, l1.z, zzp);
          w = (double)ah + (double)al;
        } else if (S.pc == 0) w = stencil7_at(c0, cs, vj, (int)r, i, jj, k, S.nx, S.ny, S.nz) * inv_nu;
        else if (S.pc == 1) w = stencil7_at(c0, cs, S.z, (int)r, i, jj, k, S.nx, S.ny, S.nz) * inv_nu;
        else w = stencil7_at(c0, cs, S.Z + (long)j * S.ldv, (int)r, i, jj, k, S.nx, S.ny, S.nz);
        S.w[r] = w;
        wv[t] = w;
      }
    }
    if (nd <= kDots64) {  // per-thread sums over all the thread's rows (reduced once below)
#pragma unroll
      for (int kk = 0; kk < kDots64; ++kk) {
        if (kk >= nd) break;
        const double *vk = S.V + (long)kk * S.ldv;
#pragma unroll
        for (int t = 0; t < kRowsPerThread; ++t) {
          const long r = t0 + t * kThreads + threadIdx.x;
          if (r < S.n) pd[kk] = fma(vk[r], wv[t], pd[kk]);
        }
      }
      continue;
    }
    for (int kk = 0; kk < nd; ++kk) {
      const double *vk = S.V + (long)kk * S.ldv;
      double p = 0.0;
#pragma unroll
      for (int t = 0; t < kRowsPerThread; ++t) {
        const long r = t0 + t * kThreads + threadIdx.x;
        if (r < S.n) p = fma(vk[r], wv[t], p);
      }
      p = warp_sum(p);
      if (lane == 0) sacc[kk * kWarps + warp] += p;
    }
  }
  if (nd <= kDots64) flush_dots64(pd, nd, sacc, warp, lane);
  if (!block_partials_and_last(sacc, nd, S.part, &sc->ticket)) return;
  __shared__ double tot[kMaxKdim + 1];
  reduce_partials(S.part, gridDim.x, nd, tot);
  __syncthreads();
  for (int kk = threadIdx.x; kk < nd; kk += blockDim.x) {
    const double h = tot[kk] / sc->nu[kk];
    sc->h1[kk] = h;
    sc->coef[kk] = h / sc->nu[kk];
    if (S.cgs1) sc->H[kk * kMaxKdim + j] = h;  // one pass: the column is the first projection
  }
  if (threadIdx.x == 0) sc->ticket = 0;
}

// w -= sum_k coef_k V_k (first pass), d2_k = (V_k, w). Last block: the
// second-pass coefficients and the Hessenberg column above the diagonal.
__global__ void __launch_bounds__(kThreads) k_arnoldi_orth(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->active || S.a32 || S.cgs1) return;
  const int j = sc->i, nd = j + 1;
  __shared__ double sacc[(kMaxKdim + 1) * kWarps];
  __shared__ double cf[kMaxKdim + 1];
  for (int t = threadIdx.x; t < nd * kWarps; t += blockDim.x) sacc[t] = 0.0;
  for (int t = threadIdx.x; t < nd; t += blockDim.x) cf[t] = sc->coef[t];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double pd[kDots64];
#pragma unroll
  for (int kk = 0; kk < kDots64; ++kk) pd[kk] = 0.0;
  for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
    double wv[kRowsPerThread];
#pragma unroll
    for (int t = 0; t < kRowsPerThread; ++t) {
      const long r = t0 + t * kThreads + threadIdx.x;
      wv[t] = 0.0;
      if (r < S.n) {
        double w = S.w[r];
        for (int kk = 0; kk < nd; ++kk) w = fma(-cf[kk], S.V[(long)kk * S.ldv + r], w);
        S.w[r] = w;
        wv[t] = w;
      }
    }
    if (nd <= kDots64) {
#pragma unroll
      for (int kk = 0; kk < kDots64; ++kk) {
        if (kk >= nd) break;
#pragma unroll
        for (int t = 0; t < kRowsPerThread; ++t) {
          const long r = t0 + t * kThreads + threadIdx.x;
          if (r < S.n) pd[kk] = fma(S.V[(long)kk * S.ldv + r], wv[t], pd[kk]);
        }
      }
      continue;
    }
    for (int kk = 0; kk < nd; ++kk) {
      double p = 0.0;
#pragma unroll
      for (int t = 0; t < kRowsPerThread; ++t) {
        const long r = t0 + t * kThreads + threadIdx.x;
        if (r < S.n) p = fma(S.V[(long)kk * S.ldv + r], wv[t], p);
      }
      p = warp_sum(p);
      if (lane == 0) sacc[kk * kWarps + warp] += p;
    }
  }
  if (nd <= kDots64) flush_dots64(pd, nd, sacc, warp, lane);
  if (!block_partials_and_last(sacc, nd, S.part, &sc->ticket)) return;
  __shared__ double tot[kMaxKdim + 1];
  reduce_partials(S.part, gridDim.x, nd, tot);
  __syncthreads();
  for (int kk = threadIdx.x; kk < nd; kk += blockDim.x) {
    const double h2 = tot[kk] / sc->nu[kk];
    sc->coef[kk] = h2 / sc->nu[kk];
    sc->H[kk * kMaxKdim + j] = sc->h1[kk] + h2;
  }
  if (threadIdx.x == 0) sc->ticket = 0;
}

// v_{j+1} = w - sum_k coef_k V_k, stored unnormalised, with its exact norm.
// Last block: Hessenberg column, Givens rotation, stop test, and at the end
// of a cycle the back substitution.
__global__ void __launch_bounds__(kThreads) k_arnoldi_next(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->active || S.a32) return;
  const int j = sc->i, nd = j + 1;
  __shared__ double cf[kMaxKdim + 1];
  __shared__ double sacc[kWarps];
  for (int t = threadIdx.x; t < nd; t += blockDim.x) cf[t] = sc->coef[t];
  if (threadIdx.x < kWarps) sacc[threadIdx.x] = 0.0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *vn = S.V + (long)nd * S.ldv;
  const bool store = nd < sc->kdim;  // the last vector of a full cycle is never used
  double p = 0.0;  // per thread over all its rows
  for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
#pragma unroll
    for (int t = 0; t < kRowsPerThread; ++t) {
      const long r = t0 + t * kThreads + threadIdx.x;
      if (r < S.n) {
        double w = S.w[r];
        for (int kk = 0; kk < nd; ++kk) w = fma(-cf[kk], S.V[(long)kk * S.ldv + r], w);
        if (store) {
          vn[r] = w;
          if (S.vcur) S.vcur[r] = (float)w;
        }
        p = fma(w, w, p);
      }
    }
  }
  p = warp_sum(p);
  if (lane == 0) sacc[warp] = p;
  if (!block_partials_and_last(sacc, 1, S.part, &sc->ticket)) return;
  __shared__ double tot[1];
  reduce_partials(S.part, gridDim.x, 1, tot);
  __syncthreads();
  if (threadIdx.x == 0) {
    sc->ticket = 0;
    arnoldi_finalize(sc, j, sqrt(tot[0]));
  }
}

// Cycle end, solution update. pc 0: x += invd * (V c); pc 1: z = V c (the
// caller applies the preconditioner and then k_add_z); pc 2: x += Z y.
__global__ void __launch_bounds__(kThreads) k_cycle_update(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->cycle_end) return;
  const int m = sc->i;
  __shared__ double cf[kMaxKdim + 1];
  for (int t = threadIdx.x; t < m; t += blockDim.x) cf[t] = S.pc == 2 ? sc->y[t] : sc->coef[t];
  __syncthreads();
  if (S.a32) {
    // FP32 cycles: the correction sum Z y is formed in FP32 (its rounding is
    // far below what the cycle resolved; the restart measures the true
    // residual of the FP64 x) and added to x in FP64
    __shared__ float cf32[kMaxKdim + 1];
    for (int t = threadIdx.x; t < m; t += blockDim.x) cf32[t] = (float)cf[t];
    __syncthreads();
    if (S.vec4 && m <= kChunk32) {
      // four consecutive rows per thread: 16-byte loads of the directions,
      // every load of the thread in flight together; same sums row by row
      for (long r0 = 4 * ((long)blockIdx.x * blockDim.x + threadIdx.x); r0 < S.n;
           r0 += 4L * gridDim.x * blockDim.x) {
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int kk = 0; kk < kChunk32; ++kk) {
          if (kk < m) {
            const float4 z = *reinterpret_cast<const float4 *>(S.Z + (long)kk * S.ldv + r0);
            acc.x = fmaf(cf32[kk], z.x, acc.x);
            acc.y = fmaf(cf32[kk], z.y, acc.y);
            acc.z = fmaf(cf32[kk], z.z, acc.z);
            acc.w = fmaf(cf32[kk], z.w, acc.w);
          }
        }
        const double2 x01 = *reinterpret_cast<const double2 *>(S.x + r0);
        const double2 x23 = *reinterpret_cast<const double2 *>(S.x + r0 + 2);
        const double xn[4] = {x01.x + (double)acc.x, x01.y + (double)acc.y, x23.x + (double)acc.z,
                              x23.y + (double)acc.w};
        *reinterpret_cast<double2 *>(S.x + r0) = make_double2(xn[0], xn[1]);
        *reinterpret_cast<double2 *>(S.x + r0 + 2) = make_double2(xn[2], xn[3]);
        if (S.df_resid) {
          float h[4], l[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) df_split(xn[q], h[q], l[q]);
          *reinterpret_cast<float4 *>(S.xs + r0) = make_float4(h[0], l[0], h[1], l[1]);
          *reinterpret_cast<float4 *>(S.xs + r0 + 2) = make_float4(h[2], l[2], h[3], l[3]);
        }
      }
      return;
    }
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < S.n; r += (long)gridDim.x * blockDim.x) {
      float acc = 0.0f;
      for (int kk = 0; kk < m; ++kk) acc = fmaf(cf32[kk], S.Z[(long)kk * S.ldv + r], acc);
      const double xn = S.x[r] + (double)acc;
      S.x[r] = xn;
      if (S.df_resid) {
        float h, l;
        df_split(xn, h, l);
        S.xs[r] = make_float2(h, l);
      }
    }
    return;
  }
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < S.n; r += (long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    if (S.pc == 2) {
      for (int kk = 0; kk < m; ++kk) acc = fma(cf[kk], (double)S.Z[(long)kk * S.ldv + r], acc);
      S.x[r] = S.x[r] + acc;
    } else {
      for (int kk = 0; kk < m; ++kk) acc = fma(cf[kk], S.V[(long)kk * S.ldv + r], acc);
      if (S.pc == 0) S.x[r] = fma(S.invd[r], acc, S.x[r]);
      else S.z[r] = acc;
    }
  }
}

__global__ void k_add_z(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  if (!S.s->cycle_end || S.pc != 1) return;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < S.n; r += (long)gridDim.x * blockDim.x)
    S.x[r] = S.x[r] + S.z2[r];
}

// Relative bound on the double-float residual of one row: |r_df - r| <=
// kDfRowBound * (|b| + sum_s |c_s x_s|). Per row the seven products carry
// about 3 * 2^-47 of their size (split of c and of x, rounded cross terms, the
// dropped lo * lo) and the eight double-float additions 2^-47 of the running
// sum each, about 2^-43.3 in all; 2^-41 leaves a factor of five.
constexpr double kDfRowBound = 4.547473508864641e-13;  // 2^-41

// True residual after a cycle; decide converged / stop / restart (V_0 = r).
// Systems with df_resid compute it in double-float and also the norm M of
// the per-row bounds; a decision closer to the tolerance than
// kDfRowBound * M is taken again from an FP64 residual, and the rest of the
// solve stays in FP64, so convergence is always decided within FP64 rounding.
__global__ void __launch_bounds__(kThreads) k_cycle_residual(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->cycle_end) return;
  const bool df = S.df_resid && !sc->use64;
  __shared__ double sacc[2 * kWarps];
  if (threadIdx.x < 2 * kWarps) sacc[threadIdx.x] = 0.0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (df) {
    // r = b - A x in double-float (about 48 bits) on the FP32 pipe, from the
    // double-float copy of x that the update wrote; |r|^2 and the squared
    // row bounds summed in FP32 per thread and FP64 across threads
    const long sy = S.nx, sz = (long)S.nx * S.ny;
    float pf = 0.0f, mf = 0.0f;  // per thread over all its rows
    for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
#pragma unroll
      for (int t = 0; t < kRowsPerThread; ++t) {
        const long r = t0 + t * kThreads + threadIdx.x;
        if (r < S.n) {
          int i, j, k;
          sys_ijk(r, S, i, j, k);
          const float *c = S.tabdf + 16 * (long)S.cls[r];
          float ah = 0.0f, al = 0.0f, mag = 0.0f;
          auto add = [&](int s, long q) {
            const float2 xv = S.xs[q];
            df_fma(ah, al, c[s], c[8 + s], xv.x, xv.y);
            mag = fmaf(fabsf(c[s]), fabsf(xv.x), mag);
          };
          add(0, r);
          if (i > 0) add(1, r - 1);
          if (i < S.nx - 1) add(2, r + 1);
          if (j > 0) add(3, r - sy);
          if (j < S.ny - 1) add(4, r + sy);
          if (k > 0) add(5, r - sz);
          if (k < S.nz - 1) add(6, r + sz);
          float bh, bl, rh, rl;
          df_split(S.b[r], bh, bl);
          df_sub(bh, bl, ah, al, rh, rl);
          S.Vf[r] = rh;
          pf = fmaf(rh, rh, pf);
          mag = 1.001f * (mag + fabsf(bh));  // the FP32 magnitudes' own rounding
          mf = fmaf(mag, mag, mf);
        }
      }
    }
    const double pr = warp_sum((double)pf), mr = warp_sum((double)mf);
    if (lane == 0) { sacc[warp] = pr; sacc[kWarps + warp] = mr; }
  } else {
  double pr = 0.0;  // per thread over all its rows
  for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
#pragma unroll
    for (int t = 0; t < kRowsPerThread; ++t) {
      const long r = t0 + t * kThreads + threadIdx.x;
      if (r < S.n) {
        int i, j, k;
        sys_ijk(r, S, i, j, k);
        long cs;
        const double *c0 = ar_row(S, r, cs);
        const double rv = S.b[r] - stencil7_at(c0, cs, S.x, (int)r, i, j, k, S.nx, S.ny, S.nz);
        if (S.a32) S.Vf[r] = (float)rv;
        else S.V[r] = rv;
        if (S.vcur) S.vcur[r] = (float)rv;
        pr = fma(rv, rv, pr);
      }
    }
  }
  pr = warp_sum(pr);
  if (lane == 0) sacc[warp] = pr;
  }
  if (!block_partials_and_last(sacc, 2, S.part, &sc->ticket)) return;
  __shared__ double tot[2];
  reduce_partials(S.part, gridDim.x, 2, tot);
  __syncthreads();
  if (threadIdx.x == 0) {
    sc->ticket = 0;
    const double rt = sqrt(tot[0]);
    sc->cycle_end = 0;
    sc->r_norm = rt;
    if (!isfinite(rt)) { sc->nonfinite = 1; sc->status = 2; sc->active = 0; return; }
    if (df) {
      const double bound = kDfRowBound * sqrt(tot[1]);
      if (rt + bound <= sc->eps) { sc->status = 1; sc->active = 0; return; }
      if (rt - bound <= sc->eps) {
        // too close to call: the next cycle end (no update, i = 0) computes the
        // FP64 residual of the same x
        sc->use64 = 1;
        sc->cycle_end = 1;
        sc->i = 0;
        return;
      }
    } else if (rt <= sc->eps) {
      sc->status = 1; sc->active = 0; return;
    }
    if (sc->iters >= sc->maxit) { sc->status = 2; sc->active = 0; return; }
    if (sc->claimed && rt >= sc->real_old) { sc->status = 3; sc->active = 0; return; }
    sc->real_old = rt;
    sc->cyc_eps = fmax(sc->eps, sc->cyc_rtol * rt);
    sc->i = 0;
    sc->claimed = 0;
    sc->nu[0] = rt;
    sc->g[0] = rt;
    sc->active = 1;
  }
}

// ---------------------------------------------------------------------------
// FP32 Arnoldi cycles (a32 systems, flexible form only). The same three steps
// on an FP32 basis: the operator is the FP32 copy, products and per-thread
// sums are FP32, sums across threads and blocks and every scalar are FP64.
// A cycle stops once its estimate fell by cyc_rtol; the restart computes the
// true residual in FP64, so the solve still meets the FP64 tolerance.

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float f4(const float4 &v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(kThreads) k_arnoldi_spmv32(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->active || !S.a32) return;
  const int j = sc->i, nd = j + 1;
  __shared__ double sacc[(kMaxKdim + 1) * kWarps];
  for (int t = threadIdx.x; t < nd * kWarps; t += blockDim.x) sacc[t] = 0.0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float *zj = S.Z + (long)j * S.ldv;
  if (nd <= kChunk32 && S.vec4) {
    // four consecutive rows per thread: coefficient planes, w and the basis
    // move as 16-byte vectors; the stencil of each row is stencil7_row_f's
    float acc[kChunk32];
#pragma unroll
    for (int kk = 0; kk < kChunk32; ++kk) acc[kk] = 0.0f;
    const long n = S.n, sy = S.nx, sz = (long)S.nx * S.ny;
    for (long t0 = (long)blockIdx.x * kTile; t0 < n; t0 += (long)gridDim.x * kTile) {
      const long r0 = t0 + 4 * threadIdx.x;
      if (r0 >= n) continue;
      float4 cp[7];
      if (S.cls) {
        load_rows4(S.tabf, __ldcs(reinterpret_cast<const ushort4 *>(S.cls + r0)), cp);
      } else {
#pragma unroll
        for (int q = 0; q < 7; ++q) cp[q] = __ldcs(reinterpret_cast<const float4 *>(S.Af + (long)q * n + r0));
      }
      float w[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const long r = r0 + q;
        int i, jj, k;
        sys_ijk(r, S, i, jj, k);
        float a = 0.0f;
        a = fmaf(f4(cp[0], q), zj[r], a);
        a = fmaf(f4(cp[1], q), i > 0 ? zj[r - 1] : 0.0f, a);
        a = fmaf(f4(cp[2], q), i < S.nx - 1 ? zj[r + 1] : 0.0f, a);
        a = fmaf(f4(cp[3], q), jj > 0 ? zj[r - sy] : 0.0f, a);
        a = fmaf(f4(cp[4], q), jj < S.ny - 1 ? zj[r + sy] : 0.0f, a);
        a = fmaf(f4(cp[5], q), k > 0 ? zj[r - sz] : 0.0f, a);
        a = fmaf(f4(cp[6], q), k < S.nz - 1 ? zj[r + sz] : 0.0f, a);
        w[q] = a;
      }
      st4(S.wf + r0, make_float4(w[0], w[1], w[2], w[3]));
#pragma unroll
      for (int kk = 0; kk < kChunk32; ++kk) {
        if (kk < nd) {
          const float4 v = ld4(S.Vf + (long)kk * S.ldv + r0);
          acc[kk] = fmaf(v.x, w[0], acc[kk]);
          acc[kk] = fmaf(v.y, w[1], acc[kk]);
          acc[kk] = fmaf(v.z, w[2], acc[kk]);
          acc[kk] = fmaf(v.w, w[3], acc[kk]);
        }
      }
    }
#pragma unroll
    for (int kk = 0; kk < kChunk32; ++kk) {
      if (kk >= nd) break;
      const float p = warp_sum_f(acc[kk]);
      if (lane == 0) sacc[kk * kWarps + warp] = (double)p;
    }
  } else
  if (nd <= kChunk32) {
    // short basis: every dot product of the thread stays in a register
    // across the whole sweep, one warp reduction per dot at the end
    float acc[kChunk32];
#pragma unroll
    for (int kk = 0; kk < kChunk32; ++kk) acc[kk] = 0.0f;
    for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
#pragma unroll
      for (int t = 0; t < kRowsPerThread; ++t) {
        const long r = t0 + t * kThreads + threadIdx.x;
        if (r < S.n) {
          int i, jj, k;
          sys_ijk(r, S, i, jj, k);
          long cs;
          const float *c0 = af_row(S, r, cs);
          const float w = stencil7_at_f(c0, cs, zj, (int)r, i, jj, k, S.nx, S.ny, S.nz);
          S.wf[r] = w;
#pragma unroll
          for (int kk = 0; kk < kChunk32; ++kk)
            if (kk < nd) acc[kk] = fmaf(S.Vf[(long)kk * S.ldv + r], w, acc[kk]);
        }
      }
    }
#pragma unroll
    for (int kk = 0; kk < kChunk32; ++kk) {
      if (kk >= nd) break;
      const float p = warp_sum_f(acc[kk]);
      if (lane == 0) sacc[kk * kWarps + warp] = (double)p;
    }
  } else
  for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
    float wv[kRowsPerThread];
#pragma unroll
    for (int t = 0; t < kRowsPerThread; ++t) {
      const long r = t0 + t * kThreads + threadIdx.x;
      wv[t] = 0.0f;
      if (r < S.n) {
        int i, jj, k;
        sys_ijk(r, S, i, jj, k);
        long cs;
        const float *c0 = af_row(S, r, cs);
        const float w = stencil7_at_f(c0, cs, zj, (int)r, i, jj, k, S.nx, S.ny, S.nz);
        S.wf[r] = w;
        wv[t] = w;
      }
    }
    for (int kk = 0; kk < nd; ++kk) {
      const float *vk = S.Vf + (long)kk * S.ldv;
      float p = 0.0f;
#pragma unroll
      for (int t = 0; t < kRowsPerThread; ++t) {
        const long r = t0 + t * kThreads + threadIdx.x;
        if (r < S.n) p = fmaf(vk[r], wv[t], p);
      }
      p = warp_sum_f(p);
      if (lane == 0) sacc[kk * kWarps + warp] += (double)p;
    }
  }
  if (!block_partials_and_last(sacc, nd, S.part, &sc->ticket)) return;
  __shared__ double tot[kMaxKdim + 1];
  reduce_partials(S.part, gridDim.x, nd, tot);
  __syncthreads();
  for (int kk = threadIdx.x; kk < nd; kk += blockDim.x) {
    const double h = tot[kk] / sc->nu[kk];
    sc->h1[kk] = h;
    sc->coef[kk] = h / sc->nu[kk];
  }
  if (threadIdx.x == 0) sc->ticket = 0;
}

__global__ void __launch_bounds__(kThreads) k_arnoldi_orth32(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->active || !S.a32) return;
  const int j = sc->i, nd = j + 1;
  __shared__ double sacc[(kMaxKdim + 1) * kWarps];
  __shared__ float cf[kMaxKdim + 1];
  for (int t = threadIdx.x; t < nd * kWarps; t += blockDim.x) sacc[t] = 0.0;
  for (int t = threadIdx.x; t < nd; t += blockDim.x) cf[t] = (float)sc->coef[t];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (nd <= kChunk32 && S.vec4) {
    float acc[kChunk32];
#pragma unroll
    for (int kk = 0; kk < kChunk32; ++kk) acc[kk] = 0.0f;
    for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
      const long r0 = t0 + 4 * threadIdx.x;
      if (r0 >= S.n) continue;
      float4 v[kChunk32];
#pragma unroll
      for (int kk = 0; kk < kChunk32; ++kk)
        v[kk] = kk < nd ? ld4(S.Vf + (long)kk * S.ldv + r0) : make_float4(0.f, 0.f, 0.f, 0.f);
      float4 w = ld4(S.wf + r0);
#pragma unroll
      for (int kk = 0; kk < kChunk32; ++kk) {
        if (kk < nd) {
          w.x = fmaf(-cf[kk], v[kk].x, w.x);
          w.y = fmaf(-cf[kk], v[kk].y, w.y);
          w.z = fmaf(-cf[kk], v[kk].z, w.z);
          w.w = fmaf(-cf[kk], v[kk].w, w.w);
        }
      }
      st4(S.wf + r0, w);
#pragma unroll
      for (int kk = 0; kk < kChunk32; ++kk) {
        acc[kk] = fmaf(v[kk].x, w.x, acc[kk]);
        acc[kk] = fmaf(v[kk].y, w.y, acc[kk]);
        acc[kk] = fmaf(v[kk].z, w.z, acc[kk]);
        acc[kk] = fmaf(v[kk].w, w.w, acc[kk]);
      }
    }
#pragma unroll
    for (int kk = 0; kk < kChunk32; ++kk) {
      if (kk >= nd) break;
      const float p = warp_sum_f(acc[kk]);
      if (lane == 0) sacc[kk * kWarps + warp] = (double)p;
    }
  } else
  if (nd <= kChunk32) {
    // short basis: each basis value is loaded once for the update and the dots
    float acc[kChunk32];
#pragma unroll
    for (int kk = 0; kk < kChunk32; ++kk) acc[kk] = 0.0f;
    for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
#pragma unroll
      for (int t = 0; t < kRowsPerThread; ++t) {
        const long r = t0 + t * kThreads + threadIdx.x;
        if (r < S.n) {
          float v[kChunk32];
#pragma unroll
          for (int kk = 0; kk < kChunk32; ++kk) v[kk] = kk < nd ? S.Vf[(long)kk * S.ldv + r] : 0.0f;
          float w = S.wf[r];
#pragma unroll
          for (int kk = 0; kk < kChunk32; ++kk)
            if (kk < nd) w = fmaf(-cf[kk], v[kk], w);
          S.wf[r] = w;
#pragma unroll
          for (int kk = 0; kk < kChunk32; ++kk) acc[kk] = fmaf(v[kk], w, acc[kk]);
        }
      }
    }
#pragma unroll
    for (int kk = 0; kk < kChunk32; ++kk) {
      if (kk >= nd) break;
      const float p = warp_sum_f(acc[kk]);
      if (lane == 0) sacc[kk * kWarps + warp] = (double)p;
    }
  } else
  for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
    float wv[kRowsPerThread];
#pragma unroll
    for (int t = 0; t < kRowsPerThread; ++t) {
      const long r = t0 + t * kThreads + threadIdx.x;
      wv[t] = 0.0f;
      if (r < S.n) {
        float w = S.wf[r];
        for (int kk = 0; kk < nd; ++kk) w = fmaf(-cf[kk], S.Vf[(long)kk * S.ldv + r], w);
        S.wf[r] = w;
        wv[t] = w;
      }
    }
    for (int kk = 0; kk < nd; ++kk) {
      float p = 0.0f;
#pragma unroll
      for (int t = 0; t < kRowsPerThread; ++t) {
        const long r = t0 + t * kThreads + threadIdx.x;
        if (r < S.n) p = fmaf(S.Vf[(long)kk * S.ldv + r], wv[t], p);
      }
      p = warp_sum_f(p);
      if (lane == 0) sacc[kk * kWarps + warp] += (double)p;
    }
  }
  if (!block_partials_and_last(sacc, nd, S.part, &sc->ticket)) return;
  __shared__ double tot[kMaxKdim + 1];
  reduce_partials(S.part, gridDim.x, nd, tot);
  __syncthreads();
  for (int kk = threadIdx.x; kk < nd; kk += blockDim.x) {
    const double h2 = tot[kk] / sc->nu[kk];
    sc->coef[kk] = h2 / sc->nu[kk];
    sc->H[kk * kMaxKdim + j] = sc->h1[kk] + h2;
  }
  if (threadIdx.x == 0) sc->ticket = 0;
}

__global__ void __launch_bounds__(kThreads) k_arnoldi_next32(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->active || !S.a32) return;
  const int j = sc->i, nd = j + 1;
  __shared__ float cf[kMaxKdim + 1];
  __shared__ double sacc[kWarps];
  for (int t = threadIdx.x; t < nd; t += blockDim.x) cf[t] = (float)sc->coef[t];
  if (threadIdx.x < kWarps) sacc[threadIdx.x] = 0.0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *vn = S.Vf + (long)nd * S.ldv;
  const bool store = nd < sc->kdim;
  // |w|^2: FP32 per thread (as the dot products of the FP32 cycle), FP64 across threads
  float pt = 0.0f;
  if (nd <= kChunk32 && S.vec4) {
    for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
      const long r0 = t0 + 4 * threadIdx.x;
      if (r0 >= S.n) continue;
      float4 w = ld4(S.wf + r0);
#pragma unroll
      for (int kk = 0; kk < kChunk32; ++kk) {
        if (kk < nd) {
          const float4 v = ld4(S.Vf + (long)kk * S.ldv + r0);
          w.x = fmaf(-cf[kk], v.x, w.x);
          w.y = fmaf(-cf[kk], v.y, w.y);
          w.z = fmaf(-cf[kk], v.z, w.z);
          w.w = fmaf(-cf[kk], v.w, w.w);
        }
      }
      if (store) st4(vn + r0, w);
      pt = fmaf(w.x, w.x, pt);
      pt = fmaf(w.y, w.y, pt);
      pt = fmaf(w.z, w.z, pt);
      pt = fmaf(w.w, w.w, pt);
    }
  } else
  for (long t0 = (long)blockIdx.x * kTile; t0 < S.n; t0 += (long)gridDim.x * kTile) {
#pragma unroll
    for (int t = 0; t < kRowsPerThread; ++t) {
      const long r = t0 + t * kThreads + threadIdx.x;
      if (r < S.n) {
        float w = S.wf[r];
        if (nd <= kChunk32) {
          float v[kChunk32];
#pragma unroll
          for (int kk = 0; kk < kChunk32; ++kk) v[kk] = kk < nd ? S.Vf[(long)kk * S.ldv + r] : 0.0f;
#pragma unroll
          for (int kk = 0; kk < kChunk32; ++kk)
            if (kk < nd) w = fmaf(-cf[kk], v[kk], w);
        } else {
          for (int kk = 0; kk < nd; ++kk) w = fmaf(-cf[kk], S.Vf[(long)kk * S.ldv + r], w);
        }
        if (store) vn[r] = w;
        pt = fmaf(w, w, pt);
      }
    }
  }
  const double ptd = warp_sum((double)pt);
  if (lane == 0) sacc[warp] = ptd;
  if (!block_partials_and_last(sacc, 1, S.part, &sc->ticket)) return;
  __shared__ double tot[1];
  reduce_partials(S.part, gridDim.x, 1, tot);
  __syncthreads();
  if (threadIdx.x == 0) {
    sc->ticket = 0;
    arnoldi_finalize(sc, j, sqrt(tot[0]));
  }
}

// Two FP32 Jacobi sweeps from zero in one pass (momentum preconditioner of
// the flexible form): z = D^-1 (2v - A D^-1 v) = D^-1 (v - sum over the
// couplings of (A D^-1)_s v_s), with v = V_j / nu_j; A D^-1 is stored (cjf), so
// the pass reads v, the six scaled couplings and D^-1 once.
template <class VT>
__device__ __forceinline__ void jacobi_two_rows(const KSys &S, const VT *__restrict__ vj, float inv_nu,
                                                float *__restrict__ out) {
  const long n = S.n, sy = S.nx, sz = (long)S.nx * S.ny;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    int i, jj, k;
    sys_ijk(r, S, i, jj, k);
    // slot s (1..6) of the scaled couplings at cj[s * cs], D^-1 at id
    const float *cj, *id;
    long cs;
    if (S.clsj) { cj = S.tabj + 8 * (long)S.clsj[r]; cs = 1; id = cj; }
    else { cj = S.Ajf + r; cs = n; id = S.invdf + r; }
    float acc = (float)vj[r] * inv_nu;
    if (i > 0) acc = fmaf(-cj[cs], (float)vj[r - 1] * inv_nu, acc);
    if (i < S.nx - 1) acc = fmaf(-cj[2 * cs], (float)vj[r + 1] * inv_nu, acc);
    if (jj > 0) acc = fmaf(-cj[3 * cs], (float)vj[r - sy] * inv_nu, acc);
    if (jj < S.ny - 1) acc = fmaf(-cj[4 * cs], (float)vj[r + sy] * inv_nu, acc);
    if (k > 0) acc = fmaf(-cj[5 * cs], (float)vj[r - sz] * inv_nu, acc);
    if (k < S.nz - 1) acc = fmaf(-cj[6 * cs], (float)vj[r + sz] * inv_nu, acc);
    out[r] = *id * acc;
  }
}

// The same, four consecutive rows per thread with 16-byte loads of the
// coefficient planes and stores of z (FP32 basis, n % 4 == 0).
__device__ __forceinline__ void jacobi_two_rows4(const KSys &S, const float *__restrict__ vj, float inv_nu,
                                                 float *__restrict__ out) {
  const long n = S.n, sy = S.nx, sz = (long)S.nx * S.ny;
  for (long r0 = 4 * ((long)blockIdx.x * blockDim.x + threadIdx.x); r0 < n; r0 += 4L * gridDim.x * blockDim.x) {
    float4 cp[7];
    float4 id;
    if (S.clsj) {
      // class records {invdf, Ajf_1..Ajf_6, 0}: slot 0 is D^-1
      load_rows4(S.tabj, __ldcs(reinterpret_cast<const ushort4 *>(S.clsj + r0)), cp);
      id = cp[0];
    } else {
#pragma unroll
      for (int q = 1; q < 7; ++q) cp[q] = __ldcs(reinterpret_cast<const float4 *>(S.Ajf + (long)q * n + r0));
      id = __ldcs(reinterpret_cast<const float4 *>(S.invdf + r0));
    }
    float z[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long r = r0 + q;
      int i, jj, k;
      sys_ijk(r, S, i, jj, k);
      float acc = vj[r] * inv_nu;
      if (i > 0) acc = fmaf(-f4(cp[1], q), vj[r - 1] * inv_nu, acc);
      if (i < S.nx - 1) acc = fmaf(-f4(cp[2], q), vj[r + 1] * inv_nu, acc);
      if (jj > 0) acc = fmaf(-f4(cp[3], q), vj[r - sy] * inv_nu, acc);
      if (jj < S.ny - 1) acc = fmaf(-f4(cp[4], q), vj[r + sy] * inv_nu, acc);
      if (k > 0) acc = fmaf(-f4(cp[5], q), vj[r - sz] * inv_nu, acc);
      if (k < S.nz - 1) acc = fmaf(-f4(cp[6], q), vj[r + sz] * inv_nu, acc);
      z[q] = f4(id, q) * acc;
    }
    *reinterpret_cast<float4 *>(out + r0) = make_float4(z[0], z[1], z[2], z[3]);
  }
}

__global__ void __launch_bounds__(kThreads) k_jacobi32_two(KSys *sys) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->active || S.pc != 2 || S.pc_cb) return;
  const int j = sc->i;
  const float inv_nu = (float)(1.0 / sc->nu[j]);
  float *out = S.Z + (long)j * S.ldv;
  // an FP64 basis is read through its FP32 copy when there is one: the same
  // values ((float) V_j), one conversion per row where the vector is formed
  // instead of one per row and neighbour here
  const float *vf = S.a32 ? S.Vf + (long)j * S.ldv : S.vcur;
  if (vf && S.vec4) jacobi_two_rows4(S, vf, inv_nu, out);
  else if (vf) jacobi_two_rows<float>(S, vf, inv_nu, out);
  else jacobi_two_rows<double>(S, S.V + (long)j * S.ldv, inv_nu, out);
}

// FP32 inner preconditioner for the flexible form: zf = D^-1 v (v = V_j / nu_j),
// then `sweeps-1` Jacobi sweeps zf <- zf + D^-1 (v - A zf); result to Z_j.
__global__ void __launch_bounds__(kThreads) k_jacobi32_first(KSys *sys, int to_z) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->active || S.pc != 2 || S.pc_cb) return;
  const int j = sc->i;
  const double inv_nu = 1.0 / sc->nu[j];
  const double *vj = S.V + (long)j * S.ldv;
  const float *vjf = S.Vf + (long)j * S.ldv;
  float *out = to_z ? S.Z + (long)j * S.ldv : S.zf;
  if (S.vcur) {  // FP64 basis through its FP32 copy: no FP64 instruction
    const float inv_nuf = (float)inv_nu;
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < S.n; r += (long)gridDim.x * blockDim.x)
      out[r] = (S.vcur[r] * inv_nuf) * S.invdf[r];
    return;
  }
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < S.n; r += (long)gridDim.x * blockDim.x)
    out[r] = (float)((S.a32 ? (double)vjf[r] : vj[r]) * inv_nu) * S.invdf[r];
}

__global__ void __launch_bounds__(kThreads) k_jacobi32_sweep(KSys *sys, int src_is_zf, int to_z) {
  KSys &S = sys[blockIdx.y];
  KScal *sc = S.s;
  if (!sc->active || S.pc != 2 || S.pc_cb) return;
  const int j = sc->i;
  const double inv_nu = 1.0 / sc->nu[j];
  const double *vj = S.V + (long)j * S.ldv;
  const float *vjf = S.Vf + (long)j * S.ldv;
  const float *src = src_is_zf ? S.zf : S.zf2;
  float *dst = to_z ? S.Z + (long)j * S.ldv : (src_is_zf ? S.zf2 : S.zf);
  const float inv_nuf = (float)inv_nu;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < S.n; r += (long)gridDim.x * blockDim.x) {
    int i, jj, k;
    sys_ijk(r, S, i, jj, k);
    long cs;
    const float *c0 = af_row(S, r, cs);
    const float az = stencil7_at_f(c0, cs, src, (int)r, i, jj, k, S.nx, S.ny, S.nz);
    const float v = S.vcur ? S.vcur[r] * inv_nuf : (float)((S.a32 ? (double)vjf[r] : vj[r]) * inv_nu);
    dst[r] = fmaf(S.invdf[r], v - az, src[r]);
  }
}

__global__ void k_flags(KSys *sys, int nsys, KFlags *out) {
  const int t = threadIdx.x;
  if (t < nsys) {
    KScal *sc = sys[t].s;
    out[t].active = sc->active;
    out[t].cycle_end = sc->cycle_end;
    out[t].status = sc->status;
    out[t].iters = sc->iters;
    out[t].i = sc->i;
    out[t].nonfinite = sc->nonfinite;
    out[t].rel = sc->b_norm > 0.0 ? sc->r_norm / sc->b_norm : sc->r_norm;
  }
}

// Loop control of the graph form: WHILE runs while any system is active or
// has a finished cycle to close; the SWITCH picks the cycle-end body (0) when
// any system closed a cycle, else the Arnoldi body (1).
__global__ void k_set_while(KSys *sys, int nsys, cudaGraphConditionalHandle hw) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned run = 0;
  for (int s = 0; s < nsys; ++s) run |= (sys[s].s->active | sys[s].s->cycle_end) ? 1u : 0u;
  cudaGraphSetConditional(hw, run);
}

__global__ void k_set_switch(KSys *sys, int nsys, cudaGraphConditionalHandle hs, unsigned long long *loops) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int end = 0;
  for (int s = 0; s < nsys; ++s) end |= sys[s].s->cycle_end;
  cudaGraphSetConditional(hs, end ? 0u : 1u);
  loops[end ? 0 : 1] += 1;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
void Krylov::configure(int nsys_, const KSysHost *hs) {
  if (nsys_ < 1 || nsys_ > kMaxSys) throw Error(IBM_ERR_ARG, "Krylov: bad system count");
  nsys = nsys_;
  int maxn = 0;
  for (int s = 0; s < nsys; ++s) {
    if (hs[s].kdim < 1 || hs[s].kdim > kMaxKdim) throw Error(IBM_ERR_ARG, "GMRES restart length must be in [1, 63]");
    maxn = std::max(maxn, hs[s].n);
  }
  nblk = persistent_blocks(maxn, 4);
  // the FP32 SpMV + dots kernel holds 80 registers (three blocks per SM): a
  // grid of as many blocks as stay resident runs in one wave
  {
    int per_sm = 0;
    IBM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_arnoldi_spmv32, kThreads, 0));
    nblk_spmv32 = std::max(1, std::min(nblk, std::max(1, per_sm) * sm_count()));
  }
  const size_t need_part = (size_t)nblk * (kMaxKdim + 2);
  for (int s = 0; s < nsys; ++s) {
    const KSysHost &h = hs[s];
    Slot &sl = slot[s];
    sl.host = h;
    if (h.a32 && h.pc != 2) throw Error(IBM_ERR_ARG, "Krylov: FP32 cycles need the flexible form");
    if (h.a32) {
      sl.V.release(); sl.w.release();
      sl.Vf.alloc((size_t)(h.kdim + 1) * h.n);
      sl.wf.alloc(h.n);
    } else {
      sl.Vf.release(); sl.wf.release();
      sl.V.alloc((size_t)(h.kdim + 1) * h.n);
      sl.w.alloc(h.n);
    }
    if (h.pc == 1) { sl.z.alloc(h.n); sl.z2.alloc(h.n); }
    if (h.a32 && h.cls && h.tabdf && h.df_residual) sl.xs.alloc(h.n);
    else sl.xs.release();
    if (h.pc == 2) {
      sl.Z.alloc((size_t)h.kdim * h.n);
      if (!h.pc_cb) { sl.zf.alloc(h.n); sl.zf2.alloc(h.n); }
    }
    if (h.pc == 2 && !h.pc_cb && !h.a32) sl.vcur.alloc(h.n);
    else sl.vcur.release();
    sl.part.alloc(need_part);
  }
  scal.alloc(nsys);
  dsys.alloc(nsys);
  dflags.alloc(nsys);
  if (!hflags) IBM_CUDA_TRY(cudaMallocHost((void **)&hflags, sizeof(KFlags) * kMaxSys));
}

size_t Krylov::bytes() const {
  size_t b = 0;
  for (int s = 0; s < nsys; ++s) {
    const Slot &sl = slot[s];
    b += sl.V.bytes() + sl.w.bytes() + sl.z.bytes() + sl.z2.bytes() + sl.part.bytes() +
         sl.Z.bytes() + sl.zf.bytes() + sl.zf2.bytes() + sl.Vf.bytes() + sl.wf.bytes() + sl.xs.bytes() +
         sl.vcur.bytes();
  }
  return b;
}

Krylov::~Krylov() {
  if (hflags) cudaFreeHost(hflags);
}

void Krylov::bind(cudaStream_t st, const double *const *b, double *const *x, unsigned mask, bool x_zero) {
  bound_mask = mask;
  bound_x_zero = x_zero;
  KSys hsys[kMaxSys];
  memset(hsys, 0, sizeof(hsys));
  for (int s = 0; s < nsys; ++s) {
    const KSysHost &h = slot[s].host;
    KSys &k = hsys[s];
    k.nx = h.nx; k.ny = h.ny; k.nz = h.nz; k.n = ((mask >> s) & 1u) ? h.n : 0;
    k.fdx = make_fastdiv((unsigned)h.nx); k.fdy = make_fastdiv((unsigned)h.ny);
    k.A = h.A; k.Ar = h.Ar; k.invd = h.invd; k.Af = h.Af; k.invdf = h.invdf; k.Ajf = h.Ajf;
    k.cls = h.cls; k.tab = h.tab; k.tabf = h.tabf; k.clsj = h.clsj; k.tabj = h.tabj;
    k.tabdf = h.tabdf;
    k.df_resid = (h.a32 && h.cls && h.tabdf && h.df_residual) ? 1 : 0;
    k.df_spmv = (h.pc == 2 && !h.a32 && h.cls && h.tabdf && h.A == h.Ar && h.df_spmv) ? 1 : 0;
    k.xs = slot[s].xs.p;
    k.V = slot[s].V.p; k.ldv = h.n;
    k.Z = slot[s].Z.p;
    k.w = slot[s].w.p; k.z = slot[s].z.p; k.z2 = slot[s].z2.p;
    k.zf = slot[s].zf.p; k.zf2 = slot[s].zf2.p;
    k.Vf = slot[s].Vf.p; k.wf = slot[s].wf.p; k.a32 = h.a32;
    k.vcur = slot[s].vcur.p;
    k.cgs1 = cgs1(h) ? 1 : 0;
    k.x_zero = x_zero ? 1 : 0;
    k.vec4 = (h.n % 4 == 0) ? 1 : 0;
    k.x = x[s]; k.b = b[s];
    k.part = slot[s].part.p;
    k.nblk = nblk;
    k.pc = h.pc;
    k.pc_cb = h.pc_cb;
    k.s = scal.p + s;
  }
  IBM_CUDA_TRY(cudaMemcpyAsync(dsys.p, hsys, sizeof(KSys) * nsys, cudaMemcpyHostToDevice, st));
  static KScal init[kMaxSys];
  memset(init, 0, sizeof(init));
  for (int s = 0; s < nsys; ++s) {
    init[s].kdim = slot[s].host.kdim;
    init[s].maxit = slot[s].host.maxit;
    init[s].tol = slot[s].host.tol;
    init[s].cyc_rtol = slot[s].host.a32 ? slot[s].host.cycle_rtol : 0.0;
  }
  IBM_CUDA_TRY(cudaMemcpyAsync(scal.p, init, sizeof(KScal) * nsys, cudaMemcpyHostToDevice, st));
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
}

void Krylov::read_flags(cudaStream_t st) {
  {
    LaunchScope ls(K_GM_UPDATE, st, 0.0);
    k_flags<<<1, 32, 0, st>>>(dsys.p, nsys, dflags.p);
  }
  IBM_CUDA_TRY(cudaMemcpyAsync(hflags, dflags.p, sizeof(KFlags) * nsys, cudaMemcpyDeviceToHost, st));
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
}

// Algorithmic bytes per row (FP64 = 8): the operator's 7 coefficients, the
// vectors each kernel must read or write once, and the basis vectors it
// sweeps. In the graph form the flags are not known on the host and no
// bytes are attributed.
void Krylov::launch_cycle_end(cudaStream_t st, const Precond &pc, const KFlags *fl, unsigned mask) {
  const dim3 grid(nblk, nsys), gridu(nblk * 2, nsys);
  KSys *dev = dsys.p;
  auto rows = [&](int s) { return ((mask >> s) & 1u) ? (double)slot[s].host.n : 0.0; };
  double bu = 0.0, br = 0.0, ba = 0.0;
  if (fl) {
    for (int s = 0; s < nsys; ++s) {
      if (!fl[s].cycle_end) continue;
      const int m = fl[s].i, pcm = slot[s].host.pc;
      bu += rows(s) * (pcm == 2 ? 4.0 * m + 16.0 : pcm == 1 ? 8.0 * m + 8.0 : 8.0 * m + 24.0);
      // a classed row is its 2-byte class instead of 7 FP64 coefficients
      br += ((slot[s].host.cls ? 34.0 : 88.0) + (slot[s].vcur.p ? 4.0 : 0.0)) * rows(s);
      if (pcm == 1) ba += 24.0 * rows(s);
    }
  }
  {
    LaunchScope ls(K_GM_UPDATE, st, bu);
    k_cycle_update<<<wave(k_cycle_update), kThreads, 0, st>>>(dev);
  }
  bool cb = false;
  for (int s = 0; s < nsys; ++s) {
    if (slot[s].host.pc != 1 || !((mask >> s) & 1u) || (fl && !fl[s].cycle_end)) continue;
    VecRef in;
    in.base = slot[s].z.p;
    OutRef out;
    out.d = slot[s].z2.p;
    pc.apply(pc.ctx, st, s, in, out, &scal.p[s].cycle_end);
    cb = true;
  }
  if (cb) {
    LaunchScope ls(K_GM_ADDZ, st, ba);
    k_add_z<<<wave(k_add_z), kThreads, 0, st>>>(dev);
  }
  LaunchScope ls(K_GM_RESID, st, br);
  k_cycle_residual<<<wave(k_cycle_residual), kThreads, 0, st>>>(dev);
}

void Krylov::launch_arnoldi(cudaStream_t st, const Precond &pc, const KFlags *fl, unsigned mask) {
  const dim3 grid(nblk, nsys), gridu(nblk * 2, nsys);
  KSys *dev = dsys.p;
  auto rows = [&](int s) { return ((mask >> s) & 1u) ? (double)slot[s].host.n : 0.0; };
  for (int s = 0; s < nsys; ++s) {
    if (!((mask >> s) & 1u) || (fl && !fl[s].active)) continue;
    const KSysHost &h = slot[s].host;
    if (h.pc == 1) {
      VecRef in;
      in.base = slot[s].V.p; in.ld = h.n; in.idx = &scal.p[s].i;
      OutRef out;
      out.d = slot[s].z.p;
      pc.apply(pc.ctx, st, s, in, out, &scal.p[s].active);
    } else if (h.pc == 2 && h.pc_cb) {
      VecRef in;
      if (h.a32) in.basef = slot[s].Vf.p;
      else in.base = slot[s].V.p;
      in.ld = h.n; in.idx = &scal.p[s].i; in.nu = scal.p[s].nu;
      OutRef out;
      out.f = slot[s].Z.p; out.ld = h.n; out.idx = &scal.p[s].i;
      pc.apply(pc.ctx, st, s, in, out, &scal.p[s].active);
    }
  }
  int inner_sweeps = 0;
  bool any64 = false, any32 = false, any_orth = false;
  double r32 = 0.0, j32two = 0.0, bsp = 0.0, bor = 0.0, bor_orth = 0.0, bnx = 0.0, bsp32 = 0.0, bor32 = 0.0;
  for (int s = 0; s < nsys; ++s) {
    if (!((mask >> s) & 1u)) continue;
    const bool a32 = slot[s].host.a32 != 0;
    (a32 ? any32 : any64) = true;
    if (!a32 && !cgs1(slot[s].host)) any_orth = true;
    if (slot[s].host.pc == 2 && !slot[s].host.pc_cb && (!fl || fl[s].active))
      inner_sweeps = std::max(inner_sweeps, std::max(1, slot[s].host.inner_sweeps));
    if (!fl || !fl[s].active) continue;
    const double j1 = fl[s].i + 1.0;
    const KSysHost &h = slot[s].host;
    // coefficient bytes of a row: 7 values, or a 2-byte class
    const double c64 = (h.cls && h.A == h.Ar) ? 2.0 : 56.0, c32 = h.cls ? 2.0 : 28.0;
    if (h.pc == 2 && !h.pc_cb) {
      r32 += rows(s) * ((a32 || slot[s].vcur.p) ? 0.75 : 1.0);  // v read as FP32 or FP64
      // two sweeps in one pass: v, z and a 2-byte class instead of 7 FP32 values
      j32two += rows(s) * (h.clsj ? 10.0 : 27.0);  // v read as FP32 (basis or copy)
      if (!a32) bnx += 4.0 * rows(s);                // the copy, written by k_arnoldi_next
    }
    if (a32) {
      bsp32 += rows(s) * (c32 + 8.0 + 4.0 * j1);
      bor32 += rows(s) * (8.0 + 4.0 * j1);
    } else {
      bsp += rows(s) * ((h.pc == 2 ? 12.0 : 16.0) + c64 + 8.0 * j1);
      bor += rows(s) * (16.0 + 8.0 * j1);
      if (!cgs1(h)) bor_orth += rows(s) * (16.0 + 8.0 * j1);
    }
  }
  if (inner_sweeps > 0) {
    if (inner_sweeps == 2) {
      LaunchScope ls(K_GM_JAC32, st, j32two);
      k_jacobi32_two<<<wave(k_jacobi32_two), kThreads, 0, st>>>(dev);
    } else if (inner_sweeps == 1) {
      LaunchScope ls(K_GM_JAC32, st, 16.0 * r32);
      k_jacobi32_first<<<gridu, kThreads, 0, st>>>(dev, 1);
    } else {
      {
        LaunchScope ls(K_GM_JAC32, st, 16.0 * r32);
        k_jacobi32_first<<<gridu, kThreads, 0, st>>>(dev, 0);
      }
      int src_zf = 1;
      for (int q = 1; q < inner_sweeps; ++q) {
        LaunchScope ls(K_GM_JAC32, st, 48.0 * r32);
        k_jacobi32_sweep<<<gridu, kThreads, 0, st>>>(dev, src_zf, q == inner_sweeps - 1);
        src_zf ^= 1;
      }
    }
  }
  if (any64) {
    {
      LaunchScope ls(K_GM_SPMV, st, bsp);
      k_arnoldi_spmv<<<wave(k_arnoldi_spmv), kThreads, 0, st>>>(dev);
    }
    if (any_orth) {
      LaunchScope ls(K_GM_ORTH, st, bor_orth);
      k_arnoldi_orth<<<wave(k_arnoldi_orth), kThreads, 0, st>>>(dev);
    }
    LaunchScope ls(K_GM_NEXT, st, bor + bnx);
    k_arnoldi_next<<<wave(k_arnoldi_next), kThreads, 0, st>>>(dev);
  }
  if (any32) {
    {
      LaunchScope ls(K_GM_SPMV, st, bsp32);
      k_arnoldi_spmv32<<<wave(k_arnoldi_spmv32), kThreads, 0, st>>>(dev);
    }
    {
      LaunchScope ls(K_GM_ORTH, st, bor32);
      k_arnoldi_orth32<<<wave(k_arnoldi_orth32), kThreads, 0, st>>>(dev);
    }
    LaunchScope ls(K_GM_NEXT, st, bor32);
    k_arnoldi_next32<<<wave(k_arnoldi_next32), kThreads, 0, st>>>(dev);
  }
}

// Grid of a grid-stride Krylov kernel: (x, nsys) with x such that all blocks
// stay resident (one wave), at most nblk (the size of the partials).
template <class K>
dim3 Krylov::wave(K kernel) const {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
  const int x = std::max(1, std::min(nblk, std::max(1, per_sm) * sm_count() / std::max(1, nsys)));
  return dim3(x, nsys);
}

void Krylov::solve(cudaStream_t st, const double *const *b, double *const *x, const Precond &pc,
                   KResult *res, unsigned mask, bool x_zero) {
  bind(st, b, x, mask, x_zero);
  const dim3 grid(nblk, nsys);
  double init_bytes = 0.0;
  for (int s = 0; s < nsys; ++s)
    if ((mask >> s) & 1u)
      init_bytes += ((x_zero ? 16.0 : slot[s].host.cls ? 26.0 : 80.0) + (slot[s].vcur.p ? 4.0 : 0.0)) * slot[s].host.n;
  {
    LaunchScope ls(K_GM_INIT, st, init_bytes);
    k_init<<<wave(k_init), kThreads, 0, st>>>(dsys.p, nsys);
  }
  for (long guard = 0;; ++guard) {
    if (guard > 4L * 1000 * 1000) throw Error(IBM_ERR_CUDA, "GMRES host loop did not terminate");
    read_flags(st);
    bool any_active = false, any_end = false;
    for (int s = 0; s < nsys; ++s) {
      any_active |= hflags[s].active != 0;
      any_end |= hflags[s].cycle_end != 0;
    }
    if (!any_active && !any_end) break;
    if (any_end) launch_cycle_end(st, pc, hflags, mask);
    else launch_arnoldi(st, pc, hflags, mask);
  }
  for (int s = 0; s < nsys; ++s) {
    res[s].iters = hflags[s].iters;
    res[s].rel_res = hflags[s].rel;
    res[s].status = hflags[s].status;
    res[s].nonfinite = hflags[s].nonfinite;
  }
  IBM_CUDA_TRY(cudaGetLastError());
}

namespace {

// Adds a conditional node after the current dependencies of the capture on
// `st` and makes it the new dependency; returns its body graphs.
void add_conditional(cudaStream_t st, cudaGraphConditionalHandle *h, cudaGraphConditionalNodeType type,
                     unsigned size, cudaGraph_t *bodies) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *ed = nullptr;
  size_t nd = 0;
  IBM_CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &ed, &nd));
  if (cs != cudaStreamCaptureStatusActive) throw Error(IBM_ERR_STATE, "graph capture not active");
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = *h;
  p.conditional.type = type;
  p.conditional.size = size;
  cudaGraphNode_t node;
  IBM_CUDA_TRY(cudaGraphAddNode(&node, g, deps, ed, nd, &p));
  for (unsigned i = 0; i < size; ++i) bodies[i] = p.conditional.phGraph_out[i];
  IBM_CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
}

cudaGraph_t capture_graph_of(cudaStream_t st) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  IBM_CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
  return g;
}

template <class F>
long long capture_body(cudaGraph_t body, cudaStream_t bs, F &&fn) {
  const long long before = launches();
  IBM_CUDA_TRY(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  fn(bs);
  cudaGraph_t out = nullptr;
  IBM_CUDA_TRY(cudaStreamEndCapture(bs, &out));
  return launches() - before;
}

}  // namespace

Krylov::GraphCounts Krylov::enqueue_graph(cudaStream_t st, const cudaStream_t body_st[2], const Precond &pc,
                                          KFlags *host_flags, unsigned long long *loops) {
  GraphCounts gc;
  const long long t0 = launches();
  const dim3 grid(nblk, nsys);
  KSys *dev = dsys.p;
  const unsigned mask = bound_mask;
  {
    LaunchScope ls(K_GM_INIT, st, 0.0);
    k_init<<<wave(k_init), kThreads, 0, st>>>(dev, nsys);
  }
  cudaGraphConditionalHandle hw;
  IBM_CUDA_TRY(cudaGraphConditionalHandleCreate(&hw, capture_graph_of(st), 0, 0));
  {
    LaunchScope ls(K_GM_UPDATE, st, 0.0);
    k_set_while<<<1, 32, 0, st>>>(dev, nsys, hw);
  }
  cudaGraph_t wbody;
  add_conditional(st, &hw, cudaGraphCondTypeWhile, 1, &wbody);
  long long end_l = 0, arn_l = 0;
  const long long loop_l = capture_body(wbody, body_st[0], [&](cudaStream_t b0) {
    cudaGraphConditionalHandle hs;
    IBM_CUDA_TRY(cudaGraphConditionalHandleCreate(&hs, wbody, 0, 0));
    {
      LaunchScope ls(K_GM_UPDATE, b0, 0.0);
      k_set_switch<<<1, 32, 0, b0>>>(dev, nsys, hs, loops);
    }
    cudaGraph_t cases[2];
    add_conditional(b0, &hs, cudaGraphCondTypeSwitch, 2, cases);
    end_l = capture_body(cases[0], body_st[1], [&](cudaStream_t b1) { launch_cycle_end(b1, pc, nullptr, mask); });
    arn_l = capture_body(cases[1], body_st[1], [&](cudaStream_t b1) { launch_arnoldi(b1, pc, nullptr, mask); });
    LaunchScope ls(K_GM_UPDATE, b0, 0.0);
    k_set_while<<<1, 32, 0, b0>>>(dev, nsys, hw);
  });
  {
    LaunchScope ls(K_GM_UPDATE, st, 0.0);
    k_flags<<<1, 32, 0, st>>>(dev, nsys, dflags.p);
  }
  IBM_CUDA_TRY(cudaMemcpyAsync(host_flags, dflags.p, sizeof(KFlags) * nsys, cudaMemcpyDeviceToHost, st));
  const long long per_iter = loop_l - end_l - arn_l;  // the two control kernels
  gc.end_body = end_l + per_iter;
  gc.arnoldi_body = arn_l + per_iter;
  gc.fixed = (launches() - t0) - loop_l;
  gc.loop = loop_l;
  return gc;
}

}  // namespace ibm

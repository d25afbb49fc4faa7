// Batched restarted GMRES (see ibm_krylov.cu).
#pragma once
#include "ibm_common.cuh"

namespace ibm {

// A vector whose location is resolved on the device: base + (*idx) * ld,
// optionally scaled by 1 / nu[*idx] (the unnormalised Krylov basis).
struct VecRef {
  const double *base = nullptr;
  const float *basef = nullptr;  // FP32 source (used instead of base when set)
  long ld = 0;
  const int *idx = nullptr;
  const double *nu = nullptr;
};
struct OutRef {
  double *d = nullptr;  // FP64 destination, or
  float *f = nullptr;   // FP32 destination
  long ld = 0;
  const int *idx = nullptr;
};

// Preconditioner callback: out = M in, every kernel gated on *gate != 0.
struct Precond {
  void *ctx = nullptr;
  void (*apply)(void *ctx, cudaStream_t st, int sys, const VecRef &in, const OutRef &out, const int *gate) = nullptr;
};

struct KSysHost {
  int nx = 0, ny = 0, nz = 0, n = 0;
  const double *A = nullptr;    // Arnoldi operator ([7][n]); A*D^-1 when pc == 0
  const double *Ar = nullptr;   // operator of the true residual
  const double *invd = nullptr;
  const float *Af = nullptr, *invdf = nullptr;
  const float *Ajf = nullptr;   // FP32 A D^-1 (pc 2 with two internal Jacobi sweeps)
  int pc = 0;                   // 0 folded Jacobi, 1 explicit FP64 callback, 2 flexible FP32
  int pc_cb = 0;                // pc 2: 1 = callback, 0 = internal FP32 Jacobi sweeps
  int inner_sweeps = 1;
  int kdim = 50, maxit = 250;
  double tol = 1e-8;
  // pc 2 only: Arnoldi cycles in FP32 (FP32 basis, FP32 operator and dot
  // products per thread, FP64 scalars); each cycle stops once its estimate
  // fell by cycle_rtol and the restart recomputes the true residual in FP64.
  int a32 = 0;
  double cycle_rtol = 0.0;
  // record classes of the operator rows and of the Jacobi records (optional)
  const uint16_t *cls = nullptr;
  const double *tab = nullptr;
  const float *tabf = nullptr;
  const uint16_t *clsj = nullptr;
  const float *tabj = nullptr;
  const float *tabdf = nullptr;  // with a32: true residuals in double-float
  int df_residual = 1;           // use them when a32 and tabdf are set
  int df_spmv = 1;               // pc 2 without a32: A z_j in double-float from tabdf
  int arnoldi_passes = 2;        // pc 2 without a32: Gram-Schmidt passes per Arnoldi step (1 or 2)
};

// One classical Gram-Schmidt pass per Arnoldi step (no re-orthogonalisation):
// FP64 cycles of the flexible form when configured. The FP64 true residual
// at each cycle end still decides convergence.
inline bool cgs1(const KSysHost &h) { return h.pc == 2 && !h.a32 && h.arnoldi_passes == 1; }

struct KResult {
  int iters = 0;
  double rel_res = 0.0;
  int status = 0;   // 1 converged, 2 iteration limit, 3 stagnation
  int nonfinite = 0;
};

class Krylov {
 public:
  ~Krylov();
  void configure(int nsys, const KSysHost *systems);
  // mask: bit s set = solve system s (the others are skipped).
  // x_zero: the caller guarantees x = 0 on entry (the first residual is b).
  void solve(cudaStream_t st, const double *const *b, double *const *x, const Precond &pc, KResult *res,
             unsigned mask = ~0u, bool x_zero = false);
  size_t bytes() const;

  // Graph form. bind() fixes the vectors (outside any capture); enqueue_graph()
  // records the whole solve into the capture running on `st`: the restart /
  // Arnoldi loop is a WHILE node whose body SWITCHes between the cycle-end
  // and the Arnoldi-step bodies, captured on body_st[0] / body_st[1].
  // After the solve the per-system flags land in host_flags (pinned) and the
  // numbers of cycle-end / Arnoldi bodies run in loops[0] / loops[1].
  // Returns the launches recorded outside the loop and per body kind.
  struct GraphCounts { long long fixed = 0, end_body = 0, arnoldi_body = 0, loop = 0; };
  void bind(cudaStream_t st, const double *const *b, double *const *x, unsigned mask, bool x_zero = false);
  GraphCounts enqueue_graph(cudaStream_t st, const cudaStream_t body_st[2], const Precond &pc, KFlags *host_flags,
                            unsigned long long *loops);

 private:
  struct Slot {
    KSysHost host;
    DBuf<double> V, w, z, z2, part;
    DBuf<float> Z, zf, zf2, Vf, wf;
    DBuf<float> vcur;  // FP64 basis with FP32 Jacobi: FP32 copy of the current basis vector
    DBuf<float2> xs;  // double-float copy of x for the double-float residual
  };
  void read_flags(cudaStream_t st);
  template <class K>
  dim3 wave(K kernel) const;
  // Launch sequences shared by the host-driven and the graph form. With
  // flags == nullptr every launch is recorded (each kernel is gated on the
  // device flags of its system); otherwise only what the flags require.
  void launch_cycle_end(cudaStream_t st, const Precond &pc, const KFlags *flags, unsigned mask);
  void launch_arnoldi(cudaStream_t st, const Precond &pc, const KFlags *flags, unsigned mask);
  unsigned bound_mask = ~0u;
  bool bound_x_zero = false;
  int nsys = 0;
  int nblk = 0;
  int nblk_spmv32 = 0;
  Slot slot[kMaxSys];
  DBuf<KScal> scal;
  DBuf<KSys> dsys;
  DBuf<KFlags> dflags;
  KFlags *hflags = nullptr;
};

}  // namespace ibm

// Launch accounting: counts, algorithmic bytes per kernel class and per step
// phase, and CUDA-event timing of one selected kernel class.
#include "ibm_common.cuh"

namespace ibm {

static const char *kNames[K_COUNT] = {
    "bc", "momentum_rhs", "scatter", "pressure_rhs", "project", "diagnostics",
    "gmres_init", "gmres_spmv_dots", "gmres_orth", "gmres_next", "gmres_update", "gmres_residual", "gmres_add",
    "gmres_fp32_jacobi",
    "mg_load", "mg_relax", "mg_residual", "mg_restrict", "mg_prolong", "mg_dense", "mg_store",
    "mg_relax_fine", "mg_coarse", "adjoint", "setup"};

const char *kernel_name(int k) { return (k >= 0 && k < K_COUNT) ? kNames[k] : "?"; }

Prof *&current_prof() {
  static thread_local Prof *p = nullptr;
  return p;
}

void Prof::reset() {
  for (int k = 0; k < K_COUNT; ++k) { launches[k] = 0; bytes[k] = 0; ms[k] = 0; timed[k] = 0; }
  for (int q = 0; q < PH_COUNT; ++q) phase_bytes[q] = 0;
}

void Prof::drain() {
  for (const Pending &e : pending) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, e.a, e.b) == cudaSuccess) {
      ms[e.k] += t;
      timed[e.k] += 1;
    }
    pool.push_back(e.a);
    pool.push_back(e.b);
  }
  pending.clear();
}

Prof::~Prof() {
  for (auto e : pool) cudaEventDestroy(e);
  for (auto &e : pending) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
}

static cudaEvent_t take_event(Prof *p) {
  if (!p->pool.empty()) {
    cudaEvent_t e = p->pool.back();
    p->pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

LaunchScope::LaunchScope(KernelId k_, cudaStream_t st_, double b, long long n) : k(k_), st(st_) {
  count_launch(n);
  Prof *p = current_prof();
  if (!p) return;
  p->launches[k] += n;
  p->bytes[k] += b;
  p->phase_bytes[p->phase] += b;
  if (p->timed_kernel == (int)k) {
    Prof::Pending e{(int)k, take_event(p), take_event(p)};
    cudaEventRecord(e.a, st);
    p->pending.push_back(e);
    slot = (int)p->pending.size() - 1;
  }
}

LaunchScope::~LaunchScope() {
  Prof *p = current_prof();
  if (p && slot >= 0 && slot < (int)p->pending.size()) cudaEventRecord(p->pending[(size_t)slot].b, st);
}

}  // namespace ibm

// The C ABI of include/ibm_gpu.h: context lifecycle, conversion of the
// reference's inputs (row-major 7-point values, masks and 1-based ids,
// id-indexed vectors, 1-based CSR) into the device layouts the kernels use,
// solver wiring and the timestep.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "ibm_adjoint.cuh"
#include "ibm_assembly.cuh"
#include "ibm_ctx.cuh"
#include "ibm_step.cuh"

namespace ibm {

thread_local long long *g_counter = nullptr;
void count_launch(long long n) {
  if (g_counter) *g_counter += n;
}
long long launches() { return g_counter ? *g_counter : 0; }

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

int persistent_blocks(int rows, int per_sm) {
  const long tiles = ((long)rows + kTile - 1) / kTile;
  const long cap = (long)sm_count() * per_sm;
  return (int)std::max(1L, std::min(tiles, cap));
}

namespace {

struct Scope {
  long long *prev;
  Prof *prev_prof;
  explicit Scope(ibm_ctx *c) : prev(g_counter), prev_prof(current_prof()) {
    g_counter = &c->launches;
    current_prof() = &c->prof;
    cudaSetDevice(c->device);
  }
  ~Scope() {
    g_counter = prev;
    current_prof() = prev_prof;
  }
};

std::string g_create_error;

template <class F>
int guarded(ibm_ctx *c, F &&f) {
  if (!c) return IBM_ERR_ARG;
  Scope sc(c);
  try {
    c->err.clear();
    return f();
  } catch (const Error &e) {
    c->err = e.msg;
    return e.code;
  } catch (const std::exception &e) {
    c->err = e.what();
    return IBM_ERR_ARG;
  }
}

// Copy n elements from a host or device pointer into a host vector.
template <class T>
std::vector<T> to_host(const T *src, size_t n) {
  std::vector<T> h(n);
  if (n) IBM_CUDA_TRY(cudaMemcpy(h.data(), src, n * sizeof(T), cudaMemcpyDefault));
  return h;
}

template <class T>
void upload(DBuf<T> &dst, const std::vector<T> &h, cudaStream_t st) {
  dst.alloc(h.size());
  if (!h.empty()) IBM_CUDA_TRY(cudaMemcpyAsync(dst.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
}

// Row-major [n][7] -> planes [7][n], inverse diagonal, FP32 copies.
__global__ void k_op_planes(const double *vals, long n, double *c, double *invd, float *cf, float *invdf) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    for (int s = 0; s < 7; ++s) {
      const double v = vals[7 * r + s];
      c[(long)s * n + r] = v;
      cf[(long)s * n + r] = (float)v;
    }
    const double d = vals[7 * r];
    const double id = d != 0.0 ? 1.0 / d : 0.0;
    invd[r] = id;
    invdf[r] = (float)id;
  }
}

// Planes [7][n] -> row-major [n][7].
__global__ void k_planes_to_rows(const double *c, long n, double *rows) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    for (int s = 0; s < 7; ++s) rows[7 * r + s] = c[(long)s * n + r];
}

// Right-Jacobi-scaled operator: cj_s(r) = c_s(r) * invd(neighbour_s(r)).
__global__ void k_op_jacobi(const double *c, const double *invd, double *cj, Box b) {
  const long n = b.n, sy = b.nx, sz = (long)b.nx * b.ny;
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    int i, j, k;
    row_ijk((int)r, b.nx, b.ny, i, j, k);
    const long nb[7] = {r, i > 0 ? r - 1 : -1, i < b.nx - 1 ? r + 1 : -1, j > 0 ? r - sy : -1,
                        j < b.ny - 1 ? r + sy : -1, k > 0 ? r - sz : -1, k < b.nz - 1 ? r + sz : -1};
    for (int s = 0; s < 7; ++s) cj[(long)s * n + r] = nb[s] >= 0 ? c[(long)s * n + r] * invd[nb[s]] : 0.0;
  }
}

__global__ void k_to_float(const double *src, float *dst, long n) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    dst[t] = (float)src[t];
}

// Class rows [K][7] -> [K][8] (slot 7 zero), their FP32 copies and their
// double-float pairs [K][16] (hi = v rounded to FP32, lo = v - hi rounded).
__global__ void k_pad_rows(const double *rows7, int K, double *rows8, float *rows8f, float *rowsdf) {
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < 8L * K; e += (long)gridDim.x * blockDim.x) {
    const long c = e / 8;
    const int s = (int)(e - 8 * c);
    const double v = s < 7 ? rows7[7 * c + s] : 0.0;
    rows8[e] = v;
    const float hi = (float)v;
    rows8f[e] = hi;
    rowsdf[16 * c + s] = hi;
    rowsdf[16 * c + 8 + s] = (float)(v - (double)hi);
  }
}

// FP32 Jacobi records {invdf, cjf_1..cjf_6, 0} per row.
__global__ void k_jacobi_records(const float *cjf, const float *invdf, long n, float *rec) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    float *o = rec + 8 * r;
    o[0] = invdf[r];
    for (int s = 1; s < 7; ++s) o[s] = cjf[(long)s * n + r];
    o[7] = 0.0f;
  }
}

__global__ void k_spmv7(const double *c, Box b, const double *x, double *y) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < b.n; r += (long)gridDim.x * blockDim.x) {
    int i, j, k;
    row_ijk((int)r, b.nx, b.ny, i, j, k);
    y[r] = stencil7_row(c, b.n, x, (int)r, i, j, k, b.nx, b.ny, b.nz);
  }
}

int grid1d(long n) {
  long b = (n + kThreads - 1) / kThreads;
  return (int)std::max(1L, std::min(b, (long)sm_count() * 8));
}

// Diagonal symmetrizer of a 7-point operator (row-major values): W with
// A = W S, S symmetric. The cut-cell divergence of the pressure operator
// divides each cell's row by its open fraction, so the pressure operator has
// this form. Each connected set of coupled rows is walked breadth first from
// its lowest row (w = 1), neighbours in slot order, w_c = w_r A[c][r] / A[r][c];
// then every coupling is checked. Returns false (winv all ones) when A is not
// of that form. winv = 1 / w.
bool diagonal_symmetrizer(const std::vector<double> &A7, const Box &b, std::vector<double> &winv) {
  const long N = b.n;
  std::vector<double> w((size_t)N, 0.0);
  std::vector<long> queue((size_t)N);
  std::vector<unsigned char> seen((size_t)N, 0);
  const long sy = b.nx, sz = (long)b.nx * b.ny;
  const long off[7] = {0, -1, 1, -sy, sy, -sz, sz};
  static const int opp[7] = {0, 2, 1, 4, 3, 6, 5};
  auto inside = [&](long r, int s) {
    const int i = (int)(r % b.nx), j = (int)((r / b.nx) % b.ny), k = (int)(r / sz);
    switch (s) {
      case 1: return i > 0; case 2: return i < b.nx - 1; case 3: return j > 0; case 4: return j < b.ny - 1;
      case 5: return k > 0; case 6: return k < b.nz - 1; default: return true;
    }
  };
  bool ok = true;
  for (long root = 0; root < N && ok; ++root) {
    if (seen[root]) continue;
    seen[root] = 1;
    w[root] = 1.0;
    long head = 0, tail = 0;
    queue[tail++] = root;
    while (head < tail && ok) {
      const long r = queue[head++];
      for (int s = 1; s < 7; ++s) {
        if (!inside(r, s) || A7[7 * r + s] == 0.0) continue;
        const long c2 = r + off[s];
        const double back = A7[7 * c2 + opp[s]];
        if (back == 0.0) { ok = false; break; }
        if (seen[c2]) continue;
        seen[c2] = 1;
        w[c2] = w[r] * back / A7[7 * r + s];
        queue[tail++] = c2;
      }
    }
  }
  for (long r = 0; r < N && ok; ++r)
    for (int s = 1; s < 7; ++s) {
      if (!inside(r, s)) continue;
      const double x = A7[7 * r + s] / w[r], y = A7[7 * (r + off[s]) + opp[s]] / w[r + off[s]];
      if (std::fabs(x - y) > 1e-10 * std::max(std::fabs(x), std::fabs(y))) { ok = false; break; }
    }
  winv.assign((size_t)N, 1.0);
  if (ok)
    for (long r = 0; r < N; ++r) winv[r] = 1.0 / w[r];
  return ok;
}

const Box &field_box(const ibm_ctx *c, int f) {
  return f == 0 ? c->g.bu : f == 1 ? c->g.bv : f == 2 ? c->g.bw : c->g.bp;
}

void mg_apply_cb(void *ctx, cudaStream_t st, int, const VecRef &in, const OutRef &out, const int *gate) {
  ibm_ctx *c = (ibm_ctx *)ctx;
  c->mg.apply(st, in, out, gate, out.f != nullptr);
}

void require_inputs(ibm_ctx *c) {
  for (int f = 0; f < 4; ++f)
    if (!c->op[f].set) throw Error(IBM_ERR_STATE, "operator of field " + std::to_string(f) + " not set");
  if (!c->masks_set) throw Error(IBM_ERR_STATE, "masks not set");
  if (!c->aux_set) throw Error(IBM_ERR_STATE, "aux vectors not set");
  if (!c->csr_set) throw Error(IBM_ERR_STATE, "projection operators not set");
}

// Record classes of an operator's rows and Jacobi records, built once per
// set of coefficients (they stay empty where the rows do not repeat enough).
void ensure_classes(ibm_ctx *c, Op7 &o) {
  if (o.cls_tried) return;
  o.cls_tried = true;
  const long n = o.b.n;
  DBuf<double> rows;  // row-major [n][7] copy of the planes
  rows.alloc((size_t)7 * n);
  {
    LaunchScope ls(K_SETUP, c->st, 0.0);
    k_planes_to_rows<<<grid1d(n), kThreads, 0, c->st>>>(o.c.p, n, rows.p);
  }
  if (build_classes<double>(c->st, rows.p, 7, n, o.cls)) {
    o.tab.alloc((size_t)8 * o.cls.K);
    o.tabf.alloc((size_t)8 * o.cls.K);
    o.tabdf.alloc((size_t)16 * o.cls.K);
    LaunchScope ls(K_SETUP, c->st, 0.0);
    k_pad_rows<<<grid1d(8L * o.cls.K), kThreads, 0, c->st>>>(o.cls.tab.p, o.cls.K, o.tab.p, o.tabf.p, o.tabdf.p);
  }
  rows.release();
  DBuf<float> jrec;
  jrec.alloc((size_t)8 * n);
  {
    LaunchScope ls(K_SETUP, c->st, 0.0);
    k_jacobi_records<<<grid1d(n), kThreads, 0, c->st>>>(o.cjf.p, o.invdf.p, n, jrec.p);
  }
  build_classes<float>(c->st, jrec.p, 8, n, o.clsj);
  IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
}

// Points a system at its operator's classes.
void use_classes(const Op7 &o, KSysHost &h) {
  if (o.cls.ok()) { h.cls = o.cls.code.p; h.tab = o.tab.p; h.tabf = o.tabf.p; h.tabdf = o.tabdf.p; }
  if (o.clsj.ok()) { h.clsj = o.clsj.code.p; h.tabj = o.clsj.tab.p; }
}

// Precision key of the configured solvers: the pressure's and the momentum's.
int precision_key(const ibm_solver_params &p) {
  const int vp = p.vel_precision >= 0 ? p.vel_precision : p.precision;
  return 4 * p.precision + vp;
}

void ensure_solvers(ibm_ctx *c) {
  if (c->solvers_ready && c->solvers_precision == precision_key(c->prm)) return;
  const ibm_solver_params &p = c->prm;
  const bool mixed = p.precision >= 1;
  const int a32 = p.precision == 2;
  // the momentum solves may take another precision than the pressure solve
  const int vprec = p.vel_precision >= 0 ? p.vel_precision : p.precision;
  const bool vmixed = vprec >= 1;
  const int va32 = vprec == 2;
  if (!vmixed && p.vel_jacobi_iters != 1)
    throw Error(IBM_ERR_UNSUPPORTED, "FP64 momentum solves support one Jacobi sweep per application");
  KSysHost hs[3];
  for (int f = 0; f < 3; ++f) {
    const Op7 &o = c->op[f];
    KSysHost &h = hs[f];
    h.nx = o.b.nx; h.ny = o.b.ny; h.nz = o.b.nz; h.n = o.b.n;
    h.Ar = o.c.p;
    h.invd = o.invd.p;
    h.Af = o.cf.p; h.invdf = o.invdf.p; h.Ajf = o.cjf.p;
    h.kdim = p.vel_kdim; h.maxit = p.vel_maxit; h.tol = p.vel_tol;
    if (vmixed) {
      h.pc = 2; h.pc_cb = 0; h.A = o.c.p; h.inner_sweeps = std::max(1, p.vel_inner_sweeps);
      h.a32 = va32; h.cycle_rtol = p.cycle_rtol32; h.df_residual = p.df_residual;
      h.df_spmv = p.df_spmv; h.arnoldi_passes = p.arnoldi_passes;
    }
    else { h.pc = 0; h.A = o.cj.p; }
    if (p.row_classes) {
      ensure_classes(c, c->op[f]);
      use_classes(o, h);
    }
  }
  c->kmom.configure(3, hs);
  const Op7 &op = c->op[3];
  KSysHost hp;
  hp.nx = op.b.nx; hp.ny = op.b.ny; hp.nz = op.b.nz; hp.n = op.b.n;
  hp.Ar = op.c.p; hp.invd = op.invd.p; hp.Af = op.cf.p; hp.invdf = op.invdf.p;
  hp.kdim = p.p_kdim; hp.maxit = p.p_maxit; hp.tol = p.p_tol;
  if (p.p_pc == 1) {
    MgParams mp;
    mp.rap = p.p_pc_rap_type == 0 ? 0 : 1;
    mp.relax = p.p_pc_relax_type == 2 ? 2 : 1;
    mp.nu1 = p.mg_nu1; mp.nu2 = p.mg_nu2; mp.omega = p.mg_omega;
    mp.coarse_max = p.mg_coarse_max; mp.max_levels = p.mg_max_levels;
    mp.cycles = std::max(1, p.p_pc_maxit);
    mp.group_ratio = p.mg_group_ratio;
    mp.options = p.mg_options;
    mp.nu_coarse = p.mg_nu_coarse;
    mp.classes = p.row_classes ? 1 : 0;
    mp.quads = p.mg_quads ? 1 : 0;
    mp.fused_coarse = p.mg_fused_coarse == 1 ? 262144 : std::max(0, p.mg_fused_coarse);
    mp.fused_sweep = p.mg_fused_sweep ? 1 : 0;
    const double h[3] = {c->g.dx, c->g.dy, c->g.dz};
    const double *winv = ((p.mg_options & 2) && c->p_sym) ? c->p_winv.p : nullptr;
    c->mg.setup(c->st, op.b, op.c.p, op.cf.p, h, mp, true, mixed, winv);
    if (mixed) {
      hp.pc = 2; hp.pc_cb = 1; hp.A = op.c.p; hp.a32 = a32; hp.cycle_rtol = p.cycle_rtol32;
      hp.df_residual = p.df_residual; hp.df_spmv = p.df_spmv; hp.arnoldi_passes = p.arnoldi_passes;
    }
    else { hp.pc = 1; hp.A = op.c.p; }
  } else {
    if (mixed) {
      hp.pc = 2; hp.pc_cb = 0; hp.A = op.c.p; hp.inner_sweeps = 1;
      hp.a32 = a32; hp.cycle_rtol = p.cycle_rtol32; hp.df_residual = p.df_residual;
      hp.df_spmv = p.df_spmv; hp.arnoldi_passes = p.arnoldi_passes;
    }
    else { hp.pc = 0; hp.A = op.cj.p; }
  }
  if (p.row_classes) {
    ensure_classes(c, c->op[3]);
    use_classes(op, hp);
  }
  c->kp.configure(1, &hp);
  c->solvers_ready = true;
  c->solvers_precision = precision_key(p);
  c->graph_ready = false;
  c->graph_bound = false;
}

int worst(int a, int b) { return std::max(a, b); }

// HYPRE's GMRES returns success when it stops because the true residual no
// longer decreases (it only flags reaching max_iter above tolerance); the
// true relative residual is reported either way.
int solve_status(const KResult &r) {
  return (r.status == 1 || r.status == 3) ? IBM_OK : IBM_NOT_CONVERGED;
}

void invalidate_graph(ibm_ctx *c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  c->gexec = nullptr;
  c->graph_ready = false;
}

// Captures one timestep into c->gexec. Launch accounting during the capture
// goes to a scratch counter; per step it is the fixed launches plus the loop
// bodies the device ran (counted on the device).
void build_step_graph(ibm_ctx *c, const Precond &none, const Precond &mgp) {
  invalidate_graph(c);
  cudaStream_t st = c->st;
  Prof *saved_prof = current_prof();
  long long *saved_counter = g_counter;
  long long cap_count = 0;
  current_prof() = nullptr;
  g_counter = &cap_count;
  cudaGraph_t graph = nullptr;
  Krylov::GraphCounts gm, gp;
  try {
    IBM_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    IBM_CUDA_TRY(cudaMemcpyAsync(c->dramp.p, c->hramp, sizeof(double), cudaMemcpyHostToDevice, st));
    IBM_CUDA_TRY(cudaMemsetAsync(c->diag.p, 0, sizeof(StepDiag), st));
    IBM_CUDA_TRY(cudaMemsetAsync(c->dloops.p, 0, sizeof(unsigned long long) * 4, st));
    IBM_CUDA_TRY(cudaEventRecordWithFlags(c->ev[0], st, cudaEventRecordExternal));
    launch_bc(c, c->u.p, c->v.p, c->w.p);
    launch_momentum_rhs(c);
    IBM_CUDA_TRY(cudaEventRecordWithFlags(c->ev[1], st, cudaEventRecordExternal));
    gm = c->kmom.enqueue_graph(st, c->cap, none, c->hflags_graph, c->dloops.p);
    IBM_CUDA_TRY(cudaEventRecordWithFlags(c->ev[2], st, cudaEventRecordExternal));
    launch_tilde(c);
    launch_pressure_rhs(c);
    IBM_CUDA_TRY(cudaEventRecordWithFlags(c->ev[5], st, cudaEventRecordExternal));
    gp = c->kp.enqueue_graph(st, c->cap, mgp, c->hflags_graph + 3, c->dloops.p + 2);
    IBM_CUDA_TRY(cudaEventRecordWithFlags(c->ev[3], st, cudaEventRecordExternal));
    launch_projection(c);
    IBM_CUDA_TRY(cudaEventRecordWithFlags(c->ev[4], st, cudaEventRecordExternal));
    IBM_CUDA_TRY(cudaMemcpyAsync(c->hdiag, c->diag.p, sizeof(StepDiag), cudaMemcpyDeviceToHost, st));
    IBM_CUDA_TRY(cudaMemcpyAsync(c->hloops, c->dloops.p, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, st));
    IBM_CUDA_TRY(cudaStreamEndCapture(st, &graph));
  } catch (...) {
    cudaGraph_t junk = nullptr;
    cudaStreamEndCapture(st, &junk);
    if (junk) cudaGraphDestroy(junk);
    current_prof() = saved_prof;
    g_counter = saved_counter;
    throw;
  }
  current_prof() = saved_prof;
  g_counter = saved_counter;
  const cudaError_t e = cudaGraphInstantiate(&c->gexec, graph, 0);
  cudaGraphDestroy(graph);
  IBM_CUDA_TRY(e);
  c->graph_fixed_launches = cap_count - gm.loop - gp.loop;
  c->graph_body_launches[0] = gm.end_body;
  c->graph_body_launches[1] = gm.arnoldi_body;
  c->graph_body_launches[2] = gp.end_body;
  c->graph_body_launches[3] = gp.arnoldi_body;
  c->graph_ready = true;
}

void fill_solve(ibm_solve_stats &o, const KResult &r) {
  o.iters = r.iters;
  o.rel_res = r.rel_res;
  o.status = solve_status(r);
}

}  // namespace
}  // namespace ibm

using namespace ibm;

extern "C" {

void ibm_solver_params_default(ibm_solver_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->vel_tol = 1.0e-6; p->vel_maxit = 250; p->vel_kdim = 50; p->vel_jacobi_iters = 1;
  p->p_tol = 1.0e-9; p->p_maxit = 250; p->p_kdim = 50;
  p->p_pc = 1; p->p_pc_maxit = 1; p->p_pc_relax_type = 1; p->p_pc_rap_type = 1;
  p->mg_nu1 = 1; p->mg_nu2 = 1; p->mg_omega = 2.0 / 3.0; p->mg_coarse_max = 64; p->mg_max_levels = 40;
  p->use_zero_initial_guess = 1; p->precision = 0; p->use_graph = 0; p->vel_inner_sweeps = 3;
  p->mg_group_ratio = 0.0;
  p->mg_options = 3;
  p->mg_nu_coarse = 0;
  p->cycle_rtol32 = 1e-5;
  p->compute_forces = 0;
  p->row_classes = 1;
  p->mg_quads = 1;
  p->df_residual = 1;
  p->mg_fused_coarse = 0;
  p->mg_fused_sweep = 0;
  p->vel_precision = -1;
  p->df_spmv = 1;
  p->df_rhs = 1;
  p->arnoldi_passes = 2;
}

const char *ibm_last_error(ibm_ctx *ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int ibm_create(const ibm_grid_desc *grid, ibm_ctx **out) {
  if (!grid || !out) return IBM_ERR_ARG;
  *out = nullptr;
  if (grid->nx < 3 || grid->ny < 3 || grid->nz < 3 || !(grid->dt > 0) || !(grid->rho > 0) || grid->Lx <= 0 ||
      grid->Ly <= 0 || grid->Lz <= 0) {
    g_create_error = "ibm_create: bad grid";
    return IBM_ERR_ARG;
  }
  if ((double)(grid->nx + 1) * (grid->ny + 1) * (grid->nz + 1) > 2.0e9) {
    g_create_error = "ibm_create: grid too large for 32-bit row indices";
    return IBM_ERR_ARG;
  }
  ibm_ctx *c = new ibm_ctx();
  c->grid = *grid;
  c->device = grid->device;
  ibm_solver_params_default(&c->prm);
  int rc = guarded(c, [&]() {
    IBM_CUDA_TRY(cudaSetDevice(grid->device));
    IBM_CUDA_TRY(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
    for (auto &e : c->ev) IBM_CUDA_TRY(cudaEventCreate(&e));
    Geometry &g = c->g;
    g.nx = grid->nx; g.ny = grid->ny; g.nz = grid->nz;
    g.NU = (long)(g.nx + 1) * g.ny * g.nz; g.NV = (long)g.nx * (g.ny + 1) * g.nz;
    g.NW = (long)g.nx * g.ny * (g.nz + 1); g.NP = (long)g.nx * g.ny * g.nz;
    g.bu = make_box(g.nx - 1, g.ny, g.nz); g.bv = make_box(g.nx, g.ny - 1, g.nz);
    g.bw = make_box(g.nx, g.ny, g.nz - 1); g.bp = make_box(g.nx, g.ny, g.nz);
    g.dx = grid->Lx / g.nx; g.dy = grid->Ly / g.ny; g.dz = grid->Lz / g.nz;
    g.rho = grid->rho; g.nu = grid->nu; g.dt = grid->dt;
    c->u.alloc(g.NU); c->v.alloc(g.NV); c->w.alloc(g.NW); c->p.alloc(g.NP);
    c->ut.alloc(g.NU); c->vt.alloc(g.NV); c->wt.alloc(g.NW);
    for (int f = 0; f < 4; ++f) {
      c->xb[f].alloc(field_box(c, f).n);
      c->bb[f].alloc(field_box(c, f).n);
      c->xb[f].zero(c->st);
      c->bb[f].zero(c->st);
    }
    c->u.zero(c->st); c->v.zero(c->st); c->w.zero(c->st); c->p.zero(c->st);
    c->diag.alloc(1);
    c->dramp.alloc(1);
    c->dloops.alloc(4);
    IBM_CUDA_TRY(cudaMallocHost((void **)&c->hramp, sizeof(double)));
    *c->hramp = 1.0;
    IBM_CUDA_TRY(cudaMallocHost((void **)&c->hflags_graph, sizeof(KFlags) * 4));
    IBM_CUDA_TRY(cudaMallocHost((void **)&c->hloops, sizeof(unsigned long long) * 4));
    for (auto &s : c->cap) IBM_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    c->part.alloc(4 * 1024);
    IBM_CUDA_TRY(cudaMallocHost((void **)&c->hdiag, sizeof(StepDiag)));
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
  if (rc != IBM_OK) {
    g_create_error = c->err;
    ibm_destroy(c);
    return rc;
  }
  *out = c;
  return IBM_OK;
}

void ibm_destroy(ibm_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->adj) {
    if (c->adj->t) ibm_destroy(c->adj->t);
    delete c->adj;
    c->adj = nullptr;
  }
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->hdiag) cudaFreeHost(c->hdiag);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->hramp) cudaFreeHost(c->hramp);
  if (c->hflags_graph) cudaFreeHost(c->hflags_graph);
  if (c->hloops) cudaFreeHost(c->hloops);
  for (auto s : c->cap)
    if (s) cudaStreamDestroy(s);
  cudaStream_t st = c->st;
  delete c;
  if (st) cudaStreamDestroy(st);
}

int ibm_set_operator(ibm_ctx *c, int field, const double *vals7, int nbx, int nby, int nbz) {
  return guarded(c, [&]() {
    if (field < 0 || field > 3 || !vals7) throw Error(IBM_ERR_ARG, "ibm_set_operator: bad field or pointer");
    const Box &b = field_box(c, field);
    if (nbx != b.nx || nby != b.ny || nbz != b.nz)
      throw Error(IBM_ERR_ARG, "ibm_set_operator: box does not match the field's solve box");
    Op7 &o = c->op[field];
    o.b = b;
    o.cls_tried = false;
    o.cls = Classes<double>();
    o.clsj = Classes<float>();
    o.tab.release();
    o.tabf.release();
    o.tabdf.release();
    const long n = b.n;
    DBuf<double> tmp;
    tmp.alloc((size_t)7 * n);
    IBM_CUDA_TRY(cudaMemcpyAsync(tmp.p, vals7, sizeof(double) * 7 * n, cudaMemcpyDefault, c->st));
    o.c.alloc((size_t)7 * n); o.cj.alloc((size_t)7 * n); o.invd.alloc(n);
    o.cf.alloc((size_t)7 * n); o.invdf.alloc(n);
    {
      LaunchScope ls(K_SETUP, c->st, 0.0, 2);
      k_op_planes<<<grid1d(n), kThreads, 0, c->st>>>(tmp.p, n, o.c.p, o.invd.p, o.cf.p, o.invdf.p);
      k_op_jacobi<<<grid1d(n), kThreads, 0, c->st>>>(o.c.p, o.invd.p, o.cj.p, b);
    }
    o.cjf.alloc((size_t)7 * n);
    {
      LaunchScope ls(K_SETUP, c->st, 0.0);
      k_to_float<<<grid1d(7 * n), kThreads, 0, c->st>>>(o.cj.p, o.cjf.p, 7 * n);
    }
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    IBM_CUDA_TRY(cudaGetLastError());
    if (field == 3) {
      const std::vector<double> hv = to_host(vals7, (size_t)7 * n);
      std::vector<double> winv;
      c->p_sym = diagonal_symmetrizer(hv, b, winv);
      upload(c->p_winv, winv, c->st);
      IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    }
    o.set = true;
    c->solvers_ready = false;
    invalidate_graph(c);
    return IBM_OK;
  });
}

}  // extern "C"

namespace ibm {
void launch_assemble_momentum(cudaStream_t st, int f, long n, const asmb::Geo &g, const unsigned char *act,
                              const int *id, double *rows, double *scale);
void launch_assemble_pressure(cudaStream_t st, long n, const asmb::Geo &g, const asmb::PInputs &in, double *rows);
}

extern "C" {

int ibm_assemble_momentum(ibm_ctx *c, double xcirc, double ycirc, double Rcirc, const uint8_t *const *active,
                          const int32_t *const *id, double *const *vals_out, double *const *scale_out) {
  return guarded(c, [&]() {
    if (!active || !id) throw Error(IBM_ERR_ARG, "ibm_assemble_momentum: null masks or ids");
    const Geometry &g = c->g;
    asmb::Geo geo;
    geo.nx = g.nx; geo.ny = g.ny; geo.nz = g.nz;
    geo.Lx = c->grid.Lx; geo.Ly = c->grid.Ly; geo.Lz = c->grid.Lz;
    geo.rho = c->grid.rho; geo.nu = c->grid.nu; geo.dt = c->grid.dt;
    geo.xcirc = xcirc; geo.ycirc = ycirc; geo.Rcirc = Rcirc;
    const long nf[3] = {g.NU, g.NV, g.NW};
    for (int f = 0; f < 3; ++f) {
      if (!active[f] || !id[f]) throw Error(IBM_ERR_ARG, "ibm_assemble_momentum: null mask or id array");
      DBuf<uint8_t> dact;
      DBuf<int32_t> did;
      dact.alloc(nf[f]);
      did.alloc(nf[f]);
      IBM_CUDA_TRY(cudaMemcpyAsync(dact.p, active[f], nf[f], cudaMemcpyDefault, c->st));
      IBM_CUDA_TRY(cudaMemcpyAsync(did.p, id[f], sizeof(int32_t) * nf[f], cudaMemcpyDefault, c->st));
      const std::vector<int32_t> hid = to_host(id[f], (size_t)nf[f]);
      const int nid = hid.empty() ? 0 : *std::max_element(hid.begin(), hid.end());
      const Box &b = field_box(c, f);
      DBuf<double> rows, sc;
      rows.alloc((size_t)7 * b.n);
      sc.alloc((size_t)nid + 1);
      const std::vector<double> ones((size_t)nid + 1, 1.0);
      IBM_CUDA_TRY(cudaMemcpyAsync(sc.p, ones.data(), sizeof(double) * ones.size(), cudaMemcpyHostToDevice, c->st));
      launch_assemble_momentum(c->st, f, b.n, geo, dact.p, did.p, rows.p, sc.p);
      IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
      IBM_CUDA_TRY(cudaGetLastError());
      if (vals_out && vals_out[f])
        IBM_CUDA_TRY(cudaMemcpy(vals_out[f], rows.p, sizeof(double) * 7 * b.n, cudaMemcpyDefault));
      if (scale_out && scale_out[f])
        IBM_CUDA_TRY(cudaMemcpy(scale_out[f], sc.p, sizeof(double) * ones.size(), cudaMemcpyDefault));
      const int rc = ibm_set_operator(c, f, rows.p, b.nx, b.ny, b.nz);
      if (rc < 0) throw Error(rc, c->err);
      // The right-hand side is scaled row by row with the same scales as the
      // rows (gpu_dense_ops.hpp:16-18): the new scales replace the ones
      // ibm_set_aux gave, so a moved body steps with consistent rows and
      // right-hand sides.
      if (c->aux_set && nid == c->n_id[f]) {
        const std::vector<double> hs = to_host(sc.p, ones.size());
        const std::vector<int32_t> *rmap[3] = {&c->h_id_u_rows, &c->h_id_v_rows, &c->h_id_w_rows};
        std::vector<double> sbox(rmap[f]->size());
        for (size_t r = 0; r < rmap[f]->size(); ++r) {
          const int rid = (*rmap[f])[r];
          sbox[r] = rid > 0 ? hs[(size_t)rid] : 0.0;
        }
        upload(c->scale_box[f], sbox, c->st);
        invalidate_graph(c);
      }
    }
    return IBM_OK;
  });
}

int ibm_assemble_pressure(ibm_ctx *c, const uint8_t *fluid_p, const int32_t *id_p, const double *beta_p,
                          const double *const *alpha, const uint8_t *const *active_q, const int32_t *const *id_q,
                          double *vals_out) {
  return guarded(c, [&]() {
    if (!fluid_p || !id_p || !beta_p || !alpha || !active_q || !id_q)
      throw Error(IBM_ERR_ARG, "ibm_assemble_pressure: null input");
    const Geometry &g = c->g;
    asmb::Geo geo;
    geo.nx = g.nx; geo.ny = g.ny; geo.nz = g.nz;
    geo.Lx = c->grid.Lx; geo.Ly = c->grid.Ly; geo.Lz = c->grid.Lz;
    geo.rho = c->grid.rho; geo.nu = c->grid.nu; geo.dt = c->grid.dt;
    geo.xcirc = geo.ycirc = geo.Rcirc = 0.0;
    const long nf[3] = {g.NU, g.NV, g.NW};
    DBuf<uint8_t> dfl, dq[3];
    DBuf<int32_t> dip, diq[3];
    DBuf<double> dbeta, dal[3];
    dfl.alloc(g.NP); dip.alloc(g.NP); dbeta.alloc(g.NP);
    IBM_CUDA_TRY(cudaMemcpyAsync(dfl.p, fluid_p, g.NP, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaMemcpyAsync(dip.p, id_p, sizeof(int32_t) * g.NP, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaMemcpyAsync(dbeta.p, beta_p, sizeof(double) * g.NP, cudaMemcpyDefault, c->st));
    asmb::PInputs in;
    int nq[3];
    for (int f = 0; f < 3; ++f) {
      if (!alpha[f] || !active_q[f] || !id_q[f]) throw Error(IBM_ERR_ARG, "ibm_assemble_pressure: null face array");
      dq[f].alloc(nf[f]); diq[f].alloc(nf[f]); dal[f].alloc(nf[f]);
      IBM_CUDA_TRY(cudaMemcpyAsync(dq[f].p, active_q[f], nf[f], cudaMemcpyDefault, c->st));
      IBM_CUDA_TRY(cudaMemcpyAsync(diq[f].p, id_q[f], sizeof(int32_t) * nf[f], cudaMemcpyDefault, c->st));
      IBM_CUDA_TRY(cudaMemcpyAsync(dal[f].p, alpha[f], sizeof(double) * nf[f], cudaMemcpyDefault, c->st));
      const std::vector<int32_t> h = to_host(id_q[f], (size_t)nf[f]);
      nq[f] = h.empty() ? 0 : *std::max_element(h.begin(), h.end());
      in.alpha[f] = dal[f].p; in.act_q[f] = dq[f].p; in.id_q[f] = diq[f].p;
    }
    in.fluid = dfl.p; in.id_p = dip.p; in.beta = dbeta.p;
    in.nQu = nq[0]; in.nQv = nq[1];
    DBuf<double> rows;
    rows.alloc((size_t)7 * g.NP);
    launch_assemble_pressure(c->st, g.NP, geo, in, rows.p);
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    IBM_CUDA_TRY(cudaGetLastError());
    if (vals_out) IBM_CUDA_TRY(cudaMemcpy(vals_out, rows.p, sizeof(double) * 7 * g.NP, cudaMemcpyDefault));
    const int rc = ibm_set_operator(c, 3, rows.p, g.nx, g.ny, g.nz);
    if (rc < 0) throw Error(rc, c->err);
    return IBM_OK;
  });
}

int ibm_set_masks(ibm_ctx *c, const uint8_t *active_u, const uint8_t *active_v, const uint8_t *active_w,
                  const uint8_t *fluid_p, const uint8_t *active_qu, const uint8_t *active_qv,
                  const uint8_t *active_qw, const int32_t *id_u, const int32_t *id_v, const int32_t *id_w,
                  const int32_t *id_p, const int32_t *id_qu, const int32_t *id_qv, const int32_t *id_qw) {
  return guarded(c, [&]() {
    if (!active_u || !active_v || !active_w || !fluid_p || !id_u || !id_v || !id_w || !id_p || !id_qu || !id_qv ||
        !id_qw)
      throw Error(IBM_ERR_ARG, "ibm_set_masks: null pointer");
    (void)active_qu; (void)active_qv; (void)active_qw;  // q membership follows the q ids, as the reference packs
    const Geometry &g = c->g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    auto au = to_host(active_u, g.NU), av = to_host(active_v, g.NV), aw = to_host(active_w, g.NW),
         fp = to_host(fluid_p, g.NP);
    auto iu = to_host(id_u, g.NU), iv = to_host(id_v, g.NV), iw = to_host(id_w, g.NW);
    c->h_id_p = to_host(id_p, g.NP);
    c->h_id_qu = to_host(id_qu, g.NU); c->h_id_qv = to_host(id_qv, g.NV); c->h_id_qw = to_host(id_qw, g.NW);
    std::vector<uint8_t> fu(g.NU), fv(g.NV), fw(g.NW), fc(g.NP);
    for (long f = 0; f < g.NU; ++f)
      fu[f] = (au[f] ? kActive : 0) | (c->h_id_qu[f] > 0 ? kQFace : 0) | ((iu[f] > 0 && au[f]) ? kRhsRow : 0);
    for (long f = 0; f < g.NV; ++f)
      fv[f] = (av[f] ? kActive : 0) | (c->h_id_qv[f] > 0 ? kQFace : 0) | ((iv[f] > 0 && av[f]) ? kRhsRow : 0);
    for (long f = 0; f < g.NW; ++f)
      fw[f] = (aw[f] ? kActive : 0) | (c->h_id_qw[f] > 0 ? kQFace : 0) | ((iw[f] > 0 && aw[f]) ? kRhsRow : 0);
    int npa = 0;
    for (long q = 0; q < g.NP; ++q) {
      fc[q] = (fp[q] && c->h_id_p[q] > 0) ? kFluid : 0;
      npa = std::max(npa, (int)c->h_id_p[q]);
    }
    c->np_active = npa;
    // inactive interior faces zeroed by the BC cleanup (gpu_dense_ops.hpp:5-10;
    // w uses the mask one plane below)
    std::vector<int> zu, zv, zw;
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 1; i < nx; ++i) {
          const long f = ((long)k * ny + j) * (nx + 1) + i;
          if (!au[f]) zu.push_back((int)f);
        }
    for (int k = 0; k < nz; ++k)
      for (int j = 1; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const long f = ((long)k * (ny + 1) + j) * nx + i;
          if (!av[f]) zv.push_back((int)f);
        }
    for (int k = 1; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const long f = ((long)k * ny + j) * nx + i;
          if (!aw[f - (long)nx * ny]) zw.push_back((int)f);
        }
    // faces the BC cleanup writes: the diagnostics recompute q there
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j) {
        fu[((long)k * ny + j) * (nx + 1)] |= kBcSet;
        fu[((long)k * ny + j) * (nx + 1) + nx] |= kBcSet;
      }
    for (int k = 0; k < nz; ++k)
      for (int i = 0; i < nx; ++i) {
        fv[((long)k * (ny + 1)) * nx + i] |= kBcSet;
        fv[((long)k * (ny + 1) + ny) * nx + i] |= kBcSet;
      }
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        fw[(long)j * nx + i] |= kBcSet;
        fw[((long)nz * ny + j) * nx + i] |= kBcSet;
      }
    for (int f : zu) fu[f] |= kBcSet;
    for (int f : zv) fv[f] |= kBcSet;
    for (int f : zw) fw[f] |= kBcSet;
    upload(c->fu, fu, c->st); upload(c->fv, fv, c->st); upload(c->fw, fw, c->st); upload(c->fc, fc, c->st);
    upload(c->zl_u, zu, c->st); upload(c->zl_v, zv, c->st); upload(c->zl_w, zw, c->st);
    c->h_act_u = au; c->h_act_v = av; c->h_act_w = aw; c->h_fluid = fp;
    c->body_set = false;
    c->masks_set = true;
    c->aux_set = false;
    c->csr_set = false;
    c->solvers_ready = false;
    invalidate_graph(c);
    // id of each solve-box row, for the conversion of the id-indexed aux vectors
    c->h_id_u_rows.clear();
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 1; i < nx; ++i) {
          const long f = ((long)k * ny + j) * (nx + 1) + i;
          c->h_id_u_rows.push_back((iu[f] > 0 && au[f]) ? iu[f] : 0);
        }
    c->h_id_v_rows.clear();
    for (int k = 0; k < nz; ++k)
      for (int j = 1; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const long f = ((long)k * (ny + 1) + j) * nx + i;
          c->h_id_v_rows.push_back((iv[f] > 0 && av[f]) ? iv[f] : 0);
        }
    c->h_id_w_rows.clear();
    for (int k = 1; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const long f = ((long)k * ny + j) * nx + i;
          c->h_id_w_rows.push_back((iw[f] > 0 && aw[f]) ? iw[f] : 0);
        }
    c->n_id[0] = *std::max_element(iu.begin(), iu.end());
    c->n_id[1] = *std::max_element(iv.begin(), iv.end());
    c->n_id[2] = *std::max_element(iw.begin(), iw.end());
    return IBM_OK;
  });
}

int ibm_set_aux(ibm_ctx *c, const double *scale_u, const double *scale_v, const double *scale_w,
                const double *rhs_u_bc, const double *rhs_v_bc, const double *rhs_w_bc, const double *div_bc_unit,
                const double *uin) {
  return guarded(c, [&]() {
    if (!c->masks_set) throw Error(IBM_ERR_STATE, "ibm_set_aux: call ibm_set_masks first");
    if (!scale_u || !scale_v || !scale_w || !rhs_u_bc || !rhs_v_bc || !rhs_w_bc || !div_bc_unit || !uin)
      throw Error(IBM_ERR_ARG, "ibm_set_aux: null pointer");
    const double *sc[3] = {scale_u, scale_v, scale_w}, *bc[3] = {rhs_u_bc, rhs_v_bc, rhs_w_bc};
    const std::vector<int32_t> *rows[3] = {&c->h_id_u_rows, &c->h_id_v_rows, &c->h_id_w_rows};
    for (int f = 0; f < 3; ++f) {
      const size_t len = (size_t)c->n_id[f] + 1;
      auto hs = to_host(sc[f], len), hb = to_host(bc[f], len);
      std::vector<double> s(rows[f]->size()), b(rows[f]->size());
      for (size_t r = 0; r < rows[f]->size(); ++r) {
        const int id = (*rows[f])[r];
        s[r] = id > 0 ? hs[(size_t)id] : 0.0;
        b[r] = id > 0 ? hb[(size_t)id] : 0.0;
      }
      upload(c->scale_box[f], s, c->st);
      upload(c->bc_box[f], b, c->st);
    }
    auto hd = to_host(div_bc_unit, (size_t)c->np_active + 1);
    std::vector<double> dcell(c->g.NP, 0.0);
    for (long q = 0; q < c->g.NP; ++q) {
      const int id = c->h_id_p[q];
      if (id > 0) dcell[q] = hd[(size_t)id];
    }
    upload(c->div_bc_cell, dcell, c->st);
    upload(c->uin, to_host(uin, (size_t)c->g.ny * c->g.nz), c->st);
    c->aux_set = true;
    invalidate_graph(c);
    return IBM_OK;
  });
}

int ibm_set_body(ibm_ctx *c, double xcirc, double ycirc, double Rcirc, const double *alpha_u,
                 const double *alpha_v) {
  return guarded(c, [&]() {
    if (!c->masks_set) throw Error(IBM_ERR_STATE, "ibm_set_body: call ibm_set_masks first");
    if (!alpha_u || !alpha_v || !(Rcirc > 0.0)) throw Error(IBM_ERR_ARG, "ibm_set_body: bad arguments");
    build_cut_force(c, xcirc, ycirc, Rcirc, to_host(alpha_u, c->g.NU), to_host(alpha_v, c->g.NV));
    invalidate_graph(c);
    return IBM_OK;
  });
}

int ibm_set_projection_csr(ibm_ctx *c, const int32_t *D_rowptr, const int32_t *D_col, const double *D_val,
                           int D_nrows, const int32_t *G_rowptr, const int32_t *G_col, const double *G_val,
                           int G_nrows) {
  return guarded(c, [&]() {
    if (!c->masks_set) throw Error(IBM_ERR_STATE, "ibm_set_projection_csr: call ibm_set_masks first");
    if (!D_rowptr || !D_col || !D_val || !G_rowptr || !G_col || !G_val)
      throw Error(IBM_ERR_ARG, "ibm_set_projection_csr: null pointer");
    const Geometry &g = c->g;
    const int nx = g.nx, ny = g.ny;
    const int nqu = *std::max_element(c->h_id_qu.begin(), c->h_id_qu.end());
    const int nqv = *std::max_element(c->h_id_qv.begin(), c->h_id_qv.end());
    const int nqw = *std::max_element(c->h_id_qw.begin(), c->h_id_qw.end());
    const int nq = nqu + nqv + nqw, np = c->np_active;
    if (D_nrows != np || G_nrows != nq) throw Error(IBM_ERR_ARG, "ibm_set_projection_csr: row counts do not match the ids");
    // inverse id maps
    std::vector<long> cell_of((size_t)np + 1, -1), face_of((size_t)nq + 1, -1);
    for (long q = 0; q < g.NP; ++q) if (c->h_id_p[q] > 0) cell_of[(size_t)c->h_id_p[q]] = q;
    for (long f = 0; f < g.NU; ++f) if (c->h_id_qu[f] > 0) face_of[(size_t)c->h_id_qu[f]] = f;
    for (long f = 0; f < g.NV; ++f) if (c->h_id_qv[f] > 0) face_of[(size_t)(nqu + c->h_id_qv[f])] = f;
    for (long f = 0; f < g.NW; ++f) if (c->h_id_qw[f] > 0) face_of[(size_t)(nqu + nqv + c->h_id_qw[f])] = f;
    auto drp = to_host(D_rowptr, (size_t)np + 1);
    auto dcol = to_host(D_col, (size_t)drp[(size_t)np]);
    auto dval = to_host(D_val, (size_t)drp[(size_t)np]);
    std::vector<double> Dc((size_t)6 * g.NP, 0.0);
    for (int r = 0; r < np; ++r) {
      const long cell = cell_of[(size_t)r + 1];
      if (cell < 0) throw Error(IBM_ERR_ARG, "ibm_set_projection_csr: D row without a cell");
      const int i = (int)(cell % nx), j = (int)((cell / nx) % ny), k = (int)(cell / ((long)nx * ny));
      for (int t = drp[(size_t)r]; t < drp[(size_t)r + 1]; ++t) {
        const int col = dcol[(size_t)t];
        if (col < 1 || col > nq) throw Error(IBM_ERR_ARG, "ibm_set_projection_csr: D column out of range");
        const long f = face_of[(size_t)col];
        int slot = -1;
        if (col <= nqu) {
          if (f == ((long)k * ny + j) * (nx + 1) + i) slot = 0;
          else if (f == ((long)k * ny + j) * (nx + 1) + i + 1) slot = 1;
        } else if (col <= nqu + nqv) {
          if (f == ((long)k * (ny + 1) + j) * nx + i) slot = 2;
          else if (f == ((long)k * (ny + 1) + j + 1) * nx + i) slot = 3;
        } else {
          if (f == ((long)k * ny + j) * nx + i) slot = 4;
          else if (f == ((long)(k + 1) * ny + j) * nx + i) slot = 5;
        }
        if (slot < 0) throw Error(IBM_ERR_UNSUPPORTED, "ibm_set_projection_csr: D entry is not a face of its cell");
        Dc[(size_t)slot * g.NP + cell] = dval[(size_t)t];
      }
    }
    auto grp = to_host(G_rowptr, (size_t)nq + 1);
    auto gcol = to_host(G_col, (size_t)grp[(size_t)nq]);
    auto gval = to_host(G_val, (size_t)grp[(size_t)nq]);
    std::vector<double> Gu((size_t)2 * g.NU, 0.0), Gv((size_t)2 * g.NV, 0.0), Gw((size_t)2 * g.NW, 0.0);
    for (int r = 0; r < nq; ++r) {
      const long f = face_of[(size_t)r + 1];
      const int q = r + 1;
      for (int t = grp[(size_t)r]; t < grp[(size_t)r + 1]; ++t) {
        const int col = gcol[(size_t)t];
        if (col < 1 || col > np) throw Error(IBM_ERR_ARG, "ibm_set_projection_csr: G column out of range");
        const long cell = cell_of[(size_t)col];
        int side = -1;
        if (q <= nqu) {
          const int i = (int)(f % (nx + 1));
          const long jk = f / (nx + 1);
          if (i > 0 && cell == jk * nx + (i - 1)) side = 0;
          else if (i < nx && cell == jk * nx + i) side = 1;
          if (side >= 0) Gu[(size_t)side * g.NU + f] = gval[(size_t)t];
        } else if (q <= nqu + nqv) {
          const int i = (int)(f % nx);
          const long jj = f / nx;
          const int j = (int)(jj % (ny + 1)), k = (int)(jj / (ny + 1));
          if (j > 0 && cell == ((long)k * ny + (j - 1)) * nx + i) side = 0;
          else if (j < ny && cell == ((long)k * ny + j) * nx + i) side = 1;
          if (side >= 0) Gv[(size_t)side * g.NV + f] = gval[(size_t)t];
        } else {
          const long plane = (long)nx * ny;
          const int k = (int)(f / plane);
          const long rem = f - (long)k * plane;
          if (k > 0 && cell == (long)(k - 1) * plane + rem) side = 0;
          else if (k < g.nz && cell == (long)k * plane + rem) side = 1;
          if (side >= 0) Gw[(size_t)side * g.NW + f] = gval[(size_t)t];
        }
        if (side < 0) throw Error(IBM_ERR_UNSUPPORTED, "ibm_set_projection_csr: G entry is not a cell of its face");
      }
    }
    upload(c->Dc, Dc, c->st);
    upload(c->Gu, Gu, c->st); upload(c->Gv, Gv, c->st); upload(c->Gw, Gw, c->st);
    c->csr_set = true;
    invalidate_graph(c);
    return IBM_OK;
  });
}

int ibm_set_solver_params(ibm_ctx *c, const ibm_solver_params *p) {
  return guarded(c, [&]() {
    if (!p) throw Error(IBM_ERR_ARG, "ibm_set_solver_params: null");
    if (p->vel_kdim < 1 || p->vel_kdim > kMaxKdim || p->p_kdim < 1 || p->p_kdim > kMaxKdim)
      throw Error(IBM_ERR_ARG, "kdim must be in [1, 63]");
    if (p->vel_maxit < 0 || p->p_maxit < 0 || !(p->vel_tol >= 0) || !(p->p_tol >= 0))
      throw Error(IBM_ERR_ARG, "bad tolerance or iteration limit");
    if (p->precision < 0 || p->precision > 2) throw Error(IBM_ERR_ARG, "precision must be 0, 1 or 2");
    if (p->vel_precision < -1 || p->vel_precision > 2) throw Error(IBM_ERR_ARG, "vel_precision must be -1, 0, 1 or 2");
    if (p->arnoldi_passes != 1 && p->arnoldi_passes != 2) throw Error(IBM_ERR_ARG, "arnoldi_passes must be 1 or 2");
    if (!(p->cycle_rtol32 > 0.0 && p->cycle_rtol32 < 1.0)) throw Error(IBM_ERR_ARG, "cycle_rtol32 must be in (0, 1)");
    if (p->p_pc != 0 && p->p_pc != 1) throw Error(IBM_ERR_ARG, "p_pc must be 0 or 1");
    if (p->mg_nu1 < 0 || p->mg_nu2 < 0 || p->mg_nu_coarse < 0 || p->mg_coarse_max < 1 || p->mg_max_levels < 1)
      throw Error(IBM_ERR_ARG, "bad multigrid parameters");
    // switching between the graph and the host-driven step keeps the solvers
    ibm_solver_params a = c->prm, b = *p;
    a.use_graph = b.use_graph = 0;
    if (std::memcmp(&a, &b, sizeof(a)) != 0) c->solvers_ready = false;
    c->prm = *p;
    invalidate_graph(c);
    return IBM_OK;
  });
}

int ibm_get_solver_params(ibm_ctx *c, ibm_solver_params *p) {
  if (!c || !p) return IBM_ERR_ARG;
  *p = c->prm;
  return IBM_OK;
}

int ibm_set_fields(ibm_ctx *c, const double *u, const double *v, const double *w, const double *p) {
  return guarded(c, [&]() {
    if (u) IBM_CUDA_TRY(cudaMemcpyAsync(c->u.p, u, sizeof(double) * c->g.NU, cudaMemcpyDefault, c->st));
    if (v) IBM_CUDA_TRY(cudaMemcpyAsync(c->v.p, v, sizeof(double) * c->g.NV, cudaMemcpyDefault, c->st));
    if (w) IBM_CUDA_TRY(cudaMemcpyAsync(c->w.p, w, sizeof(double) * c->g.NW, cudaMemcpyDefault, c->st));
    if (p) IBM_CUDA_TRY(cudaMemcpyAsync(c->p.p, p, sizeof(double) * c->g.NP, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

int ibm_get_fields(ibm_ctx *c, double *u, double *v, double *w, double *p) {
  return guarded(c, [&]() {
    if (u) IBM_CUDA_TRY(cudaMemcpyAsync(u, c->u.p, sizeof(double) * c->g.NU, cudaMemcpyDefault, c->st));
    if (v) IBM_CUDA_TRY(cudaMemcpyAsync(v, c->v.p, sizeof(double) * c->g.NV, cudaMemcpyDefault, c->st));
    if (w) IBM_CUDA_TRY(cudaMemcpyAsync(w, c->w.p, sizeof(double) * c->g.NW, cudaMemcpyDefault, c->st));
    if (p) IBM_CUDA_TRY(cudaMemcpyAsync(p, c->p.p, sizeof(double) * c->g.NP, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

namespace {

// One timestep in two halves so that several contexts can run steps at the
// same time (ibm_batch_step). step_launch queues the whole step; in graph
// mode it returns without waiting (one graph launch on the context's
// stream), in the host-driven mode it runs the step to completion (the GMRES
// host loop reads flags every iteration). step_collect waits for the
// context's stream and turns the solver flags and diagnostics into stats.
void step_launch(ibm_ctx *c, double ramp) {
  require_inputs(c);
  ensure_solvers(c);
  ensure_rhs_df(c);
  cudaStream_t st = c->st;
  *c->hramp = ramp;
  KResult *rm = c->last_rm, *rp = c->last_rp;
  const double *bm[3] = {c->bb[0].p, c->bb[1].p, c->bb[2].p};
  double *xm[3] = {c->xb[0].p, c->xb[1].p, c->xb[2].p};
  const double *bp[1] = {c->bb[3].p};
  double *xp[1] = {c->xb[3].p};
  Precond none, mgp;
  mgp.ctx = c;
  mgp.apply = mg_apply_cb;
  c->last_graph = c->prm.use_graph != 0;
  if (c->prm.use_graph) {
    // The whole step as one graph launch; the GMRES loops run on the device.
    if (!c->graph_ready || !c->graph_bound) {
      const bool zg = c->prm.use_zero_initial_guess != 0;
      c->kmom.bind(st, bm, xm, ~0u, zg);
      c->kp.bind(st, bp, xp, ~0u, true);  // k_pressure_rhs zeroes the pressure's x0 every step
      c->graph_bound = true;
    }
    if (!c->graph_ready) build_step_graph(c, none, mgp);
    IBM_CUDA_TRY(cudaGraphLaunch(c->gexec, st));
    return;
  }
  IBM_CUDA_TRY(cudaMemcpyAsync(c->dramp.p, c->hramp, sizeof(double), cudaMemcpyHostToDevice, st));
  IBM_CUDA_TRY(cudaMemsetAsync(c->diag.p, 0, sizeof(StepDiag), st));
  IBM_CUDA_TRY(cudaEventRecord(c->ev[0], st));
  {
    PhaseScope ph(PH_RHS);
    launch_bc(c, c->u.p, c->v.p, c->w.p);
    launch_momentum_rhs(c);
  }
  IBM_CUDA_TRY(cudaEventRecord(c->ev[1], st));
  {
    PhaseScope ph(PH_MOM);
    c->kmom.solve(st, bm, xm, none, rm, ~0u, c->prm.use_zero_initial_guess != 0);
  }
  IBM_CUDA_TRY(cudaEventRecord(c->ev[2], st));
  {
    PhaseScope ph(PH_RHS);
    launch_tilde(c);
    launch_pressure_rhs(c);
  }
  IBM_CUDA_TRY(cudaEventRecord(c->ev[5], st));
  {
    PhaseScope ph(PH_P);
    c->kp.solve(st, bp, xp, mgp, rp, ~0u, true);  // x0 = 0 (k_pressure_rhs), as the reference
  }
  IBM_CUDA_TRY(cudaEventRecord(c->ev[3], st));
  {
    PhaseScope ph(PH_PROJ);
    launch_projection(c);
  }
  IBM_CUDA_TRY(cudaEventRecord(c->ev[4], st));
  IBM_CUDA_TRY(cudaMemcpyAsync(c->hdiag, c->diag.p, sizeof(StepDiag), cudaMemcpyDeviceToHost, st));
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
  IBM_CUDA_TRY(cudaGetLastError());
  c->prof.drain();
}

int step_collect(ibm_ctx *c, double ramp, ibm_step_stats *stats) {
  KResult *rm = c->last_rm, *rp = c->last_rp;
  if (c->last_graph) {
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    IBM_CUDA_TRY(cudaGetLastError());
    for (int s = 0; s < 4; ++s) {
      const KFlags &f = c->hflags_graph[s];
      KResult &r = s < 3 ? rm[s] : rp[0];
      r.iters = f.iters; r.rel_res = f.rel; r.status = f.status; r.nonfinite = f.nonfinite;
    }
    const unsigned long long *lp = c->hloops;
    c->launches += c->graph_fixed_launches + (long long)lp[0] * c->graph_body_launches[0] +
                   (long long)lp[1] * c->graph_body_launches[1] + (long long)lp[2] * c->graph_body_launches[2] +
                   (long long)lp[3] * c->graph_body_launches[3];
  }
  int rc = IBM_OK;
  const StepDiag &dg = *c->hdiag;
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    stats->ramp = ramp;
    fill_solve(stats->u, rm[0]); fill_solve(stats->v, rm[1]); fill_solve(stats->w, rm[2]);
    fill_solve(stats->p, rp[0]);
    stats->div_l2 = std::sqrt(dg.div2 / std::max(1, c->np_active));
    stats->umax = dg.umax; stats->vmax = dg.vmax; stats->wmax = dg.wmax;
    if (c->prm.compute_forces)
      for (int q = 0; q < 3; ++q) stats->force[q] = dg.force[q];
    float ms;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]); stats->t_rhs_ms = ms;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[5]); stats->t_rhs_ms += ms;
    cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]); stats->t_mom_ms = ms;
    cudaEventElapsedTime(&ms, c->ev[5], c->ev[3]); stats->t_p_ms = ms;
    cudaEventElapsedTime(&ms, c->ev[3], c->ev[4]); stats->t_proj_ms = ms;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[4]); stats->t_total_ms = ms;
  }
  for (int f = 0; f < 3; ++f) rc = worst(rc, solve_status(rm[f]));
  rc = worst(rc, solve_status(rp[0]));
  const bool bad_mom = dg.nonfinite_mom || rm[0].nonfinite || rm[1].nonfinite || rm[2].nonfinite;
  const bool bad_p = dg.nonfinite_p || rp[0].nonfinite;
  if (bad_mom || bad_p) {
    rc = IBM_ERR_NONFINITE;
    c->err = bad_mom ? "non-finite momentum solve (main.cu:302-305)" : "non-finite pressure solve (main.cu:333-336)";
  }
  if (stats) stats->status = rc;
  return rc;
}


}  // namespace

int ibm_step(ibm_ctx *c, double ramp, ibm_step_stats *stats) {
  return guarded(c, [&]() {
    step_launch(c, ramp);
    return step_collect(c, ramp, stats);
  });
}

struct ibm_batch {
  std::vector<ibm_ctx *> ctx;
};

int ibm_batch_create(int n, const ibm_grid_desc *grids, ibm_batch **out) {
  if (n < 1 || !grids || !out) return IBM_ERR_ARG;
  *out = nullptr;
  ibm_batch *b = new ibm_batch;
  for (int i = 0; i < n; ++i) {
    ibm_ctx *c = nullptr;
    const int rc = ibm_create(&grids[i], &c);
    if (rc != IBM_OK) {
      ibm_batch_destroy(b);
      return rc;
    }
    b->ctx.push_back(c);
  }
  *out = b;
  return IBM_OK;
}

void ibm_batch_destroy(ibm_batch *b) {
  if (!b) return;
  for (ibm_ctx *c : b->ctx) ibm_destroy(c);
  delete b;
}

int ibm_batch_size(const ibm_batch *b) { return b ? (int)b->ctx.size() : 0; }

ibm_ctx *ibm_batch_ctx(ibm_batch *b, int i) {
  return (b && i >= 0 && i < (int)b->ctx.size()) ? b->ctx[(size_t)i] : nullptr;
}

int ibm_batch_step(ibm_batch *b, const double *ramps, ibm_step_stats *stats) {
  if (!b || !ramps) return IBM_ERR_ARG;
  const size_t n = b->ctx.size();
  std::vector<int> rc(n, IBM_OK);
  for (size_t i = 0; i < n; ++i) rc[i] = guarded(b->ctx[i], [&]() { step_launch(b->ctx[i], ramps[i]); return IBM_OK; });
  int worst_rc = IBM_OK;
  for (size_t i = 0; i < n; ++i) {
    ibm_step_stats *st = stats ? stats + i : nullptr;
    if (rc[i] == IBM_OK) rc[i] = guarded(b->ctx[i], [&]() { return step_collect(b->ctx[i], ramps[i], st); });
    else if (st) { memset(st, 0, sizeof(*st)); st->status = rc[i]; }
    if (rc[i] < 0) { if (worst_rc >= 0) worst_rc = rc[i]; }
    else if (worst_rc >= 0) worst_rc = std::max(worst_rc, rc[i]);
  }
  return worst_rc;
}

int ibm_solve(ibm_ctx *c, int field, const double *b, double *x, ibm_solve_stats *stats) {
  return guarded(c, [&]() {
    if (field < 0 || field > 3 || !b || !x) throw Error(IBM_ERR_ARG, "ibm_solve: bad arguments");
    require_inputs(c);
    ensure_solvers(c);
    const long n = field_box(c, field).n;
    IBM_CUDA_TRY(cudaMemcpyAsync(c->bb[field].p, b, sizeof(double) * n, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaMemcpyAsync(c->xb[field].p, x, sizeof(double) * n, cudaMemcpyDefault, c->st));
    KResult r[3];
    if (field < 3) {
      const double *bm[3] = {c->bb[0].p, c->bb[1].p, c->bb[2].p};
      double *xm[3] = {c->xb[0].p, c->xb[1].p, c->xb[2].p};
      Precond none;
      c->kmom.solve(c->st, bm, xm, none, r, 1u << field);
      c->graph_bound = false;
      r[0] = r[field];
    } else {
      const double *bp[1] = {c->bb[3].p};
      double *xp[1] = {c->xb[3].p};
      Precond mgp;
      mgp.ctx = c;
      mgp.apply = mg_apply_cb;
      c->kp.solve(c->st, bp, xp, mgp, r);
      c->graph_bound = false;
    }
    IBM_CUDA_TRY(cudaMemcpyAsync(x, c->xb[field].p, sizeof(double) * n, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    c->prof.drain();
    if (stats) fill_solve(*stats, r[0]);
    if (r[0].nonfinite) { c->err = "non-finite solve output"; return (int)IBM_ERR_NONFINITE; }
    return solve_status(r[0]);
  });
}

int ibm_apply_operator(ibm_ctx *c, int field, const double *x, double *y) {
  return guarded(c, [&]() {
    if (field < 0 || field > 3 || !x || !y) throw Error(IBM_ERR_ARG, "ibm_apply_operator: bad arguments");
    if (!c->op[field].set) throw Error(IBM_ERR_STATE, "operator not set");
    const Box &b = field_box(c, field);
    DBuf<double> dx, dy;
    dx.alloc(b.n); dy.alloc(b.n);
    IBM_CUDA_TRY(cudaMemcpyAsync(dx.p, x, sizeof(double) * b.n, cudaMemcpyDefault, c->st));
    {
      LaunchScope ls(K_SETUP, c->st, 72.0 * b.n);
      k_spmv7<<<grid1d(b.n), kThreads, 0, c->st>>>(c->op[field].c.p, b, dx.p, dy.p);
    }
    IBM_CUDA_TRY(cudaMemcpyAsync(y, dy.p, sizeof(double) * b.n, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

int ibm_apply_preconditioner(ibm_ctx *c, int field, const double *r, double *z) {
  return guarded(c, [&]() {
    if (field < 0 || field > 3 || !r || !z) throw Error(IBM_ERR_ARG, "ibm_apply_preconditioner: bad arguments");
    require_inputs(c);
    ensure_solvers(c);
    const Box &b = field_box(c, field);
    DBuf<double> dr, dz;
    dr.alloc(b.n); dz.alloc(b.n);
    IBM_CUDA_TRY(cudaMemcpyAsync(dr.p, r, sizeof(double) * b.n, cudaMemcpyDefault, c->st));
    if (field == 3 && c->prm.p_pc == 1) {
      VecRef in;
      in.base = dr.p;
      if (c->prm.precision >= 1) {
        DBuf<float> zf;
        zf.alloc(b.n);
        OutRef out;
        out.f = zf.p;
        c->mg.apply(c->st, in, out, nullptr, true);
        std::vector<float> hz(b.n);
        IBM_CUDA_TRY(cudaMemcpyAsync(hz.data(), zf.p, sizeof(float) * b.n, cudaMemcpyDeviceToHost, c->st));
            IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
            c->prof.drain();
        std::vector<double> zd(hz.begin(), hz.end());
        IBM_CUDA_TRY(cudaMemcpy(z, zd.data(), sizeof(double) * b.n, cudaMemcpyDefault));
        return IBM_OK;
      }
      OutRef out;
      out.d = dz.p;
      c->mg.apply(c->st, in, out, nullptr, false);
    } else {
      // one Jacobi sweep from a zero guess: z = r / diag
      std::vector<double> hr = to_host(r, (size_t)b.n), hd = to_host(c->op[field].invd.p, (size_t)b.n);
      for (long i = 0; i < b.n; ++i) hr[(size_t)i] *= hd[(size_t)i];
      IBM_CUDA_TRY(cudaMemcpy(dz.p, hr.data(), sizeof(double) * b.n, cudaMemcpyHostToDevice));
    }
    IBM_CUDA_TRY(cudaMemcpyAsync(z, dz.p, sizeof(double) * b.n, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    c->prof.drain();
    return IBM_OK;
  });
}

int ibm_get_solver_vector(ibm_ctx *c, int field, int which, double *out) {
  return guarded(c, [&]() {
    if (field < 0 || field > 3 || (which != 0 && which != 1) || !out)
      throw Error(IBM_ERR_ARG, "ibm_get_solver_vector: bad arguments");
    const long n = field_box(c, field).n;
    const double *src = which == 0 ? c->bb[field].p : c->xb[field].p;
    IBM_CUDA_TRY(cudaMemcpyAsync(out, src, sizeof(double) * n, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

int ibm_synchronize(ibm_ctx *c) {
  return guarded(c, [&]() {
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

void *ibm_stream(ibm_ctx *c) { return c ? (void *)c->st : nullptr; }

int ibm_profile_reset(ibm_ctx *c) {
  if (!c) return IBM_ERR_ARG;
  c->prof.reset();
  return IBM_OK;
}

int ibm_profile_time_kernel(ibm_ctx *c, int kernel) {
  if (!c || kernel < -1 || kernel >= K_COUNT) return IBM_ERR_ARG;
  c->prof.timed_kernel = kernel;
  return IBM_OK;
}

int ibm_profile_get(ibm_ctx *c, ibm_profile *out) {
  if (!c || !out) return IBM_ERR_ARG;
  memset(out, 0, sizeof(*out));
  out->nkernels = K_COUNT;
  for (int k = 0; k < K_COUNT && k < IBM_PROFILE_MAX_KERNELS; ++k) {
    out->launches[k] = c->prof.launches[k];
    out->bytes[k] = c->prof.bytes[k];
    out->time_ms[k] = c->prof.ms[k];
    out->timed_launches[k] = c->prof.timed[k];
  }
  for (int q = 0; q < PH_COUNT && q < 5; ++q) out->phase_bytes[q] = c->prof.phase_bytes[q];
  return IBM_OK;
}

const char *ibm_kernel_name(int kernel) { return kernel_name(kernel); }

long long ibm_kernel_launches(ibm_ctx *c) { return c ? c->launches : 0; }

int ibm_device_query(int device, char *buf, int len) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return IBM_ERR_CUDA;
  if (buf && len > 0) snprintf(buf, (size_t)len, "%s sm_%d%d SMs=%d", p.name, p.major, p.minor, p.multiProcessorCount);
  return IBM_OK;
}

// ---------------------------------------------------------------- adjoint extension
namespace {

ibm::AdjState &adj_of(ibm_ctx *c) {
  if (!c->adj || !c->adj->t) throw Error(IBM_ERR_STATE, "call ibm_adjoint_setup first");
  return *c->adj;
}

std::array<DBuf<double>, 4> snapshot(ibm_ctx *c) {
  std::array<DBuf<double>, 4> s;
  const double *src[4] = {c->u.p, c->v.p, c->w.p, c->p.p};
  const long n[4] = {c->g.NU, c->g.NV, c->g.NW, c->g.NP};
  for (int q = 0; q < 4; ++q) {
    s[q].alloc(n[q]);
    IBM_CUDA_TRY(cudaMemcpyAsync(s[q].p, src[q], sizeof(double) * n[q], cudaMemcpyDeviceToDevice, c->st));
  }
  return s;
}

// Device copy of n doubles into dst (allocated to n).
void copy_into(ibm_ctx *c, DBuf<double> &dst, const double *src, long n) {
  dst.alloc(n);
  IBM_CUDA_TRY(cudaMemcpyAsync(dst.p, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->st));
}

void restore(ibm_ctx *c, const std::array<DBuf<double>, 4> &s) {
  double *dst[4] = {c->u.p, c->v.p, c->w.p, c->p.p};
  for (int q = 0; q < 4; ++q)
    IBM_CUDA_TRY(cudaMemcpyAsync(dst[q], s[q].p, sizeof(double) * s[q].n, cudaMemcpyDeviceToDevice, c->st));
}

// A^-T b on the transposed-operator context t, host-driven: the pressure
// system alone or the three momentum systems batched in one solve, from
// t->bb into t->xb (zero initial guesses). The caller's stream must have
// produced b already. Returns the worst status; throws on a non-finite
// solution.
int transposed_solve(ibm_ctx *t, bool pressure) {
  Scope sc(t);
  ensure_solvers(t);
  const int f0 = pressure ? 3 : 0, nf = pressure ? 1 : 3;
  for (int f = f0; f < f0 + nf; ++f)
    IBM_CUDA_TRY(cudaMemsetAsync(t->xb[f].p, 0, sizeof(double) * field_box(t, f).n, t->st));
  KResult r[3];
  if (!pressure) {
    const double *bm[3] = {t->bb[0].p, t->bb[1].p, t->bb[2].p};
    double *xm[3] = {t->xb[0].p, t->xb[1].p, t->xb[2].p};
    Precond none;
    t->kmom.solve(t->st, bm, xm, none, r, ~0u, true);
  } else {
    const double *bp[1] = {t->bb[3].p};
    double *xp[1] = {t->xb[3].p};
    Precond mgp;
    mgp.ctx = t;
    mgp.apply = mg_apply_cb;
    t->kp.solve(t->st, bp, xp, mgp, r, ~0u, true);
  }
  t->graph_bound = false;
  if (t->adj_owner) t->adj_owner->adj->graph_bound = false;
  IBM_CUDA_TRY(cudaStreamSynchronize(t->st));
  t->prof.drain();
  int rc = IBM_OK;
  for (int q = 0; q < nf; ++q) {
    if (t->adj_owner) t->adj_owner->adj->last[f0 + q] = r[q];
    if (r[q].nonfinite) throw Error(IBM_ERR_NONFINITE, "non-finite transposed solve");
    rc = worst(rc, solve_status(r[q]));
  }
  return rc;
}

// The reverse sweep after the recomputed step, host-driven. The ramp is the
// step's (c->dramp), the objective weight a.dweight.
int reverse_host(ibm_ctx *c) {
  ibm::AdjState &a = *c->adj;
  ibm_ctx *t = a.t;
  const double *ramp = c->dramp.p;
  adj_force(c, a.dweight.p);
  adj_bc(c, a.lu.p, a.lv.p, a.lw.p, ramp);
  int rc = IBM_OK;
  if (c->p_sym) {
    // Ap^T mu = r  <=>  Ap (W mu) = W r, with the step's own pressure solver
    adj_projection(c, a.mu.p);
    adj_wscale(c, a.mu.p, c->bb[3].p, true);
    IBM_CUDA_TRY(cudaMemsetAsync(c->xb[3].p, 0, sizeof(double) * c->g.NP, c->st));
    const double *bp[1] = {c->bb[3].p};
    double *xp[1] = {c->xb[3].p};
    Precond mgp;
    mgp.ctx = c;
    mgp.apply = mg_apply_cb;
    KResult r[1];
    c->kp.solve(c->st, bp, xp, mgp, r, ~0u, true);
    c->graph_bound = false;
    a.last[3] = r[0];
    if (r[0].nonfinite) throw Error(IBM_ERR_NONFINITE, "non-finite transposed solve");
    rc = solve_status(r[0]);
    adj_wscale(c, c->xb[3].p, a.mu.p, false);
  } else {
    adj_projection(c, t->bb[3].p);
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    rc = transposed_solve(t, true);
    IBM_CUDA_TRY(cudaMemcpyAsync(a.mu.p, t->xb[3].p, sizeof(double) * c->g.NP, cudaMemcpyDeviceToDevice, c->st));
  }
  adj_divergence(c, a.mu.p, ramp);
  adj_bc(c, a.lu.p, a.lv.p, a.lw.p, ramp);
  double *lx[3] = {t->bb[0].p, t->bb[1].p, t->bb[2].p};
  adj_scatter(c, lx);
  IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
  rc = worst(rc, transposed_solve(t, false));
  const double *lb[3] = {t->xb[0].p, t->xb[1].p, t->xb[2].p};
  adj_momentum(c, lb);
  adj_gradient(c);
  adj_bc(c, a.lu.p, a.lv.p, a.lw.p, ramp);
  IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
  return rc;
}

// Binds the transposed context's Krylov systems to its bb / xb vectors for
// the graph form (outside any capture).
void bind_transposed(ibm_ctx *c) {
  ibm::AdjState &a = *c->adj;
  ibm_ctx *t = a.t;
  Scope sc(t);
  ensure_solvers(t);
  const double *bm[3] = {t->bb[0].p, t->bb[1].p, t->bb[2].p};
  double *xm[3] = {t->xb[0].p, t->xb[1].p, t->xb[2].p};
  t->kmom.bind(t->st, bm, xm, ~0u, true);
  const double *bp[1] = {t->bb[3].p};
  double *xp[1] = {t->xb[3].p};
  t->kp.bind(t->st, bp, xp, ~0u, true);
  IBM_CUDA_TRY(cudaStreamSynchronize(t->st));
  a.graph_bound = true;
}

// The reverse sweep captured as one graph on c->st: the adjoint kernels and
// the graph forms of the transposed solves (restart and Arnoldi loops as
// conditional nodes on the device). Inputs that change per call are read on
// the device: the ramp (c->dramp, written by the recomputed step), the
// weight (a.dweight, copied from pinned memory by the graph) and the
// linearisation point (a.u1 / v1 / w1, copied in before the launch).
void build_adjoint_graph(ibm_ctx *c) {
  ibm::AdjState &a = *c->adj;
  ibm_ctx *t = a.t;
  if (a.gexec) cudaGraphExecDestroy(a.gexec);
  a.gexec = nullptr;
  a.graph_ready = false;
  bind_transposed(c);
  cudaStream_t st = c->st;
  Prof *saved_prof = current_prof();
  long long *saved_counter = g_counter;
  long long cap_count = 0;
  current_prof() = nullptr;
  g_counter = &cap_count;
  cudaGraph_t graph = nullptr;
  Krylov::GraphCounts gm, gp;
  Precond none, mgp, mgc;
  mgp.ctx = t;
  mgp.apply = mg_apply_cb;
  mgc.ctx = c;
  mgc.apply = mg_apply_cb;
  const double *ramp = c->dramp.p;
  try {
    IBM_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    IBM_CUDA_TRY(cudaMemcpyAsync(a.dweight.p, a.hweight, sizeof(double), cudaMemcpyHostToDevice, st));
    IBM_CUDA_TRY(cudaMemsetAsync(t->dloops.p, 0, sizeof(unsigned long long) * 4, st));
    launch_bc(c, a.u1.p, a.v1.p, a.w1.p);
    adj_force(c, a.dweight.p);
    adj_bc(c, a.lu.p, a.lv.p, a.lw.p, ramp);
    if (c->p_sym) {
      adj_projection(c, a.mu.p);
      adj_wscale(c, a.mu.p, c->bb[3].p, true);
      IBM_CUDA_TRY(cudaMemsetAsync(c->xb[3].p, 0, sizeof(double) * c->g.NP, st));
      gp = c->kp.enqueue_graph(st, c->cap, mgc, c->hflags_graph + 3, t->dloops.p + 2);
      adj_wscale(c, c->xb[3].p, a.mu.p, false);
    } else {
      adj_projection(c, t->bb[3].p);
      IBM_CUDA_TRY(cudaMemsetAsync(t->xb[3].p, 0, sizeof(double) * t->g.bp.n, st));
      gp = t->kp.enqueue_graph(st, t->cap, mgp, t->hflags_graph + 3, t->dloops.p + 2);
      IBM_CUDA_TRY(cudaMemcpyAsync(a.mu.p, t->xb[3].p, sizeof(double) * c->g.NP, cudaMemcpyDeviceToDevice, st));
    }
    adj_divergence(c, a.mu.p, ramp);
    adj_bc(c, a.lu.p, a.lv.p, a.lw.p, ramp);
    double *lx[3] = {t->bb[0].p, t->bb[1].p, t->bb[2].p};
    adj_scatter(c, lx);
    for (int f = 0; f < 3; ++f)
      IBM_CUDA_TRY(cudaMemsetAsync(t->xb[f].p, 0, sizeof(double) * field_box(t, f).n, st));
    gm = t->kmom.enqueue_graph(st, t->cap, none, t->hflags_graph, t->dloops.p);
    const double *lb[3] = {t->xb[0].p, t->xb[1].p, t->xb[2].p};
    adj_momentum(c, lb);
    adj_gradient(c);
    adj_bc(c, a.lu.p, a.lv.p, a.lw.p, ramp);
    IBM_CUDA_TRY(cudaMemcpyAsync(t->hloops, t->dloops.p, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, st));
    IBM_CUDA_TRY(cudaStreamEndCapture(st, &graph));
  } catch (...) {
    cudaGraph_t junk = nullptr;
    cudaStreamEndCapture(st, &junk);
    if (junk) cudaGraphDestroy(junk);
    current_prof() = saved_prof;
    g_counter = saved_counter;
    throw;
  }
  current_prof() = saved_prof;
  g_counter = saved_counter;
  const cudaError_t e = cudaGraphInstantiate(&a.gexec, graph, 0);
  cudaGraphDestroy(graph);
  IBM_CUDA_TRY(e);
  a.graph_fixed_launches = cap_count - gm.loop - gp.loop;
  a.graph_body_launches[0] = gm.end_body;
  a.graph_body_launches[1] = gm.arnoldi_body;
  a.graph_body_launches[2] = gp.end_body;
  a.graph_body_launches[3] = gp.arnoldi_body;
  a.graph_ready = true;
}

// Launches the captured reverse sweep and reads the transposed solves' flags.
int reverse_graph(ibm_ctx *c) {
  ibm::AdjState &a = *c->adj;
  ibm_ctx *t = a.t;
  if (c->p_sym && !c->graph_bound) {
    // as the step graph binds them (a host-driven solve on this context unbinds)
    const bool zg = c->prm.use_zero_initial_guess != 0;
    const double *bm[3] = {c->bb[0].p, c->bb[1].p, c->bb[2].p};
    double *xm[3] = {c->xb[0].p, c->xb[1].p, c->xb[2].p};
    const double *bp[1] = {c->bb[3].p};
    double *xp[1] = {c->xb[3].p};
    c->kmom.bind(c->st, bm, xm, ~0u, zg);
    c->kp.bind(c->st, bp, xp, ~0u, true);
    c->graph_bound = true;
  }
  if (!a.graph_ready) build_adjoint_graph(c);
  else if (!a.graph_bound) bind_transposed(c);
  IBM_CUDA_TRY(cudaGraphLaunch(a.gexec, c->st));
  IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
  IBM_CUDA_TRY(cudaGetLastError());
  const unsigned long long *lp = t->hloops;
  c->launches += a.graph_fixed_launches + (long long)lp[0] * a.graph_body_launches[0] +
                 (long long)lp[1] * a.graph_body_launches[1] + (long long)lp[2] * a.graph_body_launches[2] +
                 (long long)lp[3] * a.graph_body_launches[3];
  int rc = IBM_OK;
  for (int s = 0; s < 4; ++s) {
    const KFlags &f = (s == 3 && c->p_sym) ? c->hflags_graph[3] : t->hflags_graph[s];
    KResult r;
    r.iters = f.iters; r.rel_res = f.rel; r.status = f.status; r.nonfinite = f.nonfinite;
    a.last[s] = r;
    if (r.nonfinite) throw Error(IBM_ERR_NONFINITE, "non-finite transposed solve");
    rc = worst(rc, solve_status(r));
  }
  return rc;
}

void sync_transposed_params(ibm_ctx *c) {
  ibm_ctx *t = c->adj->t;
  ibm_solver_params p = c->prm;
  p.use_graph = 0;
  p.compute_forces = 0;
  if (c->p_sym) p.p_pc = 0;  // the pressure transpose is solved with the step's own solver
  if (memcmp(&p, &t->prm, sizeof(p)) != 0) {
    const int rc = ibm_set_solver_params(t, &p);
    if (rc < 0) throw Error(rc, "transposed context: " + t->err);
    c->adj->graph_ready = false;
  }
}

}  // namespace

int ibm_adjoint_setup(ibm_ctx *c, const double *beta_p) {
  return guarded(c, [&]() {
    if (!beta_p) throw Error(IBM_ERR_ARG, "ibm_adjoint_setup: null beta_p");
    require_inputs(c);
    if (!c->adj) c->adj = new ibm::AdjState();
    ibm::AdjState &a = *c->adj;
    if (a.gexec) cudaGraphExecDestroy(a.gexec);
    a.gexec = nullptr;
    a.graph_ready = false;
    if (a.t) { ibm_destroy(a.t); a.t = nullptr; }
    int rc = ibm_create(&c->grid, &a.t);
    if (rc < 0) throw Error(rc, "transposed context: " + g_create_error);
    a.t->adj_owner = c;
    for (int f = 0; f < 4; ++f) {
      const Box &b = field_box(c, f);
      DBuf<double> rows;
      rows.alloc((size_t)7 * b.n);
      launch_transpose7(c->st, c->op[f].c.p, b, rows.p);
      IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
      rc = ibm_set_operator(a.t, f, rows.p, b.nx, b.ny, b.nz);
      if (rc < 0) throw Error(rc, "transposed context: " + a.t->err);
    }
    sync_transposed_params(c);
    const Geometry &g = c->g;
    const auto beta = to_host(beta_p, (size_t)g.NP);
    const auto fc = to_host(c->fc.p, (size_t)g.NP);
    const int nyz = g.ny * g.nz;
    std::vector<double> bdx(nyz, 0.0), winl(nyz, 0.0);
    for (int t = 0; t < nyz; ++t) {
      const long cell = (long)t * g.nx;
      if (fc[cell] & kFluid) {
        bdx[t] = beta[cell] * g.dx;
        winl[t] = 1.0 / bdx[t];
      }
    }
    upload(a.bdx, bdx, c->st);
    upload(a.winl, winl, c->st);
    a.lu.alloc(g.NU); a.lv.alloc(g.NV); a.lw.alloc(g.NW); a.lp.alloc(g.NP);
    a.cu.alloc(g.NU); a.cv.alloc(g.NV); a.cw.alloc(g.NW);
    a.gu.alloc(g.NU); a.gv.alloc(g.NV); a.gw.alloc(g.NW);
    a.u1.alloc(g.NU); a.v1.alloc(g.NV); a.w1.alloc(g.NW);
    a.mu.alloc(g.NP);
    a.dg.alloc(nyz); a.acc.alloc(1);
    a.dweight.alloc(1);
    if (!a.hweight) IBM_CUDA_TRY(cudaMallocHost((void **)&a.hweight, sizeof(double)));
    a.lu.zero(c->st); a.lv.zero(c->st); a.lw.zero(c->st); a.lp.zero(c->st);
    a.dg.zero(c->st); a.acc.zero(c->st);
    a.tape.clear();
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    // solver set-up of both contexts now rather than in the first reverse step
    ensure_solvers(c);
    {
      Scope sc(a.t);
      ensure_solvers(a.t);
    }
    return IBM_OK;
  });
}

int ibm_set_inflow(ibm_ctx *c, const double *g) {
  return guarded(c, [&]() {
    ibm::AdjState &a = adj_of(c);
    if (!g) throw Error(IBM_ERR_ARG, "ibm_set_inflow: null profile");
    const size_t nyz = (size_t)c->g.ny * c->g.nz;
    DBuf<double> dg;
    dg.alloc(nyz);
    IBM_CUDA_TRY(cudaMemcpyAsync(dg.p, g, sizeof(double) * nyz, cudaMemcpyDefault, c->st));
    (void)a;
    adj_set_inflow(c, dg.p);
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

int ibm_step_forward(ibm_ctx *c, double ramp, ibm_step_stats *stats) {
  return guarded(c, [&]() {
    ibm::AdjState &a = adj_of(c);
    require_inputs(c);
    ibm::TapeEntry e;
    if (!a.spare.empty()) {
      e = std::move(a.spare.back());
      a.spare.pop_back();
    }
    double *f[4] = {c->u.p, c->v.p, c->w.p, c->p.p};
    const long n[4] = {c->g.NU, c->g.NV, c->g.NW, c->g.NP};
    for (int q = 0; q < 4; ++q) copy_into(c, e.s0[q], f[q], n[q]);
    step_launch(c, ramp);
    const int rc = step_collect(c, ramp, &e.stats);
    if (rc >= 0) {
      for (int q = 0; q < 3; ++q) {
        copy_into(c, e.b[q], c->bb[q].p, field_box(c, q).n);
        copy_into(c, e.x[q], c->xb[q].p, field_box(c, q).n);
      }
      for (int q = 0; q < 4; ++q) copy_into(c, e.s1[q], f[q], n[q]);
      e.ramp = ramp;
      IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
      a.tape.push_back(std::move(e));
    }
    if (stats) *stats = e.stats;
    return rc;
  });
}

int ibm_step_backward(ibm_ctx *c, double ramp, double weight, ibm_step_stats *stats) {
  return guarded(c, [&]() {
    ibm::AdjState &a = adj_of(c);
    if (a.tape.empty()) throw Error(IBM_ERR_STATE, "ibm_step_backward: no step on the tape (ibm_step_forward)");
    if (ramp != a.tape.back().ramp) throw Error(IBM_ERR_ARG, "ibm_step_backward: ramp differs from the taped step's");
    sync_transposed_params(c);
    ibm::TapeEntry e = std::move(a.tape.back());
    a.tape.pop_back();
    // the taped step's forward results: momentum right-hand sides and
    // solutions into bb / xb, the end-of-step fields into u, v, w, p
    for (int q = 0; q < 3; ++q) {
      IBM_CUDA_TRY(cudaMemcpyAsync(c->bb[q].p, e.b[q].p, sizeof(double) * e.b[q].n, cudaMemcpyDeviceToDevice, c->st));
      IBM_CUDA_TRY(cudaMemcpyAsync(c->xb[q].p, e.x[q].p, sizeof(double) * e.x[q].n, cudaMemcpyDeviceToDevice, c->st));
    }
    restore(c, e.s1);
    *c->hramp = ramp;
    IBM_CUDA_TRY(cudaMemcpyAsync(c->dramp.p, c->hramp, sizeof(double), cudaMemcpyHostToDevice, c->st));
    // post-BC start velocities: the convection's linearisation point
    IBM_CUDA_TRY(cudaMemcpyAsync(a.u1.p, e.s0[0].p, sizeof(double) * c->g.NU, cudaMemcpyDeviceToDevice, c->st));
    IBM_CUDA_TRY(cudaMemcpyAsync(a.v1.p, e.s0[1].p, sizeof(double) * c->g.NV, cudaMemcpyDeviceToDevice, c->st));
    IBM_CUDA_TRY(cudaMemcpyAsync(a.w1.p, e.s0[2].p, sizeof(double) * c->g.NW, cudaMemcpyDeviceToDevice, c->st));
    *a.hweight = weight;
    const int rr = c->prm.use_graph ? reverse_graph(c) : (
        [&]() {
          IBM_CUDA_TRY(cudaMemcpyAsync(a.dweight.p, a.hweight, sizeof(double), cudaMemcpyHostToDevice, c->st));
          launch_bc(c, a.u1.p, a.v1.p, a.w1.p);
          return reverse_host(c);
        })();
    IBM_CUDA_TRY(cudaGetLastError());
    c->prof.drain();
    if (stats) *stats = e.stats;
    const int rc = e.stats.status;
    a.spare.push_back(std::move(e));
    return worst(rc, rr);
  });
}

int ibm_adjoint_reset(ibm_ctx *c) {
  return guarded(c, [&]() {
    ibm::AdjState &a = adj_of(c);
    a.lu.zero(c->st); a.lv.zero(c->st); a.lw.zero(c->st); a.lp.zero(c->st);
    a.dg.zero(c->st); a.acc.zero(c->st);
    for (auto &e : a.tape) a.spare.push_back(std::move(e));
    a.tape.clear();
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

int ibm_adjoint_set(ibm_ctx *c, const double *lu, const double *lv, const double *lw, const double *lp) {
  return guarded(c, [&]() {
    ibm::AdjState &a = adj_of(c);
    const double *src[4] = {lu, lv, lw, lp};
    DBuf<double> *dst[4] = {&a.lu, &a.lv, &a.lw, &a.lp};
    for (int q = 0; q < 4; ++q) {
      if (src[q]) IBM_CUDA_TRY(cudaMemcpyAsync(dst[q]->p, src[q], sizeof(double) * dst[q]->n, cudaMemcpyDefault, c->st));
      else dst[q]->zero(c->st);
    }
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

int ibm_adjoint_get(ibm_ctx *c, double *lu, double *lv, double *lw, double *lp, double *dg, double *dnu) {
  return guarded(c, [&]() {
    ibm::AdjState &a = adj_of(c);
    double *dst[6] = {lu, lv, lw, lp, dg, dnu};
    const DBuf<double> *src[6] = {&a.lu, &a.lv, &a.lw, &a.lp, &a.dg, &a.acc};
    for (int q = 0; q < 6; ++q)
      if (dst[q]) IBM_CUDA_TRY(cudaMemcpyAsync(dst[q], src[q]->p, sizeof(double) * src[q]->n, cudaMemcpyDefault, c->st));
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

int ibm_adjoint_solve_stats(ibm_ctx *c, ibm_solve_stats *out) {
  return guarded(c, [&]() {
    if (!out) throw Error(IBM_ERR_ARG, "ibm_adjoint_solve_stats: null output");
    ibm::AdjState &a = adj_of(c);
    for (int q = 0; q < 4; ++q) fill_solve(out[q], a.last[q]);
    return IBM_OK;
  });
}

int ibm_adjoint_tape_depth(ibm_ctx *c) {
  return guarded(c, [&]() { return (int)adj_of(c).tape.size(); });
}

int ibm_checkpoint_save(ibm_ctx *c, int slot) {
  return guarded(c, [&]() {
    ibm::AdjState &a = adj_of(c);
    a.ckpt[slot] = snapshot(c);
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

int ibm_checkpoint_load(ibm_ctx *c, int slot) {
  return guarded(c, [&]() {
    ibm::AdjState &a = adj_of(c);
    auto it = a.ckpt.find(slot);
    if (it == a.ckpt.end()) throw Error(IBM_ERR_ARG, "ibm_checkpoint_load: no checkpoint in slot " + std::to_string(slot));
    restore(c, it->second);
    IBM_CUDA_TRY(cudaStreamSynchronize(c->st));
    return IBM_OK;
  });
}

int ibm_checkpoint_clear(ibm_ctx *c) {
  return guarded(c, [&]() {
    adj_of(c).ckpt.clear();
    return IBM_OK;
  });
}

}  // extern "C"

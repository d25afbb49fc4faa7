// Semicoarsening multigrid preconditioner for the pressure operator (see ibm_mg.cu).
#pragma once
#include "ibm_common.cuh"
#include "ibm_krylov.cuh"

namespace ibm {

struct MgParams {
  int rap = 0;          // 0 Galerkin 27-point, 1 collapsed to 7 points
  int relax = 1;        // 1 weighted Jacobi, 2 two-colour (red-black) relaxation
  int nu1 = 1, nu2 = 1;
  double omega = 2.0 / 3.0;
  int coarse_max = 64;
  int max_levels = 40;
  int cycles = 1;       // V-cycles per application
  int nu_coarse = 0;    // sweeps each way on the coarser relaxed levels (0: nu1 / nu2)
  double group_ratio = 0.0;  // see ibm_solver_params.mg_group_ratio
  int options = 3;      // see ibm_solver_params.mg_options
  int classes = 1;      // colour-split records as record classes where they repeat (ibm_classes.cu)
  int quads = 1;        // FP32 7-point phases and residual four points per thread (nx % 4 == 0)
  int fused_sweep = 0;    // FP32 7-point levels: one kernel per two-colour sweep (k_relax_rb_sweep)
  long fused_coarse = 0;  // FP32: levels from the first one below the finest with at most this many
                          // points run as one persistent cooperative kernel (ibm_mg.cu); 0: off
};

template <class T>
struct MgLevelT {
  Box b;
  int cdir = -1;        // direction coarsened to reach the next level; -1 on the coarsest
  int relax = 1;        // 0 inside a coarsening group: restrict and interpolate only
  int ns = 7;           // stencil slots stored: 7 (Struct order) or 27
  const T *A = nullptr; // [ns][n] planes (level 0 points at the operator itself)
  DBuf<T> Aown, wd, invd, pm, pp, x, bv, r, t, dense;
  DBuf<T> rb;           // colour-split coefficients for the in-place two-colour relaxation (7-point, even nx)
  DBuf<T> rb27;         // colour-split 27-point coefficients + inverse diagonal (two-colour relaxation)
  Classes<T> rbc;       // the classes of rb or rb27 (W 8 or 28); the plain records are then released
};

class Multigrid {
 public:
  // Builds the hierarchy from a 7-point operator (FP64 planes, and FP32 planes
  // when fp32 is requested). h = grid spacing used to pick coarsening directions.
  // winv (device, may be null): the hierarchy is built on diag(winv) A and
  // every application scales its input by winv.
  void setup(cudaStream_t st, const Box &b, const double *A7, const float *A7f, const double h[3],
             const MgParams &p, bool fp64, bool fp32, const double *winv);
  // out = M in (every kernel gated on *gate when gate != nullptr).
  void apply(cudaStream_t st, const VecRef &in, const OutRef &out, const int *gate, bool use_fp32);
  int levels() const { return (int)L64.size() ? (int)L64.size() : (int)L32.size(); }
  void level_info(int l, int dims[3], int *cdir, int *ns) const;
  // Copies level l's coefficients as [n][27] (FP64 hierarchy).
  void level_coef27(cudaStream_t st, int l, double *host_out) const;
  size_t bytes() const;
  MgParams prm;

 private:
  template <class T>
  void build(cudaStream_t st, std::vector<MgLevelT<T>> &L, const Box &b, const T *A7, const double h[3]);
  template <class T>
  void cycle(cudaStream_t st, std::vector<MgLevelT<T>> &L, int l, const int *gate);
  void build_tail(cudaStream_t st);
  std::vector<MgLevelT<double>> L64;
  std::vector<MgLevelT<float>> L32;
  // The fused coarse levels of the FP32 hierarchy: the phase list (device
  // copy of the kernel's descriptors), its barrier state, the buffer the
  // phases leave level 1's correction in, their algorithmic bytes, blocks.
  DBuf<unsigned char> tail_ops_;
  DBuf<unsigned> tail_bar_;
  int tail_nops_ = 0, tail_blocks_ = 0, tail_level_ = 0;
  float *tail_out_ = nullptr;
  double tail_bytes_ = 0.0;
  const double *winv_ = nullptr;
  DBuf<float> winvf_;   // FP32 copy of winv_ for the FP32 hierarchy
};

}  // namespace ibm

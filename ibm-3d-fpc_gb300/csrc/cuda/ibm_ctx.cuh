// The solver context behind the C ABI (one GPU, one stream).
#pragma once
#include "ibm_common.cuh"
#include "ibm_krylov.cuh"
#include "ibm_mg.cuh"

namespace ibm {

// Face flag bits (u, v, w faces; full MAC layouts).
constexpr uint8_t kActive = 1;   // active_{u,v,w} at the face itself
constexpr uint8_t kQFace = 2;    // id_q > 0: part of the projection vector q
constexpr uint8_t kRhsRow = 4;   // id > 0 && active: a solved (non-identity) momentum row
constexpr uint8_t kBcSet = 8;    // the BC cleanup overwrites this face (boundary plane or zero list)
// Cell flag bit.
constexpr uint8_t kFluid = 1;    // fluid_p && id_p > 0

struct StepDiag {                // written by the diagnostics kernel
  double div2, umax, vmax, wmax;
  int nonfinite_mom, nonfinite_p;
  unsigned ticket;
  int pad;
  double force[3];               // force of the fluid on the body (k_forces)
  unsigned fticket;
  int pad2;
};

struct Geometry {
  int nx, ny, nz;
  long NU, NV, NW, NP;           // full MAC sizes
  Box bu, bv, bw, bp;            // solve boxes
  double dx, dy, dz, rho, nu, dt;
};

struct AdjState;  // adjoint extension (ibm_adjoint.cuh)

}  // namespace ibm

struct ibm_ctx;
namespace ibm {
// cut-surface force (ibm_force.cu)
void launch_forces_cut(ibm_ctx *c);
void adj_force_cut(ibm_ctx *c, const double *weight, double *lu, double *lp, double *acc);
void build_cut_force(ibm_ctx *c, double xcirc, double ycirc, double Rcirc, const std::vector<double> &alpha_u,
                     const std::vector<double> &alpha_v);
}  // namespace ibm

struct ibm_ctx {
  ibm_grid_desc grid;
  ibm::Geometry g;
  int device = 0;
  cudaStream_t st = nullptr;
  ibm_solver_params prm;
  std::string err;
  long long launches = 0;

  ibm::Op7 op[4];
  bool p_sym = false;            // the pressure operator is W S (W diagonal, S symmetric)
  ibm::DBuf<double> p_winv;      // 1 / W
  bool masks_set = false, aux_set = false, csr_set = false;
  int np_active = 0;             // number of fluid cells with an id (the reference's Np)
  ibm::DBuf<uint8_t> fu, fv, fw, fc;
  ibm::DBuf<double> scale_box[3], bc_box[3];
  ibm::DBuf<double> div_bc_cell, uin;
  ibm::DBuf<double> Dc;          // [6][NP]: u_w, u_e, v_s, v_n, w_b, w_t
  ibm::DBuf<double> Gu, Gv, Gw;  // [2][faces]: coefficient of the lower / upper cell
  ibm::DBuf<int> zl_u, zl_v, zl_w;
  // host copies needed to convert the CSR (kept after ibm_set_masks)
  std::vector<int32_t> h_id_p, h_id_qu, h_id_qv, h_id_qw;
  std::vector<int32_t> h_id_u_rows, h_id_v_rows, h_id_w_rows;  // id of each solve-box row (0: identity row)
  int n_id[3] = {0, 0, 0};       // largest momentum ids
  std::vector<uint8_t> h_act_u, h_act_v, h_act_w, h_fluid;  // masks (for ibm_set_body)
  // cut-surface force (ibm_set_body; ibm_force.cu): entry codes, indices, weights
  bool body_set = false;
  long cf_n = 0;
  ibm::DBuf<uint8_t> cf_code;
  ibm::DBuf<int> cf_idx;
  ibm::DBuf<double> cf_w;

  ibm::DBuf<double> u, v, w, p, ut, vt, wt;
  ibm::DBuf<float2> df_u, df_v, df_w, df_p;  // double-float copies of u, v, w, p (df_rhs)
  ibm::DBuf<double> xb[4], bb[4];
  ibm::DBuf<double> part;        // diagnostics block partials
  ibm::DBuf<ibm::StepDiag> diag;
  ibm::StepDiag *hdiag = nullptr;
  // results of the step being collected (the halves of ibm_step)
  ibm::KResult last_rm[3], last_rp[1];
  bool last_graph = false;

  bool solvers_ready = false;
  int solvers_precision = -1;
  ibm::Krylov kmom, kp;
  ibm::Multigrid mg;
  cudaEvent_t ev[6] = {};
  ibm::Prof prof;

  // Inlet ramp of the current step, read by the kernels on the device.
  ibm::DBuf<double> dramp;
  double *hramp = nullptr;            // pinned staging copy
  // Captured step (use_graph): one launch runs the whole step, GMRES loops included.
  cudaGraphExec_t gexec = nullptr;
  bool graph_ready = false;
  bool graph_bound = false;           // the Krylov system tables hold the step's full masks
  cudaStream_t cap[2] = {};           // streams that capture conditional-node bodies
  ibm::KFlags *hflags_graph = nullptr;  // pinned: u, v, w, p solve flags after a graph step
  ibm::DBuf<unsigned long long> dloops;  // loop-body counters (momentum x2, pressure x2)
  unsigned long long *hloops = nullptr;  // pinned copy
  long long graph_fixed_launches = 0;
  long long graph_body_launches[4] = {0, 0, 0, 0};
  // Adjoint extension: transposed-operator context, lambdas, tape, checkpoints.
  ibm::AdjState *adj = nullptr;
  ibm_ctx *adj_owner = nullptr;       // a transposed-operator context: the context it serves
};

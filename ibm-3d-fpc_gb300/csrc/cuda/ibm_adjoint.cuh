// Adjoint extension: state and launchers of the reverse sweep of one step.
//
// The reference has no adjoint. The step is s1 = step(s0; g, nu) with g the
// inflow profile (u at the inlet = ramp g, and the inlet column's divergence
// lift -g / (beta dx)) and nu the viscosity (momentum operators, row scales
// and inlet diffusion lift); the reverse sweep maps the lambda of the
// end-of-step fields to the lambda of the step-start fields and accumulates
// dJ/dg and dJ/dnu. Dense transposes are kernels here; the transposed solves
// run on a second context that holds the transposed operators.
#pragma once
#include <array>
#include <map>
#include <vector>

#include "ibm_ctx.cuh"

namespace ibm {

// One step on the tape: its start state and what the reverse sweep needs of
// its forward computation (the momentum right-hand sides and solutions, the
// end-of-step fields), so that the reverse step does not recompute it.
struct TapeEntry {
  std::array<DBuf<double>, 4> s0;         // u, v, w, p at the step start
  std::array<DBuf<double>, 3> b, x;       // momentum right-hand sides and solutions (solve boxes)
  std::array<DBuf<double>, 4> s1;         // u, v, w, p at the step end
  double ramp = 0.0;
  ibm_step_stats stats;
};

struct AdjState {
  ibm_ctx *t = nullptr;                   // context on the transposed operators
  DBuf<double> lu, lv, lw, lp;            // lambda of the current state (full MAC arrays, cells)
  DBuf<double> cu, cv, cw;                // per-face lambda of the convection
  DBuf<double> gu, gv, gw;                // per-face lambda of the pressure gradient
  DBuf<double> u1, v1, w1;                // post-BC step-start velocities (the convection's linearisation point)
  DBuf<double> dg, acc;                   // dJ/dg[ny*nz]; acc[0] = dJ/dnu
  DBuf<double> bdx, winl;                 // per inlet cell: beta dx and 1 / (beta dx) (0: not fluid)
  DBuf<double> mu;                        // Ap^-T of the projection's lambda (cells)
  DBuf<double> dweight;                   // objective weight of the step being reversed (device copy)
  double *hweight = nullptr;              // pinned staging copy
  std::vector<TapeEntry> tape;            // steps pushed by ibm_step_forward
  std::vector<TapeEntry> spare;           // popped entries kept for reuse (no allocation per step)
  std::map<int, std::array<DBuf<double>, 4>> ckpt;  // checkpoints (ibm_checkpoint_save)
  // The reverse sweep captured as one graph (forward steps in graph mode):
  // the transposed solves run their loops on the device.
  cudaGraphExec_t gexec = nullptr;
  bool graph_ready = false;
  bool graph_bound = false;               // the transposed Krylov systems are bound to the graph's vectors
  long long graph_fixed_launches = 0;
  long long graph_body_launches[4] = {0, 0, 0, 0};
  KResult last[4];                        // the last reverse sweep's transposed solves (u, v, w, p)
  ~AdjState();
};

// Row-major [n][7] transpose of a planes [7][n] operator on box b.
void launch_transpose7(cudaStream_t st, const double *planes, const Box &b, double *rows);
// Lambda of the BC cleanup (inlet values ramp g, ramp read on the device):
// the overwritten faces' lambdas become 0, the outlet copy hands its lambda
// to u[nx-1], dg += ramp lambda at the inlet.
void adj_bc(ibm_ctx *c, double *lu, double *lv, double *lw, const double *ramp);
// lambda += weight dF_x/d(fields) at the context's end-of-step fields; acc += weight dF_x/dnu.
void adj_force(ibm_ctx *c, const double *weight);
// rphi = lambda_p - (dt/rho) G^T lambda_q on fluid cells (0 elsewhere).
void adj_projection(ibm_ctx *c, double *rphi);
// lambda_q += -(rho/dt) D^T mu; dg += (rho/dt) ramp mu / (beta dx) on the inlet column.
void adj_divergence(ibm_ctx *c, const double *mu, const double *ramp);
// lx[f] = lambda on the solve-box interiors, which become 0.
void adj_scatter(ibm_ctx *c, double *const *lx);
// From lb[f] = A^-T lx[f]: the right-hand sides' lambdas (u, convection, gradient) and dJ/dnu.
void adj_momentum(ibm_ctx *c, const double *const *lb);
// lambda_p += G^T of the gradient lambdas.
void adj_gradient(ibm_ctx *c);
// y = x / winv (divide) or x * winv: the diagonal W of Ap = W S (S symmetric)
// turns Ap^T = W^-1 Ap W into a solve with Ap itself.
void adj_wscale(ibm_ctx *c, const double *x, double *y, bool divide);
// Inflow g: u at the inlet and the inlet column's divergence lift.
void adj_set_inflow(ibm_ctx *c, const double *g);

}  // namespace ibm

// Launchers of the dense per-step kernels (ibm_step.cu). The inlet ramp is
// read on the device from ctx->dramp, so a captured step replays with the
// ramp of each call.
#pragma once
#include "ibm_ctx.cuh"

namespace ibm {
void launch_bc(ibm_ctx *c, double *u, double *v, double *w);
void launch_momentum_rhs(ibm_ctx *c);
// The right-hand side of mixed-precision momentum solves is double-float
// (df_rhs); its field copies are allocated outside any graph capture.
bool momentum_rhs_df(const ibm_solver_params &p);
void ensure_rhs_df(ibm_ctx *c);
void launch_tilde(ibm_ctx *c);
void launch_pressure_rhs(ibm_ctx *c);
void launch_projection(ibm_ctx *c);
}  // namespace ibm

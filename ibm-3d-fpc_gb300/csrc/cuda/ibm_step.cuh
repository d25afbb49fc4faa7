// Launchers of the dense per-step kernels (ibm_step.cu). The inlet ramp is
// read on the device from ctx->dramp, so a captured step replays with the
// ramp of each call.
#pragma once
#include "ibm_ctx.cuh"

namespace ibm {
void launch_bc(ibm_ctx *c, double *u, double *v, double *w);
void launch_momentum_rhs(ibm_ctx *c);
void launch_tilde(ibm_ctx *c);
void launch_pressure_rhs(ibm_ctx *c);
void launch_projection(ibm_ctx *c);
}  // namespace ibm

// Launchers of the dense per-step kernels (ibm_step.cu).
#pragma once
#include "ibm_ctx.cuh"

namespace ibm {
void launch_bc(ibm_ctx *c, double *u, double *v, double *w, double ramp);
void launch_momentum_rhs(ibm_ctx *c);
void launch_tilde(ibm_ctx *c, double ramp);
void launch_pressure_rhs(ibm_ctx *c, double ramp);
void launch_projection(ibm_ctx *c, double ramp);
}  // namespace ibm

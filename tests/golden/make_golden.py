"""Regenerate the golden fixtures in this directory.

Needs the reference sources (compiled by oracle/Makefile into oracle/_ref/)
and the oracle; run from the repository root:

    python tests/golden/make_golden.py

Fixtures (all small, compressed):
  setup_channel_32x12x12.npz  reference setup arrays, benchmark channel geometry
  setup_default_32x12x12.npz  reference setup arrays, the reference's default geometry
                              and the run example of README_BUILD.txt (dt 2e-3)
  twins_channel_32x12x12.npz  seeded fields and the reference's CPU BC cleanup and
                              centred convection of them
  oracle_channel_32x12x12.npz oracle state after 5 steps (ramp over 4 steps), tight tolerances,
                              PFMG's plain multigrid rules
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import importlib  # noqa: E402

import pyoracle  # noqa: E402

SETUP_NAMES = ["beta_p", "alpha_u", "alpha_v", "alpha_w", "fluid_p", "active_u", "active_v", "active_w",
               "active_qu", "active_qv", "active_qw", "id_u", "id_v", "id_w", "id_p", "id_qu", "id_qv", "id_qw",
               "scale_u", "scale_v", "scale_w", "rhs_u_bc", "rhs_v_bc", "rhs_w_bc", "div_bc_unit", "Au_vals",
               "Av_vals", "Aw_vals", "Ap_vals", "uin", "D_rowptr", "D_col", "D_val", "G_rowptr", "G_col", "G_val",
               "counts"]


def params_fields(p):
    return {n: getattr(p, n) for n, _ in p._fields_}


def main():
    pyoracle.build(with_reference=True)
    ibm = importlib.import_module("ibm-3d-fpc_gb300")
    chan = ibm.channel_params(32, 12, 12, Um=0.45, dt=1e-3)
    dflt = ibm.channel_params(32, 12, 12, Lx=2.2, xcirc=0.2, ycirc=0.2, Um=0.45, dt=2e-3)
    for tag, prm in (("channel", chan), ("default", dflt)):
        ref = pyoracle.ReferenceCase(prm)
        arrs = {n: ref.array(n) for n in SETUP_NAMES}
        np.savez_compressed(os.path.join(HERE, f"setup_{tag}_32x12x12.npz"),
                            params=np.array(list(params_fields(prm).values())), **arrs)
        print("wrote setup", tag)

    ref = pyoracle.ReferenceCase(chan)
    nx, ny, nz = 32, 12, 12
    rng = np.random.default_rng(20261203)
    u = rng.standard_normal((nx + 1) * ny * nz)
    v = rng.standard_normal(nx * (ny + 1) * nz)
    w = rng.standard_normal(nx * ny * (nz + 1))
    uin_step = 0.7 * ref.array("uin")
    ub, vb, wb = ref.enforce_bc(u, v, w, uin_step)
    cu, cv, cw = ref.convection(ub, vb, wb)
    np.savez_compressed(os.path.join(HERE, "twins_channel_32x12x12.npz"), u=u, v=v, w=w, ramp=0.7,
                        u_bc=ub, v_bc=vb, w_bc=wb, conv_u=cu, conv_v=cv, conv_w=cw)
    print("wrote twins")

    case = ibm.Case(chan)
    orc = pyoracle.Oracle(case, vel_tol=1e-13, p_tol=1e-13, mg_options=0)  # PFMG's plain multigrid rules
    stats = []
    for step in range(1, 6):
        st = orc.step(min(1.0, step / 4.0))
        stats.append([st.u.iters, st.v.iters, st.w.iters, st.p.iters, st.div_l2, st.umax, st.vmax, st.wmax])
    fu, fv, fw, fp = orc.fields()
    np.savez_compressed(os.path.join(HERE, "oracle_channel_32x12x12.npz"), u=fu, v=fv, w=fw, p=fp,
                        stats=np.array(stats), ramp_steps=4, nsteps=5)
    print("wrote oracle steps", stats[-1])


if __name__ == "__main__":
    main()

"""Small, fixed workloads for profiler captures (ncu) of single kernels.

    python ibm-3d-fpc_gb300/profile_case.py pc   640 128 64 [--repeat 4]
    python ibm-3d-fpc_gb300/profile_case.py step 640 128 64 [--repeat 3]

``pc``   applies the pressure preconditioner (mixed precision, the benchmark's
         multigrid settings) ``repeat`` times through ibm_apply_preconditioner.
``step`` runs ``repeat`` host-driven timesteps (every kernel launched from the
         host, so a profiler sees each launch) from the benchmark's initial state.

Both use Krylov bases of 8 vectors so that the device footprint stays at a few
GB for the sizes above.
"""
from __future__ import annotations

import argparse
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["pc", "step"])
    ap.add_argument("nx", type=int)
    ap.add_argument("ny", type=int)
    ap.add_argument("nz", type=int)
    ap.add_argument("--repeat", type=int, default=4)
    ap.add_argument("--precision", type=int, default=2)
    a = ap.parse_args()
    sys.path.insert(0, os.path.dirname(HERE))
    ibm = importlib.import_module(os.path.basename(HERE))
    case = ibm.Case(ibm.channel_params(a.nx, a.ny, a.nz, Um=2.25, dt=2e-4))
    prm = ibm.solver_params(vel_tol=1e-8, p_tol=1e-8, vel_kdim=8, p_kdim=8, p_pc_rap_type=0, p_pc_relax_type=2,
                            mg_nu1=3, mg_nu2=3, mg_nu_coarse=2, mg_omega=1.0, mg_group_ratio=1.5, mg_options=3,
                            precision=a.precision, use_graph=0)
    s = ibm.Solver(case, prm)
    if a.mode == "pc":
        r = np.random.default_rng(3).standard_normal(a.nx * a.ny * a.nz)
        for _ in range(a.repeat):
            z = s.apply_preconditioner(ibm.FIELD_P, r)
        print("pc ok", float(np.abs(z).max()))
    else:
        for _ in range(a.repeat):
            st = s.step(1.0)
        print("step ok", st.p.iters, st.div_l2)
    return 0


if __name__ == "__main__":
    sys.exit(main())

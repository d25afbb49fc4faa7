"""Small, fixed workloads for profiler captures (ncu) of single kernels.

    python ibm-3d-fpc_gb300/profile_case.py pc   640 128 64 [--repeat 4]
    python ibm-3d-fpc_gb300/profile_case.py step 640 128 64 [--repeat 3]
    ... [--set name=value ...] [--time kernel_class]

``pc``   applies the pressure preconditioner (mixed precision, the benchmark's
         multigrid settings) ``repeat`` times through ibm_apply_preconditioner.
``step`` runs ``repeat`` host-driven timesteps (every kernel launched from the
         host, so a profiler sees each launch) from the benchmark's initial state.

Both use Krylov bases of 8 vectors so that the device footprint stays at a few
GB for the sizes above. ``--set`` overrides solver parameters (e.g. mg_quads=0);
``--time`` brackets every launch of one kernel class with CUDA events and
prints the mean per-launch time and algorithmic bandwidth (after one untimed
repetition).
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
    ap.add_argument("--set", action="append", default=[])
    ap.add_argument("--time", default=None)
    a = ap.parse_args()
    sys.path.insert(0, os.path.dirname(HERE))
    ibm = importlib.import_module(os.path.basename(HERE))
    case = ibm.Case(ibm.channel_params(a.nx, a.ny, a.nz, Um=2.25, dt=2e-4))
    prm = ibm.solver_params(vel_tol=1e-8, p_tol=1e-8, vel_kdim=8, p_kdim=8, p_pc_rap_type=0, p_pc_relax_type=2,
                            mg_nu1=3, mg_nu2=3, mg_nu_coarse=2, mg_omega=1.0, mg_group_ratio=1.5, mg_options=3,
                            precision=a.precision, use_graph=0)
    for kv in a.set:
        k, v = kv.split("=")
        setattr(prm, k, type(getattr(prm, k))(float(v)) if "." in v else int(v))
    s = ibm.Solver(case, prm)
    timed = None
    if a.time:
        timed = ibm.kernel_names().index(a.time)
    lib = s._lib
    r = np.random.default_rng(3).standard_normal(a.nx * a.ny * a.nz)
    for rep in range(a.repeat):
        if timed is not None and rep == 1:
            s.profile_reset()
            lib.ibm_profile_time_kernel(s._ctx, timed)
        if a.mode == "pc":
            z = s.apply_preconditioner(ibm.FIELD_P, r)
        else:
            st = s.step(1.0)
    if a.mode == "pc":
        print("pc ok", float(np.abs(z).max()))
    else:
        print("step ok", st.p.iters, st.div_l2)
    if timed is not None:
        pr = s.profile()
        n = max(pr.timed_launches[timed], 1)
        ms = pr.time_ms[timed] / n
        gb = pr.bytes[timed] / max(pr.launches[timed], 1) / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
        print(f"{a.time}: {pr.timed_launches[timed]} launches, {ms * 1e3:.2f} us each, {gb:.0f} GB/s algorithmic")
    return 0


if __name__ == "__main__":
    sys.exit(main())

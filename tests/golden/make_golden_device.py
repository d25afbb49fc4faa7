"""Regenerate refkernels_channel_32x12x12.npz: the outputs of the reference's
own device kernels (gpu_dense_ops.hpp, compiled from its sources by
``make -C oracle refcubin``) for one timestep's dense stages on a seeded
state, with seeded vectors standing in for the four solve outputs.

Needs a CUDA GPU (sm_103a) and oracle/_ref/ref_kernels.cubin; run from the
repository root:

    python tests/golden/make_golden_device.py

The CPU tests compare the oracle's stages with these bit for bit.
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import refgpu  # noqa: E402

SHAPE = (32, 12, 12)
RAMP = 0.7
SEED = 20261204


def state_and_solves(case):
    nx, ny, nz = case.shape
    rng = np.random.default_rng(SEED)
    u = rng.standard_normal((nx + 1) * ny * nz)
    v = 0.3 * rng.standard_normal(nx * (ny + 1) * nz)
    w = 0.3 * rng.standard_normal(nx * ny * (nz + 1))
    p = rng.standard_normal(nx * ny * nz) * case.array("fluid_p")
    xs = [rng.standard_normal(n) for n in ((nx - 1) * ny * nz, nx * (ny - 1) * nz, nx * ny * (nz - 1), nx * ny * nz)]
    return (u, v, w, p), xs


def main():
    ibm = importlib.import_module("ibm-3d-fpc_gb300")
    case = ibm.Case(ibm.channel_params(*SHAPE, Um=0.45, dt=1e-3))
    (u, v, w, p), xs = state_and_solves(case)
    out = refgpu.ReferenceStep(case).run(u, v, w, p, RAMP, lambda f, rhs: xs[f])
    np.savez_compressed(os.path.join(HERE, "refkernels_channel_32x12x12.npz"), ramp=RAMP, seed=SEED,
                        **{k: np.asarray(val) for k, val in out.items()})
    print("wrote refkernels", {k: float(np.abs(np.asarray(val)).max()) for k, val in out.items()})


if __name__ == "__main__":
    main()

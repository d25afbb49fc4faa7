"""The reference's own device kernels (gpu_dense_ops.hpp, compiled from its
sources into a cubin and launched in the order of main.cu:249-357 by
oracle/refgpu.py) against the library's step and against the oracle's
restatement of them, on the same state and the same solve outputs.

Both sides take the library's solve outputs, so every dense stage is
compared: momentum right-hand sides (BC cleanup, convection, G p, the
right-hand-side build), the pressure right-hand side (scatter, BC, packing,
D q), the projected fields (G phi, q correction, unpacking, BC, p += phi)
and the diagnostics. The reference leaves floating-point contraction to
nvcc in one expression (the momentum right-hand side's first difference,
which nvcc contracts into one fused multiply-add); the library and the
oracle spell that contraction out, so every stage is compared bit for bit.

Skipped where the cubin was not built (it needs the reference's sources).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

refgpu = pytest.importorskip("refgpu")
if not refgpu.available():
    pytest.skip("the reference's kernels were not built here (make -C oracle refcubin needs its sources)",
                allow_module_level=True)

STAGES = ("rhs_u", "rhs_v", "rhs_w", "rhs_p", "u", "v", "w", "p")


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def random_state(case, seed):
    nx, ny, nz = case.shape
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((nx + 1) * ny * nz), 0.3 * rng.standard_normal(nx * (ny + 1) * nz),
            0.3 * rng.standard_normal(nx * ny * (nz + 1)), rng.standard_normal(nx * ny * nz) * case.array("fluid_p"))


@pytest.mark.parametrize("shape,um,dt,ramp", [((48, 16, 16), 1.0, 1e-3, 0.6), ((160, 32, 32), 0.45, 1e-3, 0.25),
                                             ((640, 128, 128), 2.25, 2e-4, 1.0)],
                         ids=["48x16x16", "160x32x32", "640x128x128"])
def test_reference_kernels_match_library_and_oracle(ibm, pyoracle, shape, um, dt, ramp):
    case = ibm.Case(ibm.channel_params(*shape, Um=um, nu=1e-3, dt=dt))
    s = ibm.Solver(case, ibm.solver_params(vel_tol=1e-10, p_tol=1e-10, vel_maxit=500, p_maxit=500))
    try:
        u, v, w, p = random_state(case, sum(shape))
        s.set_fields(u, v, w, p)
        st = s.step(ramp)
        assert st.status in (ibm.IBM_OK, ibm.IBM_NOT_CONVERGED)
        ours = {"rhs_" + "uvw"[f]: s.solver_vector(f, 0) for f in range(3)}
        ours["rhs_p"] = s.solver_vector(3, 0)
        xs = [s.solver_vector(f, 1) for f in range(4)]
        ours.update(zip("uvwp", s.fields()))

        ref = refgpu.ReferenceStep(case).run(u, v, w, p, ramp, lambda f, rhs: xs[f])

        orc = pyoracle.Oracle(case)
        ub, vb, wb = orc.bc_cleanup(u, v, w, ramp)
        oracle = dict(zip(("rhs_u", "rhs_v", "rhs_w"), orc.momentum_rhs(ub, vb, wb, p)))
        orc.set_fields(ub, vb, wb, p)
        ut, vt, wt = orc.tilde(*xs[:3], ramp)
        oracle["rhs_p"] = orc.pressure_rhs(ut, vt, wt, ramp)
        ost = orc.projection(ut, vt, wt, xs[3], ramp)
        oracle.update(zip("uvwp", orc.fields()))

        report = {k: (bits_equal(ours[k], ref[k]), rel_err(ours[k], ref[k]), bits_equal(oracle[k], ref[k]),
                      rel_err(oracle[k], ref[k])) for k in STAGES}
        print(shape, report)
        for k in STAGES:
            assert report[k][0] and report[k][2], (k, report[k])
        assert st.umax == ref["umax"] and st.vmax == ref["vmax"] and st.wmax == ref["wmax"]
        assert ost.umax == ref["umax"]
        assert abs(st.div_l2 - ref["div_l2"]) <= 1e-12 * max(ref["div_l2"], 1e-300) + 1e-300
    finally:
        s.close()

"""Fused multigrid kernels against one launch per phase: the same per-point
arithmetic, so V-cycles and whole steps must agree bit for bit, repeatedly
(a missed barrier, a stale read or a halo mistake would show as a
difference).

- mg_fused_coarse: every phase below a level in one persistent cooperative
  kernel with grid-wide barriers;
- mg_fused_sweep: both colour phases of a 7-point level's sweep in one
  kernel on shared-memory tiles with a halo, out of place."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def bench_like(ibm, **kw):
    base = dict(vel_tol=1e-8, p_tol=1e-8, p_pc=1, p_pc_rap_type=0, p_pc_relax_type=2, mg_nu1=3, mg_nu2=3,
                mg_nu_coarse=2, mg_omega=1.0, mg_group_ratio=1.5, mg_coarse_max=2560, mg_options=3)
    base.update(kw)
    return ibm.solver_params(**base)


@pytest.mark.parametrize("shape,fuse", [((48, 16, 16), 1), ((96, 32, 16), 1), ((640, 128, 128), 1),
                                        ((640, 128, 128), 1 << 30)],
                         ids=["48x16x16", "96x32x16", "640x128x128", "640x128x128-all-coarse"])
def test_fused_vcycle_bitwise(ibm, shape, fuse):
    """mg_fused_coarse 1 fuses from the first level of at most 262144 points
    (160x32x32 on the 640x128x128 channel); 2^30 fuses every level below the
    finest."""
    case = ibm.Case(ibm.channel_params(*shape, Um=2.25, dt=2e-4))
    fused = ibm.Solver(case, bench_like(ibm, precision=1, mg_fused_coarse=fuse))
    plain = ibm.Solver(case, bench_like(ibm, precision=1, mg_fused_coarse=0))
    try:
        rng = np.random.default_rng(7)
        n = shape[0] * shape[1] * shape[2]
        for _ in range(3):
            r = rng.standard_normal(n)
            za = fused.apply_preconditioner(ibm.FIELD_P, r)
            zb = plain.apply_preconditioner(ibm.FIELD_P, r)
            assert np.all(np.isfinite(za))
            assert bits_equal(za, zb)
        pa, pb = fused.profile(), plain.profile()
        names = ibm.kernel_names()
        k = names.index("mg_coarse")
        assert pa.launches[k] > 0 and pb.launches[k] == 0
        default = ibm.solver_params()
        assert default.mg_fused_coarse == 0
    finally:
        fused.close()
        plain.close()


@pytest.mark.parametrize("shape,steps", [((160, 32, 32), 4), ((640, 128, 128), 2)])
def test_fused_graph_steps_bitwise(ibm, shape, steps):
    """The benchmark's step (precision 2, graph-captured, conditional Krylov
    loops around the cooperative kernel node) fused and unfused."""
    case = ibm.Case(ibm.channel_params(*shape, Um=2.25, dt=2e-4))
    a = ibm.Solver(case, bench_like(ibm, precision=2, use_graph=1, vel_inner_sweeps=2, mg_fused_coarse=1 << 30))
    b = ibm.Solver(case, bench_like(ibm, precision=2, use_graph=1, vel_inner_sweeps=2, mg_fused_coarse=0))
    try:
        for _ in range(steps):
            sa, sb = a.step(1.0), b.step(1.0)
            assert sa.status == sb.status == ibm.IBM_OK
            assert sa.p.iters == sb.p.iters
        for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
            assert bits_equal(x, y), name
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("shape", [(48, 16, 16), (96, 32, 16), (200, 40, 24), (640, 128, 128)])
def test_fused_sweep_vcycle_bitwise(ibm, shape):
    """48 and 200 points a line leave a partial tile in x, 40 and 24 lines
    partial tiles in y and z."""
    case = ibm.Case(ibm.channel_params(*shape, Um=2.25, dt=2e-4))
    fused = ibm.Solver(case, bench_like(ibm, precision=1, mg_fused_sweep=1))
    plain = ibm.Solver(case, bench_like(ibm, precision=1, mg_fused_sweep=0))
    try:
        rng = np.random.default_rng(8)
        n = shape[0] * shape[1] * shape[2]
        for _ in range(3):
            r = rng.standard_normal(n)
            za = fused.apply_preconditioner(ibm.FIELD_P, r)
            zb = plain.apply_preconditioner(ibm.FIELD_P, r)
            assert np.all(np.isfinite(za))
            assert bits_equal(za, zb)
    finally:
        fused.close()
        plain.close()


@pytest.mark.parametrize("shape,steps", [((160, 32, 32), 4), ((640, 128, 128), 2)])
def test_fused_sweep_graph_steps_bitwise(ibm, shape, steps):
    case = ibm.Case(ibm.channel_params(*shape, Um=2.25, dt=2e-4))
    a = ibm.Solver(case, bench_like(ibm, precision=2, use_graph=1, vel_inner_sweeps=2, mg_fused_sweep=1))
    b = ibm.Solver(case, bench_like(ibm, precision=2, use_graph=1, vel_inner_sweeps=2, mg_fused_sweep=0))
    try:
        for _ in range(steps):
            sa, sb = a.step(1.0), b.step(1.0)
            assert sa.status == sb.status == ibm.IBM_OK
            assert sa.p.iters == sb.p.iters
        for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
            assert bits_equal(x, y), name
    finally:
        a.close()
        b.close()

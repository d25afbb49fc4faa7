"""Record classes (row_classes = 1, the default) against the plain layout.

Kernels that read a 2-byte class per row and the row from the table of
distinct rows compute with the same values in the same order as the kernels
that read the rows themselves, so every result must be bitwise equal. The
algorithmic bytes the library books for the class-reading kernels show that
the classes were in use.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


@pytest.fixture(scope="module")
def case48(ibm):
    return ibm.Case(ibm.channel_params(48, 16, 16, Um=1.0, dt=1e-3))


def bench_like(ibm, **kw):
    base = dict(vel_tol=1e-10, p_tol=1e-10, p_pc_rap_type=0, p_pc_relax_type=2, mg_nu1=3, mg_nu2=3,
                mg_nu_coarse=2, mg_omega=1.0, mg_group_ratio=1.5, mg_options=3)
    base.update(kw)
    return ibm.solver_params(**base)


def relax_fine_bytes_per_launch(ibm, solver, r):
    k = ibm.kernel_names().index("mg_relax_fine")
    solver.profile_reset()
    solver.apply_preconditioner(ibm.FIELD_P, r)
    prof = solver.profile()
    assert prof.launches[k] > 0
    return prof.bytes[k] / prof.launches[k]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("rap", [0, 1])
def test_vcycle_bitwise_with_classes(ibm, case48, precision, rap):
    r = np.random.default_rng(5).standard_normal(case48.shape[0] * case48.shape[1] * case48.shape[2])
    a = ibm.Solver(case48, bench_like(ibm, precision=precision, p_pc_rap_type=rap, row_classes=0))
    b = ibm.Solver(case48, bench_like(ibm, precision=precision, p_pc_rap_type=rap, row_classes=1))
    za = a.apply_preconditioner(ibm.FIELD_P, r)
    zb = b.apply_preconditioner(ibm.FIELD_P, r)
    assert bits_equal(za, zb)
    # classed records book 2 bytes per record instead of 8 values
    assert relax_fine_bytes_per_launch(ibm, b, r) < 0.6 * relax_fine_bytes_per_launch(ibm, a, r)


@pytest.mark.parametrize("classes", [0, 1])
@pytest.mark.parametrize("shape", [(48, 16, 16), (36, 10, 7)])
def test_vcycle_quads_bitwise(ibm, classes, shape):
    """Four points per thread (FP32 phases and residual of 7-point levels)
    against one point per thread, including odd line and plane counts."""
    case = ibm.Case(ibm.channel_params(*shape, Um=1.0, dt=1e-3))
    r = np.random.default_rng(8).standard_normal(shape[0] * shape[1] * shape[2])
    z = [ibm.Solver(case, bench_like(ibm, precision=1, row_classes=classes, mg_quads=q))
         .apply_preconditioner(ibm.FIELD_P, r) for q in (0, 1)]
    assert bits_equal(z[0], z[1])


@pytest.mark.parametrize("precision,graph", [(0, 0), (1, 0), (2, 0), (2, 1)])
def test_steps_bitwise_with_classes(ibm, case48, precision, graph):
    # the double-float residual (precision 2 with classes) and the double-float
    # Arnoldi product (precision 1 with classes) are checked on their own below
    kw = dict(precision=precision, use_graph=graph, df_residual=0, df_spmv=0)
    a = ibm.Solver(case48, bench_like(ibm, row_classes=0, **kw))
    b = ibm.Solver(case48, bench_like(ibm, row_classes=1, **kw))
    for step in range(1, 6):
        ramp = min(1.0, step / 3.0)
        sa = a.step(ramp)
        sb = b.step(ramp)
        assert sa.status == sb.status == ibm.IBM_OK
        for f in "uvwp":
            assert getattr(sa, f).iters == getattr(sb, f).iters, f
    for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
        assert bits_equal(x, y), name
    if graph == 0:
        # the true residuals read 2-byte classes instead of 7 FP64 coefficients
        k = ibm.kernel_names().index("gmres_residual")
        per = []
        for s in (a, b):
            s.profile_reset()
            s.step(1.0)
            prof = s.profile()
            per.append(prof.bytes[k] / max(prof.launches[k], 1))
        assert per[1] < 0.5 * per[0]


@pytest.mark.parametrize("graph", [0, 1])
def test_double_float_residual(ibm, case48, graph):
    """FP32 cycles whose restarts compute the true residual in double-float
    (about 48 bits on the FP32 pipe) against the FP64 residual: same
    iteration counts within one, fields within the solve tolerance, and a
    tight pressure solve still reaches 1e-12."""
    kw = dict(precision=2, use_graph=graph)
    a = ibm.Solver(case48, bench_like(ibm, df_residual=0, **kw))
    b = ibm.Solver(case48, bench_like(ibm, df_residual=1, **kw))
    for step in range(1, 6):
        ramp = min(1.0, step / 3.0)
        sa = a.step(ramp)
        sb = b.step(ramp)
        assert sa.status == sb.status == ibm.IBM_OK
        for f in "uvwp":
            assert abs(getattr(sa, f).iters - getattr(sb, f).iters) <= 1, f
    for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
        assert np.abs(x - y).max() <= 1e-7 * max(np.abs(x).max(), 1e-30), name
    s = ibm.Solver(case48, bench_like(ibm, precision=2, df_residual=1, p_tol=1e-12, p_maxit=400))
    rng = np.random.default_rng(4)
    nx, ny, nz = case48.shape
    rhs = rng.standard_normal(nx * ny * nz) * case48.array("fluid_p")
    rhs -= rhs.mean() * case48.array("fluid_p")
    x, st = s.solve(ibm.FIELD_P, rhs)
    assert st.status == ibm.IBM_OK
    r = rhs - s.apply_operator(ibm.FIELD_P, x)
    assert np.linalg.norm(r) <= 2e-12 * np.linalg.norm(rhs)


@pytest.mark.parametrize("graph", [0, 1])
def test_double_float_arnoldi_product(ibm, case48, graph):
    """FP64 flexible GMRES whose Arnoldi product A z_j (z_j the FP32
    flexible basis) is formed in double-float on the FP32 pipe, against the
    FP64 product: same iteration counts within one, fields within the solve
    tolerance, and tight momentum and pressure solves still reach 1e-12 in
    the FP64 true residual."""
    kw = dict(precision=1, use_graph=graph)
    a = ibm.Solver(case48, bench_like(ibm, df_spmv=0, **kw))
    b = ibm.Solver(case48, bench_like(ibm, df_spmv=1, **kw))
    for step in range(1, 6):
        ramp = min(1.0, step / 3.0)
        sa = a.step(ramp)
        sb = b.step(ramp)
        assert sa.status == sb.status == ibm.IBM_OK
        for f in "uvwp":
            assert abs(getattr(sa, f).iters - getattr(sb, f).iters) <= 1, f
    for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
        assert np.abs(x - y).max() <= 1e-7 * max(np.abs(x).max(), 1e-30), name
    s = ibm.Solver(case48, bench_like(ibm, precision=1, df_spmv=1, vel_tol=1e-12, p_tol=1e-12,
                                      vel_maxit=400, p_maxit=400))
    rng = np.random.default_rng(6)
    nx, ny, nz = case48.shape
    fluid = case48.array("fluid_p").astype(np.float64)
    for field in (ibm.FIELD_U, ibm.FIELD_P):
        if field == ibm.FIELD_U:  # the u box; rows outside the fluid are identity rows
            rhs = rng.standard_normal((nx - 1) * ny * nz)
        else:
            rhs = rng.standard_normal(nx * ny * nz) * fluid
            rhs -= rhs.mean() * fluid
        x, st = s.solve(field, rhs)
        assert st.status == ibm.IBM_OK, field
        r = rhs - s.apply_operator(field, x)
        assert np.linalg.norm(r) <= 2e-12 * np.linalg.norm(rhs), field


@pytest.mark.parametrize("graph", [0, 1])
def test_steps_bitwise_quads(ibm, case48, graph):
    """Steps with the quartet kernels (including the finest level's first and
    last phases with the V-cycle's input load and output store fused in)
    against one point per thread and separate load / store kernels."""
    a = ibm.Solver(case48, bench_like(ibm, precision=2, use_graph=graph, mg_quads=0))
    b = ibm.Solver(case48, bench_like(ibm, precision=2, use_graph=graph, mg_quads=1))
    for step in range(1, 5):
        sa = a.step(min(1.0, step / 3.0))
        sb = b.step(min(1.0, step / 3.0))
        for f in "uvwp":
            assert getattr(sa, f).iters == getattr(sb, f).iters, f
    for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
        assert bits_equal(x, y), name

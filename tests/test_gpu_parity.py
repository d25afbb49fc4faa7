"""CUDA path against the CPU oracle, through the C ABI.

Dense per-step kernels (operator apply, BC + convection + gradient + momentum
right-hand side, scatter + divergence + pressure right-hand side, projection)
are compared bit for bit: the device kernels and the oracle spell out the same
floating-point operations. Solves are compared at tight tolerance (1e-13)
where the discrete solution is unique to round-off; fields must agree to
1e-10 relative (the tolerance the hot path is held to).
"""
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden")
REL_TOL = 1e-10


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def rel_err(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def tight(ibm, **kw):
    base = dict(vel_tol=1e-13, p_tol=1e-13, vel_maxit=500, p_maxit=500, mg_coarse_max=64)
    base.update(kw)
    return ibm.solver_params(**base)


@pytest.fixture(scope="module")
def case32(ibm):
    return ibm.Case(ibm.channel_params(32, 12, 12, Um=0.45, dt=1e-3))


@pytest.fixture(scope="module")
def case48(ibm):
    return ibm.Case(ibm.channel_params(48, 16, 16, Um=1.0, dt=1e-3))


def random_state(case, seed):
    nx, ny, nz = case.shape
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((nx + 1) * ny * nz), 0.3 * rng.standard_normal(nx * (ny + 1) * nz),
            0.3 * rng.standard_normal(nx * ny * (nz + 1)), rng.standard_normal(nx * ny * nz) * case.array("fluid_p"))


def test_operator_apply_bitwise(ibm, pyoracle, case48):
    s = ibm.Solver(case48, tight(ibm))
    orc = pyoracle.Oracle(case48)
    rng = np.random.default_rng(1)
    for f, n in enumerate(orc.box_sizes()):
        x = rng.standard_normal(n)
        assert bits_equal(s.apply_operator(f, x), orc.apply_operator(f, x)), f
    assert s.launches() > 0


@pytest.mark.parametrize("shape", [(32, 12, 12), (48, 16, 16), (40, 24, 8)])
def test_dense_step_kernels_bitwise(ibm, pyoracle, shape):
    """One step from a seeded random state: each dense stage of the device
    step equals the oracle's stage applied to the device's own solve outputs."""
    case = ibm.Case(ibm.channel_params(*shape, Um=0.8, dt=1e-3))
    s = ibm.Solver(case, tight(ibm))
    orc = pyoracle.Oracle(case, vel_tol=1e-13, p_tol=1e-13)
    u, v, w, p = random_state(case, sum(shape))
    s.set_fields(u, v, w, p)
    ramp = 0.6
    st = s.step(ramp)
    assert st.status in (ibm.IBM_OK, ibm.IBM_NOT_CONVERGED)
    ub, vb, wb = orc.bc_cleanup(u, v, w, ramp)
    bu, bv, bw = orc.momentum_rhs(ub, vb, wb, p)
    for f, ref in enumerate((bu, bv, bw)):
        assert bits_equal(s.solver_vector(f, 0), ref), f"momentum rhs {f}"
    xu, xv, xw = (s.solver_vector(f, 1) for f in range(3))
    orc.set_fields(ub, vb, wb, p)
    ut, vt, wt = orc.tilde(xu, xv, xw, ramp)
    assert bits_equal(s.solver_vector(3, 0), orc.pressure_rhs(ut, vt, wt, ramp)), "pressure rhs"
    xp = s.solver_vector(3, 1)
    ost = orc.projection(ut, vt, wt, xp, ramp)
    for a, b, name in zip(s.fields(), orc.fields(), "uvwp"):
        assert bits_equal(a, b), f"projected {name}"
    assert abs(st.umax - ost.umax) == 0 and abs(st.vmax - ost.vmax) == 0 and abs(st.wmax - ost.wmax) == 0
    assert abs(st.div_l2 - ost.div_l2) <= 1e-12 * max(ost.div_l2, 1e-300) + 1e-300


def test_solves_match_oracle(ibm, pyoracle, case48):
    s = ibm.Solver(case48, tight(ibm))
    orc = pyoracle.Oracle(case48, vel_tol=1e-13, p_tol=1e-13)
    rng = np.random.default_rng(5)
    for f, n in enumerate(orc.box_sizes()):
        b = rng.standard_normal(n)
        xg, stg = s.solve(f, b)
        xo, sto = orc.solve(f, b)
        assert stg.status == ibm.IBM_OK and stg.rel_res <= 1e-13
        r = b - orc.apply_operator(f, xg)
        assert np.linalg.norm(r) / np.linalg.norm(b) <= 2e-13
        assert rel_err(xg, xo) <= REL_TOL, f
        assert abs(stg.iters - sto.iters) <= 2


@pytest.mark.parametrize("rap,relax", [(1, 1), (0, 1), (1, 2)])
def test_multistep_parity(ibm, pyoracle, case48, rap, relax):
    s = ibm.Solver(case48, tight(ibm, p_pc_rap_type=rap, p_pc_relax_type=relax))
    orc = pyoracle.Oracle(case48, vel_tol=1e-13, p_tol=1e-13, mg_rap=rap, mg_relax=relax)
    for step in range(1, 11):
        ramp = min(1.0, step / 5.0)
        st = s.step(ramp)
        so = orc.step(ramp)
        assert st.status == ibm.IBM_OK and so.status == 0
        assert st.div_l2 < 1e-9
    for a, b, name in zip(s.fields(), orc.fields(), "uvwp"):
        assert rel_err(a, b) <= REL_TOL, name


@pytest.mark.parametrize("rap,relax,group,options,nu", [(1, 1, 0.0, 3, (1, 0)), (0, 1, 0.0, 3, (1, 0)),
                                                        (1, 2, 0.0, 3, (1, 0)), (0, 2, 1.5, 3, (1, 0)),
                                                        (1, 2, 1.5, 3, (1, 0)), (1, 2, 1.5, 0, (1, 0)),
                                                        (0, 2, 1.5, 1, (1, 0)), (1, 1, 0.0, 2, (1, 0)),
                                                        (0, 2, 1.5, 3, (3, 2)), (0, 2, 0.0, 3, (2, 1))])
def test_multigrid_vcycle_matches_oracle(ibm, pyoracle, case48, rap, relax, group, options, nu):
    """One V-cycle of the device multigrid equals the oracle's (same levels,
    coarse operators, smoothers, relaxed and unrelaxed levels); FP64 to
    round-off, the FP32 hierarchy to single precision."""
    omega = 1.0 if relax == 2 else 2.0 / 3.0
    kw = dict(p_pc_rap_type=rap, p_pc_relax_type=relax, mg_group_ratio=group, mg_omega=omega, mg_options=options,
              mg_nu1=nu[0], mg_nu2=nu[0], mg_nu_coarse=nu[1])
    orc = pyoracle.Oracle(case48, mg_rap=rap, mg_relax=relax, mg_group_ratio=group, mg_omega=omega,
                          mg_options=options, mg_nu1=nu[0], mg_nu2=nu[0], mg_nu_coarse=nu[1])
    r = np.random.default_rng(11).standard_normal(orc.box_sizes()[3])
    zo = orc.mg_vcycle(r)
    s64 = ibm.Solver(case48, ibm.solver_params(**kw))
    assert rel_err(s64.apply_preconditioner(ibm.FIELD_P, r), zo) <= 1e-10
    s32 = ibm.Solver(case48, ibm.solver_params(precision=1, **kw))
    assert rel_err(s32.apply_preconditioner(ibm.FIELD_P, r), zo) <= 1e-4


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_graph_step_matches_stream_step(ibm, case48, precision):
    """The captured step (one graph launch, GMRES loops on the device) gives
    the same fields and iteration counts as the host-driven step."""
    kw = dict(vel_tol=1e-10, p_tol=1e-10, precision=precision, p_pc_relax_type=2, mg_omega=1.0,
              mg_group_ratio=1.5)
    a = ibm.Solver(case48, ibm.solver_params(use_graph=0, **kw))
    b = ibm.Solver(case48, ibm.solver_params(use_graph=1, **kw))
    for step in range(1, 6):
        sa = a.step(min(1.0, step / 3.0))
        l0 = b.launches()
        sb = b.step(min(1.0, step / 3.0))
        assert b.launches() > l0
        assert sb.status == sa.status == ibm.IBM_OK
        for f in "uvwp":
            assert getattr(sa, f).iters == getattr(sb, f).iters, f
    for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
        assert bits_equal(x, y), name


def test_golden_oracle_steps(ibm, case32):
    g = np.load(os.path.join(GOLDEN, "oracle_channel_32x12x12.npz"))
    s = ibm.Solver(case32, tight(ibm))
    s.run(int(g["nsteps"]), ramp_steps=int(g["ramp_steps"]))
    for a, name in zip(s.fields(), "uvwp"):
        assert rel_err(a, g[name]) <= REL_TOL, name


def test_benchmark_channel_160x32x32(ibm, pyoracle):
    """The 160x32x32 channel (Um 0.45, nu 1e-3, dt 1e-3) for 3 steps at tight
    tolerance against the oracle."""
    case = ibm.Case(ibm.channel_params(160, 32, 32, Um=0.45, nu=1e-3, dt=1e-3))
    s = ibm.Solver(case, tight(ibm))
    orc = pyoracle.Oracle(case, vel_tol=1e-13, p_tol=1e-13)
    for step in range(1, 4):
        s.step(min(1.0, step / 2.0))
        orc.step(min(1.0, step / 2.0))
    for a, b, name in zip(s.fields(), orc.fields(), "uvwp"):
        assert rel_err(a, b) <= REL_TOL, name


@pytest.mark.parametrize("graph", [0, 1])
def test_nonzero_initial_guess_matches_oracle(ibm, pyoracle, case48, graph):
    """use_zero_initial_guess 0: the momentum solves start from the current
    velocities (main.cu's x0, immersed_operators.hpp:500-530), the pressure
    solve still from zero as the reference's pressure right-hand side kernel
    sets it; fields match the oracle to the hot path's 1e-10."""
    s = ibm.Solver(case48, tight(ibm, use_zero_initial_guess=0, use_graph=graph))
    orc = pyoracle.Oracle(case48, vel_tol=1e-13, p_tol=1e-13, use_zero_initial_guess=0)
    for step in range(1, 4):
        st = s.step(min(1.0, step / 2.0))
        orc.step(min(1.0, step / 2.0))
        assert st.status == ibm.IBM_OK
    for a, b, name in zip(s.fields(), orc.fields(), "uvwp"):
        assert rel_err(a, b) <= REL_TOL, name


@pytest.mark.parametrize("precision", [1, 2])
def test_mixed_precision_error(ibm, pyoracle, case48, precision):
    """FP32 preconditioners inside FP64 flexible GMRES (precision 1), and FP32
    Arnoldi cycles with FP64 restarts (precision 2), at 1e-8: velocity within
    1e-6 of the FP64 oracle."""
    s = ibm.Solver(case48, ibm.solver_params(vel_tol=1e-8, p_tol=1e-8, precision=precision))
    orc = pyoracle.Oracle(case48, vel_tol=1e-13, p_tol=1e-13)
    for step in range(1, 11):
        st = s.step(min(1.0, step / 5.0))
        orc.step(min(1.0, step / 5.0))
        assert st.status == ibm.IBM_OK
        assert st.p.rel_res <= 1e-8 and st.u.rel_res <= 1e-8  # true FP64 residuals
    gu, gv, gw, gp = s.fields()
    ou, ov, ow, op = orc.fields()
    vel_err = max(np.abs(gu - ou).max(), np.abs(gv - ov).max(), np.abs(gw - ow).max()) / np.abs(ou).max()
    assert vel_err <= 1e-6


@pytest.mark.parametrize("vel_precision", [1, 2])
def test_double_float_momentum_rhs(ibm, pyoracle, case48, vel_precision):
    """With mixed-precision momentum solves the momentum right-hand side is
    evaluated in double-float (df_rhs 1, the default): against the oracle's
    FP64 right-hand side from the same seeded random state it is within
    2^-40 of the largest entry and not bitwise equal (the double-float kernel
    ran); df_rhs 0 keeps the FP64 kernel, bitwise the oracle's."""
    orc = pyoracle.Oracle(case48, vel_tol=1e-13, p_tol=1e-13)
    u, v, w, p = random_state(case48, 77)
    ramp = 0.6
    ub, vb, wb = orc.bc_cleanup(u, v, w, ramp)
    ref = orc.momentum_rhs(ub, vb, wb, p)
    for df in (1, 0):
        s = ibm.Solver(case48, ibm.solver_params(precision=1, vel_precision=vel_precision, df_rhs=df))
        s.set_fields(u, v, w, p)
        s.step(ramp)
        for f in range(3):
            got = s.solver_vector(f, 0)
            if df:
                assert np.abs(got - ref[f]).max() <= 2.0 ** -40 * np.abs(ref[f]).max(), f
                assert not bits_equal(got, ref[f]), f
            else:
                assert bits_equal(got, ref[f]), f
        s.close()


@pytest.mark.parametrize("graph", [0, 1])
def test_single_pass_gram_schmidt(ibm, pyoracle, case48, graph):
    """FP64 flexible GMRES with one classical Gram-Schmidt pass per Arnoldi
    step (arnoldi_passes 1) against two passes: iteration counts within one
    and fields within 1e-7 over five steps; at 1e-12 every solve still
    converges (true FP64 residuals) and the fields agree with the FP64
    oracle to 1e-9."""
    kw = dict(vel_tol=1e-8, p_tol=1e-8, precision=1, use_graph=graph)
    a = ibm.Solver(case48, ibm.solver_params(arnoldi_passes=2, **kw))
    b = ibm.Solver(case48, ibm.solver_params(arnoldi_passes=1, **kw))
    for step in range(1, 6):
        ramp = min(1.0, step / 3.0)
        sa, sb = a.step(ramp), b.step(ramp)
        assert sa.status == sb.status == ibm.IBM_OK
        for f in "uvwp":
            assert abs(getattr(sa, f).iters - getattr(sb, f).iters) <= 1, f
    for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
        assert rel_err(y, x) <= 1e-7, name
    s = ibm.Solver(case48, ibm.solver_params(vel_tol=1e-12, p_tol=1e-12, precision=1, arnoldi_passes=1,
                                             vel_maxit=500, p_maxit=500, use_graph=graph))
    orc = pyoracle.Oracle(case48, vel_tol=1e-13, p_tol=1e-13)
    for step in range(1, 4):
        st = s.step(min(1.0, step / 2.0))
        orc.step(min(1.0, step / 2.0))
        assert st.status == ibm.IBM_OK
        for f in "uvwp":
            assert getattr(st, f).rel_res <= 1e-12, f
    for x, y, name in zip(s.fields(), orc.fields(), "uvwp"):
        assert rel_err(x, y) <= 1e-9, name


def test_fp32_cycles_reach_tight_tolerance(ibm, pyoracle, case48):
    """precision 2 restarts its FP32 cycles from FP64 true residuals, so it
    reaches tolerances far below FP32 resolution: 1e-12 on every solve."""
    s = ibm.Solver(case48, ibm.solver_params(vel_tol=1e-12, p_tol=1e-12, precision=2, vel_maxit=500,
                                             p_maxit=500))
    orc = pyoracle.Oracle(case48, vel_tol=1e-13, p_tol=1e-13)
    for step in range(1, 4):
        st = s.step(min(1.0, step / 2.0))
        orc.step(min(1.0, step / 2.0))
        assert st.status == ibm.IBM_OK
        for f in "uvwp":
            assert getattr(st, f).rel_res <= 1e-12, f
    for a, b, name in zip(s.fields(), orc.fields(), "uvwp"):
        assert rel_err(a, b) <= 1e-9, name


@pytest.mark.parametrize("model", [1, 2], ids=["staircase", "cut-surface"])
def test_forces_match_oracle(ibm, pyoracle, case48, model):
    """Body force of the device step equals the oracle's on the same fields
    (1: staircase pressure and wall shear; 2: cut-surface force from the
    operators' wall distances and the faces' open fractions); off by
    default."""
    s = ibm.Solver(case48, tight(ibm, compute_forces=model))
    orc = pyoracle.Oracle(case48, vel_tol=1e-13, p_tol=1e-13, cut_force=model == 2)
    for step in range(1, 5):
        st = s.step(min(1.0, step / 2.0))
        so = orc.step(min(1.0, step / 2.0))
    fo = np.array(so.force)
    fg = np.array(st.force)
    assert np.abs(fg - fo).max() <= 1e-9 * np.abs(fo).max()
    assert fo[0] > 0  # the flow drags the cylinder downstream
    s.set_params(tight(ibm, compute_forces=0))
    assert tuple(s.step(1.0).force) == (0.0, 0.0, 0.0)


def test_not_converged_is_a_warning(ibm, case32):
    s = ibm.Solver(case32, ibm.solver_params(vel_tol=1e-14, p_tol=1e-14, vel_maxit=1, p_maxit=1))
    st = s.step(1.0)
    assert st.status == ibm.IBM_NOT_CONVERGED
    assert st.p.iters == 1 and st.p.status == ibm.IBM_NOT_CONVERGED


def test_nonfinite_detected(ibm, case32):
    s = ibm.Solver(case32)
    u, v, w, p = case32.initial_fields()
    nx, ny, nz = case32.shape
    u = u.copy()
    u[(5 * ny + 6) * (nx + 1) + 10] = np.nan
    s.set_fields(u, v, w, p)
    with pytest.raises(ibm.IBMError) as e:
        s.step(1.0)
    assert e.value.code == -3


def test_zero_rhs_returns_immediately(ibm, case32):
    s = ibm.Solver(case32)
    x, st = s.solve(ibm.FIELD_V, np.zeros((32) * 11 * 12))
    assert st.iters == 0 and st.status == ibm.IBM_OK and not np.any(x)


def test_unsupported_csr_rejected(ibm, case32):
    import ctypes as C
    s = ibm.Solver(case32)
    a = case32.array
    col = a("D_col").copy()
    col[0] = col[0] + 7  # no longer a face of its cell
    cnt = case32.counts
    rc = s._lib.ibm_set_projection_csr(s._ctx, C.c_void_p(a("D_rowptr").ctypes.data), C.c_void_p(col.ctypes.data),
                                       C.c_void_p(a("D_val").ctypes.data), cnt["np"],
                                       C.c_void_p(a("G_rowptr").ctypes.data), C.c_void_p(a("G_col").ctypes.data),
                                       C.c_void_p(a("G_val").ctypes.data), cnt["nqu"] + cnt["nqv"] + cnt["nqw"])
    assert rc == -6

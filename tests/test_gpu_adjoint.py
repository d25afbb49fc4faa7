"""Adjoint extension on the GPU (ibm_adjoint_setup, ibm_step_forward /
ibm_step_backward, checkpoints) against the CPU oracle's reverse sweep and
against central finite differences of the GPU's own forward steps.

The reverse sweep sums the convection transpose with FP64 atomics, so the
GPU and oracle lambdas agree to rounding and solver tolerance, not bitwise.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (48, 16, 16)
ORACLE_KW = dict(vel_tol=1e-13, p_tol=1e-13, p_pc=1, mg_rap=0, mg_relax=2, mg_group_ratio=1.5)


@pytest.fixture(scope="module")
def inflow():
    return importlib.import_module("ibm-3d-fpc_gb300.inflow")


def case_nu(ibm, nu=1e-3):
    return ibm.Case(ibm.channel_params(*SHAPE, Um=1.0, dt=2e-3, nu=nu))


def fp64_params(ibm, **kw):
    base = dict(vel_tol=1e-13, p_tol=1e-13, vel_maxit=500, p_maxit=500, precision=0, use_graph=0,
                p_pc_rap_type=0, p_pc_relax_type=2, mg_group_ratio=1.5, compute_forces=1)
    base.update(kw)
    return ibm.solver_params(**base)


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("graph,model", [(0, 1), (1, 1), (0, 2), (1, 2)],
                         ids=["host-staircase", "graph-staircase", "host-cut", "graph-cut"])
def test_backward_step_matches_oracle(ibm, pyoracle, graph, model):
    """One reverse step, host-driven or as the captured graph (transposed
    solves with their loops on the device), with the staircase (1) or the
    cut-surface (2) drag as the objective's force."""
    case = case_nu(ibm)
    o = pyoracle.Oracle(case, cut_force=model == 2, **ORACLE_KW)
    ot = pyoracle.Oracle(pyoracle.TransposedCase(case), **ORACLE_KW)
    o.step(1.0)
    s0 = o.fields()
    s = ibm.Solver(case, fp64_params(ibm, use_graph=graph, compute_forces=model))
    s.adjoint_setup()
    s.set_fields(*s0)
    rng = np.random.default_rng(11)
    lam1 = [rng.standard_normal(x.size) for x in s0]
    s.step_forward(1.0)
    assert s.tape_depth() == 1
    s.adjoint_set(*lam1)
    st = s.step_backward(1.0, weight=0.3)
    assert st.status == ibm.IBM_OK
    assert s.tape_depth() == 0
    lu, lv, lw, lp, dg, dnu = s.adjoint_get()
    lam = [x.copy() for x in lam1]
    dg_o = np.zeros(SHAPE[1] * SHAPE[2])
    o.set_fields(*s0)
    dnu_o = o.step_backward(ot, 1.0, case.array("beta_p"), 0.3, lam, dg_o)
    for x, y, name in zip((lu, lv, lw, lp), lam, "uvwp"):
        assert rel_err(x, y) <= 1e-8, name
    assert rel_err(dg, dg_o) <= 1e-8
    assert abs(dnu - dnu_o) <= 1e-8 * abs(dnu_o)
    # the context holds the recomputed step's end-of-step fields
    o.set_fields(*s0)
    o.step(1.0)
    for x, y, name in zip(s.fields(), o.fields(), "uvwp"):
        assert rel_err(x, y) <= 1e-9, name
    # a second reverse step reuses the captured graph with another weight
    s.set_fields(*s0)
    s.adjoint_reset()
    s.step_forward(1.0)
    s.adjoint_set(*lam1)
    s.step_backward(1.0, weight=0.0)
    lam = [x.copy() for x in lam1]
    dg_o = np.zeros(SHAPE[1] * SHAPE[2])
    o.set_fields(*s0)
    o.step_backward(ot, 1.0, case.array("beta_p"), 0.0, lam, dg_o)
    lu, lv, lw, lp, dg, _ = s.adjoint_get()
    for x, y, name in zip((lu, lv, lw, lp), lam, "uvwp"):
        assert rel_err(x, y) <= 1e-8, name
    assert rel_err(dg, dg_o) <= 1e-8


def test_set_inflow_is_the_setup(ibm, inflow):
    case = case_nu(ibm)
    g = inflow.inflow_from_coefficients(case, np.random.default_rng(2).uniform(-0.05, 0.05, 64))
    a = ibm.Solver(case, fp64_params(ibm, vel_tol=1e-10, p_tol=1e-10))
    a.adjoint_setup()
    a.set_inflow(g)
    a.set_fields(*inflow.InflowCase(case, g).initial_fields())
    b = ibm.Solver(inflow.InflowCase(case, g), fp64_params(ibm, vel_tol=1e-10, p_tol=1e-10))
    for step in range(1, 4):
        a.step(min(1.0, step / 2))
        b.step(min(1.0, step / 2))
    for x, y, name in zip(a.fields(), b.fields(), "uvwp"):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), name


def test_drag_gradient_matches_oracle_with_checkpoints(ibm, pyoracle, inflow):
    case = case_nu(ibm)
    g = inflow.inflow_from_coefficients(case, np.random.default_rng(3).uniform(-0.05, 0.05, 64))
    icase = inflow.InflowCase(case, g)
    ramps = [0.5, 1.0, 1.0, 1.0, 1.0]
    window = {2, 3, 4, 5}
    J_o, dg_o, dnu_o, _ = pyoracle.drag_gradient(icase, ramps, window, **ORACLE_KW)
    s = ibm.Solver(icase, fp64_params(ibm))
    s.adjoint_setup()
    J, dg, dnu = s.drag_gradient(ramps, window, checkpoint_every=2)
    assert abs(J - J_o) <= 1e-8 * abs(J_o)
    assert rel_err(dg, dg_o) <= 1e-7
    assert abs(dnu - dnu_o) <= 1e-7 * abs(dnu_o)


def gpu_objective(ibm, case, g, ramps, window, params):
    s = ibm.Solver(case, params)
    s.adjoint_setup()
    s.set_inflow(g)
    J = 0.0
    for k, ramp in enumerate(ramps, start=1):
        st = s.step(ramp)
        if k in window:
            J += st.force[0] / len(window)
    return J


@pytest.mark.parametrize("model", [1, 2], ids=["staircase", "cut-surface"])
def test_gpu_gradient_matches_finite_differences(ibm, inflow, model):
    base = case_nu(ibm)
    rng = np.random.default_rng(5)
    g0 = inflow.inflow_from_coefficients(base, rng.uniform(-0.05, 0.05, 64))
    ramps = [0.5, 1.0, 1.0, 1.0]
    window = {2, 3, 4}
    prm = fp64_params(ibm, compute_forces=model)
    s = ibm.Solver(base, prm)
    s.adjoint_setup()
    s.set_inflow(g0)
    s.set_fields(*inflow.InflowCase(base, g0).initial_fields())
    J, dg, dnu = s.drag_gradient(ramps, window, checkpoint_every=3)
    B = inflow.legendre_basis(base)
    d = rng.standard_normal(64)
    h = 1e-6
    jp = gpu_objective(ibm, inflow.InflowCase(base, g0 + B @ (h * d)), g0 + B @ (h * d), ramps, window, prm)
    jm = gpu_objective(ibm, inflow.InflowCase(base, g0 - B @ (h * d)), g0 - B @ (h * d), ramps, window, prm)
    fd = (jp - jm) / (2 * h)
    assert abs((B.T @ dg) @ d - fd) <= 1e-5 * abs(fd)
    jp = gpu_objective(ibm, inflow.InflowCase(case_nu(ibm, 1e-3 + h), g0), g0, ramps, window, prm)
    jm = gpu_objective(ibm, inflow.InflowCase(case_nu(ibm, 1e-3 - h), g0), g0, ramps, window, prm)
    fd = (jp - jm) / (2 * h)
    assert abs(dnu - fd) <= 1e-5 * abs(fd)


def test_mixed_precision_graph_adjoint(ibm, inflow):
    """The graph-captured FP32-cycle step (the benchmark's form) in the
    forward and recomputed steps, FP32-cycle transposed solves: the gradient
    agrees with the FP64 one to the solves' tolerance."""
    case = case_nu(ibm)
    g = inflow.inflow_from_coefficients(case, np.random.default_rng(6).uniform(-0.05, 0.05, 64))
    ramps = [0.5, 1.0, 1.0]
    window = {2, 3}
    out = []
    for prm in (fp64_params(ibm), fp64_params(ibm, precision=2, use_graph=1, vel_tol=1e-12, p_tol=1e-12)):
        s = ibm.Solver(inflow.InflowCase(case, g), prm)
        s.adjoint_setup()
        out.append(s.drag_gradient(ramps, window, checkpoint_every=2))
    (J0, dg0, dnu0), (J1, dg1, dnu1) = out
    assert abs(J1 - J0) <= 1e-8 * abs(J0)
    assert rel_err(dg1, dg0) <= 1e-6
    assert abs(dnu1 - dnu0) <= 1e-6 * abs(dnu0)


@pytest.mark.parametrize("shape,graph", [((36, 10, 7), 0), ((20, 9, 11), 1)])
def test_backward_step_odd_grids(ibm, pyoracle, shape, graph):
    """Odd line and plane counts: the boundary planes, the convection's
    fallbacks and the solve boxes' edges in the reverse kernels."""
    case = ibm.Case(ibm.channel_params(*shape, Um=1.0, dt=2e-3))
    o = pyoracle.Oracle(case, **ORACLE_KW)
    ot = pyoracle.Oracle(pyoracle.TransposedCase(case), **ORACLE_KW)
    o.step(1.0)
    s0 = o.fields()
    s = ibm.Solver(case, fp64_params(ibm, use_graph=graph))
    s.adjoint_setup()
    s.set_fields(*s0)
    rng = np.random.default_rng(12)
    lam1 = [rng.standard_normal(x.size) for x in s0]
    s.step_forward(0.7)
    s.adjoint_set(*lam1)
    s.step_backward(0.7, weight=0.2)
    lu, lv, lw, lp, dg, dnu = s.adjoint_get()
    lam = [x.copy() for x in lam1]
    dg_o = np.zeros(shape[1] * shape[2])
    o.set_fields(*s0)
    dnu_o = o.step_backward(ot, 0.7, case.array("beta_p"), 0.2, lam, dg_o)
    for x, y, name in zip((lu, lv, lw, lp), lam, "uvwp"):
        assert rel_err(x, y) <= 1e-8, name
    assert rel_err(dg, dg_o) <= 1e-8
    assert abs(dnu - dnu_o) <= 1e-8 * max(abs(dnu_o), 1e-30)

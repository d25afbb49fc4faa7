"""Adjoint extension on the CPU: the oracle's reverse sweep against central
finite differences of the oracle's own forward steps, and the inflow
parameterisation against the setup's arrays.

Objective: mean end-of-step drag F_x over steps 2..4 of four steps (ramps
0.5, 1, 1, 1) on a 48x16x16 channel; parameters: the inflow profile through
8x8 Legendre coefficients (base parabolic profile plus a perturbation drawn
as U(-0.05, 0.05) Um) and nu. Central differences with h = 1e-6; solves at a
relative residual of 1e-13 so that the solver tolerance stays far below the
difference quotient's own error.
"""
import importlib

import numpy as np
import pytest

SHAPE = (48, 16, 16)
ORACLE_KW = dict(vel_tol=1e-13, p_tol=1e-13, p_pc=1, mg_rap=0, mg_relax=2, mg_group_ratio=1.5)
RAMPS = [0.5, 1.0, 1.0, 1.0]
WINDOW = {2, 3, 4}


@pytest.fixture(scope="module")
def inflow():
    return importlib.import_module("ibm-3d-fpc_gb300.inflow")


def case_nu(ibm, nu):
    return ibm.Case(ibm.channel_params(*SHAPE, Um=1.0, dt=2e-3, nu=nu))


def test_inflow_case_reproduces_the_setup(ibm, inflow):
    case = case_nu(ibm, 1e-3)
    same = inflow.InflowCase(case, case.array("uin"))
    for name in ("uin", "div_bc_unit", "rhs_u_bc", "Ap_vals"):
        assert np.array_equal(same.array(name).view(np.uint8), case.array(name).view(np.uint8)), name
    # the inlet weights are the derivative of the divergence lift
    g = np.random.default_rng(1).standard_normal(case.shape[1] * case.shape[2])
    lift = inflow.InflowCase(case, g).array("div_bc_unit")
    nx, ny, nz = case.shape
    idp = case.array("id_p").reshape(nz, ny, nx)[:, :, 0].ravel()
    wts = inflow.inlet_weights(case)
    m = wts != 0
    assert np.allclose(lift[idp[m]], -g[m] * wts[m], rtol=1e-14, atol=0)


def test_legendre_basis(ibm, inflow):
    case = case_nu(ibm, 1e-3)
    B = inflow.legendre_basis(case)
    assert B.shape == (case.shape[1] * case.shape[2], 64)
    assert np.allclose(B[:, 0], 1.0)
    # L_1(yh) L_0(zh) is the y coordinate mapped to [-1, 1]
    ny = case.shape[1]
    yh = 2.0 * (np.arange(ny) + 0.5) / ny - 1.0
    assert np.allclose(B[:ny, 1], yh)


@pytest.mark.parametrize("cut_force", [False, True], ids=["staircase", "cut-surface"])
def test_oracle_adjoint_matches_finite_differences(ibm, pyoracle, inflow, cut_force):
    base = case_nu(ibm, 1e-3)
    rng = np.random.default_rng(3)
    c = rng.uniform(-0.05, 0.05, 64) * base.params.Um
    g0 = inflow.inflow_from_coefficients(base, c)
    kw = dict(ORACLE_KW, cut_force=cut_force)
    J, dg, dnu, _ = pyoracle.drag_gradient(inflow.InflowCase(base, g0), RAMPS, WINDOW, **kw)
    assert np.isfinite(J) and J != 0.0
    B = inflow.legendre_basis(base)
    dc = B.T @ dg
    h = 1e-6
    # a random direction in coefficient space
    d = rng.standard_normal(64)
    jp = pyoracle.drag_objective(inflow.InflowCase(base, g0 + B @ (h * d)), RAMPS, WINDOW, **kw)
    jm = pyoracle.drag_objective(inflow.InflowCase(base, g0 - B @ (h * d)), RAMPS, WINDOW, **kw)
    fd = (jp - jm) / (2 * h)
    assert abs(dc @ d - fd) <= 1e-5 * abs(fd)
    # the leading coefficient on its own
    e = np.zeros(64)
    e[0] = 1.0
    jp = pyoracle.drag_objective(inflow.InflowCase(base, g0 + B @ (h * e)), RAMPS, WINDOW, **kw)
    jm = pyoracle.drag_objective(inflow.InflowCase(base, g0 - B @ (h * e)), RAMPS, WINDOW, **kw)
    fd = (jp - jm) / (2 * h)
    assert abs(dc[0] - fd) <= 1e-5 * abs(fd)
    # nu: the operators, row scales, inlet lift and wall shear all change
    jp = pyoracle.drag_objective(inflow.InflowCase(case_nu(ibm, 1e-3 + h), g0), RAMPS, WINDOW, **kw)
    jm = pyoracle.drag_objective(inflow.InflowCase(case_nu(ibm, 1e-3 - h), g0), RAMPS, WINDOW, **kw)
    fd = (jp - jm) / (2 * h)
    assert abs(dnu - fd) <= 1e-5 * abs(fd)


def test_oracle_adjoint_is_the_transpose_of_the_step(ibm, pyoracle, inflow):
    """<lambda_0, ds_0> = <lambda_1, ds_1> for the step's tangent, with the
    tangent taken by central differences of one oracle step (exact: with
    exact solves the step is quadratic in the state)."""
    case = case_nu(ibm, 1e-3)
    o = pyoracle.Oracle(case, **ORACLE_KW)
    ot = pyoracle.Oracle(pyoracle.TransposedCase(case), **ORACLE_KW)
    o.step(1.0)
    s0 = o.fields()
    rng = np.random.default_rng(7)
    lam1 = [rng.standard_normal(x.size) for x in s0]
    lam = [x.copy() for x in lam1]
    dg = np.zeros(case.shape[1] * case.shape[2])
    o.step_backward(ot, 1.0, case.array("beta_p"), 0.0, lam, dg)
    ds = [rng.standard_normal(x.size) * 1e-3 for x in s0]
    h = 1.0  # the step is quadratic in the state: the central difference is exact

    def step_from(eps):
        o.set_fields(*[x + eps * y for x, y in zip(s0, ds)])
        o.step(1.0)
        return o.fields()

    sp, sm = step_from(h), step_from(-h)
    lhs = sum(float(l @ d) for l, d in zip(lam, ds))
    rhs = sum(float(l @ ((a - b) / (2 * h))) for l, a, b in zip(lam1, sp, sm))
    assert abs(lhs - rhs) <= 1e-9 * abs(rhs)


class _FakeSolver:
    """Records the calls of Solver.drag_gradient (no GPU): each step adds
    the ramp to a scalar state, the drag is the state itself."""

    def __init__(self, ibm):
        self.ibm = ibm
        self.params = ibm._native.SolverParams()
        self.state = 0.0
        self.tape = []
        self.ckpt = {}
        self.calls = []

    def set_params(self, p):
        self.params = p

    def adjoint_reset(self):
        self.tape.clear()
        self.calls.append("reset")

    def checkpoint_clear(self):
        self.ckpt.clear()

    def checkpoint_save(self, slot):
        self.ckpt[slot] = self.state

    def checkpoint_load(self, slot):
        self.state = self.ckpt[slot]

    def _advance(self, ramp):
        self.state += ramp
        st = self.ibm.StepStats()
        st.force[0] = self.state
        return st

    def step(self, ramp):
        self.calls.append(("step", ramp))
        return self._advance(ramp)

    def step_forward(self, ramp):
        self.calls.append(("fwd", ramp, self.state))
        self.tape.append((self.state, ramp))
        return self._advance(ramp)

    def step_backward(self, ramp, weight):
        start, r = self.tape.pop()
        assert r == ramp
        self.calls.append(("bwd", ramp, start, weight))
        return self.ibm.StepStats()

    def fields(self):
        return (self.state,)

    def set_fields(self, *f):
        self.state = f[0]

    def adjoint_get(self):
        return None, None, None, None, "dg", "dnu"


def test_drag_gradient_checkpoint_schedule(ibm):
    """The reverse sweep replays each checkpoint segment and reverses its
    steps in order, with the step's own ramp and weight 1/|window| inside
    the objective window; the fields end at the forward sweep's end."""
    fake = _FakeSolver(ibm)
    ramps = [0.1 * k for k in range(1, 8)]
    J, dg, dnu = ibm.Solver.drag_gradient(fake, ramps, window={5, 6, 7}, checkpoint_every=3)
    states = np.cumsum(ramps)
    assert J == pytest.approx(states[4:].mean())
    assert fake.state == pytest.approx(states[-1])
    bwd = [c for c in fake.calls if c[0] == "bwd"]
    assert [b[1] for b in bwd] == ramps[::-1]
    starts = np.concatenate([[0.0], states[:-1]])
    assert [b[2] for b in bwd] == pytest.approx(list(starts[::-1]))
    assert [b[3] for b in bwd] == pytest.approx([1 / 3] * 3 + [0.0] * 4)
    # segments 7, 4-6, 1-3: each replayed from its checkpoint right before its reversal
    order = [c[0] for c in fake.calls if c[0] in ("fwd", "bwd")]
    assert order == ["fwd"] + ["bwd"] + ["fwd"] * 3 + ["bwd"] * 3 + ["fwd"] * 3 + ["bwd"] * 3
    assert fake.params.compute_forces == 1


@pytest.mark.parametrize("shape", [(36, 10, 7), (20, 9, 11)])
def test_oracle_adjoint_transpose_odd_grids(ibm, pyoracle, shape):
    """The transpose identity on grids with odd line and plane counts, where
    the convection's out-of-range fallbacks and the boundary planes differ."""
    case = ibm.Case(ibm.channel_params(*shape, Um=1.0, dt=2e-3))
    o = pyoracle.Oracle(case, **ORACLE_KW)
    ot = pyoracle.Oracle(pyoracle.TransposedCase(case), **ORACLE_KW)
    o.step(1.0)
    s0 = o.fields()
    rng = np.random.default_rng(9)
    lam1 = [rng.standard_normal(x.size) for x in s0]
    lam = [x.copy() for x in lam1]
    dg = np.zeros(case.shape[1] * case.shape[2])
    o.step_backward(ot, 0.7, case.array("beta_p"), 0.0, lam, dg)
    ds = [rng.standard_normal(x.size) * 1e-3 for x in s0]
    dgdir = rng.standard_normal(dg.size) * 1e-3
    # with exact solves the step is a quadratic polynomial in the state and
    # the inflow (only the convection is nonlinear), so the central
    # difference is exact for any h: a large one keeps solver noise out
    h = 1.0
    uin = case.array("uin")

    def step_from(eps):
        # perturb the state and the inflow together: <lam1, J ds> + <dg, dg_dir>
        oc = pyoracle.Oracle(importlib.import_module("ibm-3d-fpc_gb300.inflow").InflowCase(case, uin + eps * dgdir),
                             **ORACLE_KW)
        oc.set_fields(*[x + eps * y for x, y in zip(s0, ds)])
        oc.step(0.7)
        return oc.fields()

    sp, sm = step_from(h), step_from(-h)
    lhs = sum(float(l @ d) for l, d in zip(lam, ds)) + float(dg @ dgdir)
    rhs = sum(float(l @ ((a - b) / (2 * h))) for l, a, b in zip(lam1, sp, sm))
    assert abs(lhs - rhs) <= 1e-9 * abs(rhs)


def test_cut_surface_force_of_a_closed_body(ibm, pyoracle):
    """A uniform pressure on the fluid cells and no flow give no cut-surface
    force: the fluid cells' faces (partly open where the cylinder cuts them,
    closed towards non-fluid cells) close around the body."""
    case = case_nu(ibm, 1e-3)
    o = pyoracle.Oracle(case, cut_force=True)
    u, v, w, p = o.fields()
    o.set_fields(np.zeros_like(u), np.zeros_like(v), np.zeros_like(w), 3.0 * case.array("fluid_p"))
    f = o.forces()
    assert np.abs(f).max() <= 1e-15
    # a pressure rising along x pushes the body against it: F_x < 0
    nx, ny, nz = case.shape
    ramp = np.broadcast_to(np.arange(nx, dtype=float), (nz, ny, nx)).ravel() * case.array("fluid_p")
    o.set_fields(np.zeros_like(u), np.zeros_like(v), np.zeros_like(w), ramp)
    assert o.forces()[0] < 0

"""The CPU oracle, pinned to the reference.

- BC cleanup and convection: bitwise equal to the reference's CPU twins
  (immersed_operators.hpp:990-1053), live where the reference is compiled
  here, otherwise against the committed golden fixtures.
- Solves: the reference's solver (HYPRE) is not vendored; the oracle's
  solutions are pinned by their residual against the reference-identical
  operators.
- Multigrid: the coarse operators equal R A P formed explicitly with sparse
  matrices.
"""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


@pytest.fixture(scope="module")
def case32(ibm):
    return ibm.Case(ibm.channel_params(32, 12, 12, Um=0.45, dt=1e-3))


def test_bc_and_convection_match_reference_twins_golden(case32, pyoracle):
    g = np.load(os.path.join(GOLDEN, "twins_channel_32x12x12.npz"))
    orc = pyoracle.Oracle(case32)
    ub, vb, wb = orc.bc_cleanup(g["u"], g["v"], g["w"], float(g["ramp"]))
    assert bits_equal(ub, g["u_bc"]) and bits_equal(vb, g["v_bc"]) and bits_equal(wb, g["w_bc"])
    cu, cv, cw = orc.convection(ub, vb, wb)
    assert bits_equal(cu, g["conv_u"]) and bits_equal(cv, g["conv_v"]) and bits_equal(cw, g["conv_w"])


@pytest.mark.parametrize("shape", [(48, 16, 16), (40, 24, 8), (160, 32, 32)])
def test_bc_and_convection_match_reference_twins_live(ibm, pyoracle, shape):
    if not pyoracle.reference_available():
        pytest.skip("reference checker not built")
    prm = ibm.channel_params(*shape, Um=1.3)
    case = ibm.Case(prm)
    ref = pyoracle.ReferenceCase(prm)
    orc = pyoracle.Oracle(case)
    rng = np.random.default_rng(sum(shape))
    nx, ny, nz = shape
    u = rng.standard_normal((nx + 1) * ny * nz)
    v = rng.standard_normal(nx * (ny + 1) * nz)
    w = rng.standard_normal(nx * ny * (nz + 1))
    ramp = 0.37
    r = ref.enforce_bc(u, v, w, ramp * case.array("uin"))
    o = orc.bc_cleanup(u, v, w, ramp)
    for a, b in zip(r, o):
        assert bits_equal(a, b)
    rc = ref.convection(*r)
    oc = orc.convection(*o)
    for a, b in zip(rc, oc):
        assert bits_equal(a, b)


@pytest.mark.parametrize("mg_options,tol", [(0, 1e-12), (3, 1e-10)])
def test_oracle_steps_match_golden(case32, pyoracle, mg_options, tol):
    """The fixture was made with PFMG's plain multigrid rules (mg_options 0):
    with those the oracle reproduces it to round-off; with the cut-cell-aware
    hierarchy (the default) the solves stop at other iterates of the same
    tight tolerance, which moves the fields by at most 1e-10 relative."""
    g = np.load(os.path.join(GOLDEN, "oracle_channel_32x12x12.npz"))
    orc = pyoracle.Oracle(case32, vel_tol=1e-13, p_tol=1e-13, mg_options=mg_options)
    for step in range(1, int(g["nsteps"]) + 1):
        orc.step(min(1.0, step / float(g["ramp_steps"])))
    u, v, w, p = orc.fields()
    for a, b in zip((u, v, w, p), (g["u"], g["v"], g["w"], g["p"])):
        scale = max(np.abs(b).max(), 1e-300)
        assert np.abs(a - b).max() <= tol * scale


def test_solves_satisfy_reference_equations(case32, pyoracle):
    """Each oracle solve leaves ||b - A x|| / ||b|| at the requested tolerance,
    with A the reference-identical embedded operator."""
    orc = pyoracle.Oracle(case32, vel_tol=1e-12, p_tol=1e-12)
    rng = np.random.default_rng(3)
    for field, n in enumerate(orc.box_sizes()):
        b = rng.standard_normal(n)
        x, st = orc.solve(field, b)
        assert st.status == 0
        r = b - orc.apply_operator(field, x)
        assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.01e-12
        assert st.rel_res <= 1e-12


def test_operator_apply_matches_dense_matrix(case32, pyoracle):
    """The 7-point apply equals the explicit matrix assembled from the
    row-major Struct values (HYPRE Struct stencil semantics)."""
    orc = pyoracle.Oracle(case32)
    nx, ny, nz = case32.shape
    for field, (bx, by, bz), name in ((0, (nx - 1, ny, nz), "Au_vals"), (3, (nx, ny, nz), "Ap_vals")):
        A = case32.array(name).reshape(-1, 7)
        n = bx * by * bz
        x = np.random.default_rng(field).standard_normal(n)
        X = x.reshape(bz, by, bx)
        pad = np.zeros((bz + 2, by + 2, bx + 2))
        pad[1:-1, 1:-1, 1:-1] = X
        nb = [X, pad[1:-1, 1:-1, :-2], pad[1:-1, 1:-1, 2:], pad[1:-1, :-2, 1:-1], pad[1:-1, 2:, 1:-1],
              pad[:-2, 1:-1, 1:-1], pad[2:, 1:-1, 1:-1]]
        y = sum(A[:, s] * nb[s].ravel() for s in range(7))
        assert np.allclose(orc.apply_operator(field, x), y, rtol=1e-14, atol=1e-12 * np.abs(y).max())


def _explicit_A(A27, dims):
    """Sparse matrix of a 27-point operator stored [n][27]."""
    import scipy.sparse as sp
    nx, ny, nz = dims
    n = nx * ny * nz
    rows, cols, vals = [], [], []
    idx = np.arange(n).reshape(nz, ny, nx)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    for s in range(27):
        ox, oy, oz = s % 3 - 1, (s // 3) % 3 - 1, s // 9 - 1
        ii, jj, kk = i + ox, j + oy, k + oz
        ok = (ii >= 0) & (ii < nx) & (jj >= 0) & (jj < ny) & (kk >= 0) & (kk < nz)
        r = idx[ok]
        rows.append(r); cols.append(idx[kk[ok], jj[ok], ii[ok]]); vals.append(A27[r, s])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def _explicit_P(dims, d, pm, pp):
    """Interpolation for semicoarsening along d: even points inject, odd
    points take pm / pp of their lower / upper coarse neighbours."""
    import scipy.sparse as sp
    nx, ny, nz = dims
    n = nx * ny * nz
    idx = np.arange(n).reshape(nz, ny, nx)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cdims = list(dims)
    cdims[d] = (dims[d] + 1) // 2
    cidx = np.arange(cdims[0] * cdims[1] * cdims[2]).reshape(cdims[2], cdims[1], cdims[0])
    f = [i, j, k][d]
    pr, pc, pv = [], [], []
    for sel, cf, wts in ((f % 2 == 0, f // 2, None), (f % 2 == 1, (f - 1) // 2, pm),
                         ((f % 2 == 1) & ((f + 1) // 2 < cdims[d]), (f + 1) // 2, pp)):
        c3 = [i, j, k]
        c3 = [c.copy() for c in c3]
        c3[d] = cf
        pr.append(idx[sel]); pc.append(cidx[c3[2][sel], c3[1][sel], c3[0][sel]])
        pv.append(np.ones(sel.sum()) if wts is None else wts[idx[sel]])
    return sp.csr_matrix((np.concatenate(pv), (np.concatenate(pr), np.concatenate(pc))),
                         shape=(n, cdims[0] * cdims[1] * cdims[2]))


def _coupled(A27):
    off = A27.copy()
    off[:, 13] = 0.0
    return np.any(off != 0.0, axis=1)


def _interp_weights(A27, d, dims=None, aware=False):
    """PFMG's weights; with `aware`, coupled points without coupling along d
    take the constant from their coupled coarse neighbours."""
    od = np.array([(s % 3 - 1, (s // 3) % 3 - 1, s // 9 - 1)[d] for s in range(27)])
    c0 = A27[:, od == 0].sum(axis=1)
    cm = A27[:, od < 0].sum(axis=1)
    cp = A27[:, od > 0].sum(axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        pm, pp = np.where(c0 != 0, -cm / c0, 0.0), np.where(c0 != 0, -cp / c0, 0.0)
    if aware:
        cpl = _coupled(A27)
        n = len(pm)
        stride = [1, dims[0], dims[0] * dims[1]][d]
        idx = np.arange(n)
        coord = [idx % dims[0], (idx // dims[0]) % dims[1], idx // (dims[0] * dims[1])][d]
        lo = np.zeros(n, bool)
        hi = np.zeros(n, bool)
        lo[coord > 0] = cpl[idx[coord > 0] - stride]
        hi[coord < dims[d] - 1] = cpl[idx[coord < dims[d] - 1] + stride]
        dec = cpl & (cm == 0) & (cp == 0)
        nf = lo.astype(float) + hi.astype(float)
        pm = np.where(dec, np.where(nf > 0, lo / np.maximum(nf, 1), 0.0), pm)
        pp = np.where(dec, np.where(nf > 0, hi / np.maximum(nf, 1), 0.0), pp)
    return pm, pp


@pytest.mark.parametrize("rap,options", [(0, 0), (1, 0), (0, 3), (1, 3)])
def test_multigrid_coarse_operators_are_rap(case32, pyoracle, rap, options):
    orc = pyoracle.Oracle(case32, mg_rap=rap, mg_coarse_max=16, mg_options=options)
    levels = orc.mg_levels()
    assert len(levels) >= 4
    dirs = [cd for _, cd in levels[:-1]]
    assert set(dirs) == {0, 1, 2}  # semicoarsening visits every direction
    for l in range(min(3, len(levels) - 1)):
        dims, d = levels[l]
        Af = orc.mg_level_coef(l)
        pm, pp = _interp_weights(Af, d, dims, aware=bool(options & 1))
        A, P = _explicit_A(Af, dims), _explicit_P(dims, d, pm, pp)
        Ac = (P.T @ A @ P).toarray()
        Cc = orc.mg_level_coef(l + 1)
        got = _explicit_A(Cc, levels[l + 1][0]).toarray()
        scale = np.abs(Ac).max()
        if rap == 0:
            assert np.abs(got - Ac).max() <= 1e-12 * scale
            continue
        # collapsed: same row sums
        assert np.allclose(got.sum(axis=1), Ac.sum(axis=1), atol=1e-9 * scale)
        nxc, nyc, nzc = levels[l + 1][0]
        if options & 1:
            # no collapsed coupling lands on an uncoupled point
            cpl = _coupled(_to27_from_dense(Ac, levels[l + 1][0]))
            assert not np.any((got != 0) & ~np.eye(len(got), dtype=bool) & ~cpl[None, :])
        else:
            # plain collapse: same action on linear functions
            kk, jj, ii = np.meshgrid(np.arange(nzc), np.arange(nyc), np.arange(nxc), indexing="ij")
            for lin in (ii.ravel(), jj.ravel(), kk.ravel()):
                assert np.allclose(got @ lin, Ac @ lin, atol=1e-8 * scale * max(nxc, nyc, nzc))


def _to27_from_dense(M, dims):
    nx, ny, nz = dims
    n = nx * ny * nz
    out = np.zeros((n, 27))
    r, c = np.nonzero(M)
    ri, rj, rk = r % nx, (r // nx) % ny, r // (nx * ny)
    ci, cj, ck = c % nx, (c // nx) % ny, c // (nx * ny)
    out[r, (ci - ri + 1) + 3 * (cj - rj + 1) + 9 * (ck - rk + 1)] = M[r, c]
    return out


def test_pressure_operator_is_diagonally_symmetrizable(case32):
    """The cut-cell pressure operator is W S with S symmetric and W the
    inverse open fraction of cut cells: the form the symmetrized hierarchy
    (mg_options bit 1) relies on."""
    nx, ny, nz = case32.shape
    ap = case32.array("Ap_vals").reshape(-1, 7)
    beta = case32.array("beta_p")
    fl = case32.array("fluid_p").astype(bool)
    S = ap * np.where(fl, beta, 1.0)[:, None]
    sy, sz = nx, nx * ny
    idx = np.arange(nx * ny * nz)
    i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    for s, (off, opp, ok) in enumerate([(1, 1, i < nx - 1), (sy, 3, j < ny - 1), (sz, 5, k < nz - 1)]):
        up = 2 * s + 2  # +x, +y, +z slots
        r = idx[ok]
        assert np.allclose(S[r, up], S[r + off, opp], rtol=1e-12, atol=0)
    r = idx[j < ny - 1]
    assert np.abs(ap[r, 4] - ap[r + sy, 3]).max() > 0  # the operator itself is not symmetric


def test_multigrid_vcycle_contracts(case32, pyoracle):
    """One V-cycle as a stationary iteration reduces the error of the
    pressure system."""
    for rap, relax in ((0, 1), (1, 1), (1, 2)):
        orc = pyoracle.Oracle(case32, mg_rap=rap, mg_relax=relax)
        n = orc.box_sizes()[3]
        rng = np.random.default_rng(7)
        x_true = rng.standard_normal(n)
        b = orc.apply_operator(3, x_true)
        x = np.zeros(n)
        errs = []
        for _ in range(6):
            r = b - orc.apply_operator(3, x)
            x = x + orc.mg_vcycle(r)
            errs.append(np.linalg.norm(x - x_true) / np.linalg.norm(x_true))
        assert errs[-1] < 0.2 * errs[0], (rap, relax, errs)


def test_step_properties(case32, pyoracle):
    """After the projection the discrete divergence vanishes to round-off,
    the outlet u face copies the last interior face, walls are zero."""
    orc = pyoracle.Oracle(case32, vel_tol=1e-12, p_tol=1e-12)
    for step in range(1, 4):
        st = orc.step(min(1.0, step / 2.0))
        assert st.status == 0 and st.div_l2 < 1e-10
    u, v, w, p = orc.fields()
    nx, ny, nz = case32.shape
    U = u.reshape(nz, ny, nx + 1)
    assert np.array_equal(U[:, :, nx], U[:, :, nx - 1])
    assert np.all(v.reshape(nz, ny + 1, nx)[:, [0, ny], :] == 0)
    assert np.all(w.reshape(nz + 1, ny, nx)[[0, nz], :, :] == 0)
    assert np.all(p.reshape(-1)[case32.array("fluid_p") == 0] == 0)


def test_forces_of_a_closed_body(case32, pyoracle):
    """Staircase force definition: a uniform pressure on a closed body and
    still fluid give no net force; the pressure force is linear in p."""
    orc = pyoracle.Oracle(case32)
    nx, ny, nz = case32.shape
    fl = (case32.array("fluid_p") > 0) & (case32.array("id_p") > 0)
    zu, zv, zw = np.zeros((nx + 1) * ny * nz), np.zeros(nx * (ny + 1) * nz), np.zeros(nx * ny * (nz + 1))
    orc.set_fields(zu, zv, zw, np.where(fl, 3.0, 0.0))
    assert np.abs(orc.forces()).max() <= 1e-12
    rng = np.random.default_rng(4)
    p1, p2 = rng.standard_normal(nx * ny * nz) * fl, rng.standard_normal(nx * ny * nz) * fl
    orc.set_fields(zu, zv, zw, p1)
    f1 = orc.forces()
    orc.set_fields(zu, zv, zw, p2)
    f2 = orc.forces()
    orc.set_fields(zu, zv, zw, 2.0 * p1 + p2)
    assert np.allclose(orc.forces(), 2.0 * f1 + f2, rtol=1e-12, atol=1e-14)
    assert np.abs(f1).max() > 0


def test_oracle_dense_stages_match_reference_device_kernels_golden(pyoracle):
    """The oracle's BC cleanup, convection, gradient and momentum
    right-hand-side build, scatter, divergence and pressure right-hand side,
    and projection, bit for bit against the reference's own device kernels
    (gpu_dense_ops.hpp run on a GB300 by tests/golden/make_golden_device.py),
    fed the same seeded state and seeded stand-ins for the solve outputs."""
    path = os.path.join(GOLDEN, "refkernels_channel_32x12x12.npz")
    if not os.path.exists(path):
        pytest.skip("fixture not generated (tests/golden/make_golden_device.py needs a GPU)")
    import importlib
    sys.path.insert(0, GOLDEN)
    mgd = importlib.import_module("make_golden_device")
    g = np.load(path)
    ibm = importlib.import_module("ibm-3d-fpc_gb300")
    case = ibm.Case(ibm.channel_params(*mgd.SHAPE, Um=0.45, dt=1e-3))
    (u, v, w, p), xs = mgd.state_and_solves(case)
    ramp = float(g["ramp"])
    orc = pyoracle.Oracle(case)
    ub, vb, wb = orc.bc_cleanup(u, v, w, ramp)
    got = dict(zip(("rhs_u", "rhs_v", "rhs_w"), orc.momentum_rhs(ub, vb, wb, p)))
    orc.set_fields(ub, vb, wb, p)
    ut, vt, wt = orc.tilde(*xs[:3], ramp)
    got["rhs_p"] = orc.pressure_rhs(ut, vt, wt, ramp)
    st = orc.projection(ut, vt, wt, xs[3], ramp)
    got.update(zip("uvwp", orc.fields()))
    for k, val in got.items():
        assert np.array_equal(val.view(np.uint64), g[k].view(np.uint64)), k
    assert st.umax == float(g["umax"]) and st.vmax == float(g["vmax"]) and st.wmax == float(g["wmax"])
    assert abs(st.div_l2 - float(g["div_l2"])) <= 1e-12 * float(g["div_l2"])

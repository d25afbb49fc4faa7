"""Host setup (libibmhost) against the reference's own setup code.

The reference is compiled from its sources into oracle/_ref/ where they are
present (this container); the committed golden fixtures carry its outputs
everywhere else. Equality is bitwise.
"""
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")
NAMES = ["beta_p", "alpha_u", "alpha_v", "alpha_w", "fluid_p", "active_u", "active_v", "active_w", "active_qu",
         "active_qv", "active_qw", "id_u", "id_v", "id_w", "id_p", "id_qu", "id_qv", "id_qw", "scale_u", "scale_v",
         "scale_w", "rhs_u_bc", "rhs_v_bc", "rhs_w_bc", "div_bc_unit", "Au_vals", "Av_vals", "Aw_vals", "Ap_vals",
         "uin", "D_rowptr", "D_col", "D_val", "G_rowptr", "G_col", "G_val"]


def assert_bitwise(a, b, name):
    assert a.shape == b.shape, f"{name}: shape {a.shape} vs {b.shape}"
    if a.dtype == np.float64:
        bad = np.flatnonzero(a.view(np.uint64) != b.view(np.uint64))
    else:
        bad = np.flatnonzero(a != b)
    assert bad.size == 0, f"{name}: {bad.size} entries differ, first at {bad[:5]}: {a[bad[:5]]} vs {b[bad[:5]]}"


def test_sum_order_model_matches_std_unordered_map(ibm):
    from importlib import import_module
    native = import_module("ibm-3d-fpc_gb300._native")
    assert native.host().ibm_host_check_sum_order(200000, 12345) == 0


@pytest.mark.parametrize("tag", ["channel", "default"])
def test_setup_matches_reference_golden(ibm, tag):
    g = np.load(os.path.join(GOLDEN, f"setup_{tag}_32x12x12.npz"))
    vals = list(g["params"])
    prm = ibm.CaseParams(int(vals[0]), int(vals[1]), int(vals[2]), *vals[3:10], int(vals[10]), *vals[11:])
    case = ibm.Case(prm)
    for n in NAMES:
        assert_bitwise(g[n], case.array(n), n)
    c = case.counts
    assert [c["nu"], c["nv"], c["nw"], c["np"], c["nqu"], c["nqv"], c["nqw"], c["n_pruned"]] == list(g["counts"])


CASES = [
    dict(nx=48, ny=16, nz=16),
    dict(nx=160, ny=32, nz=32),
    dict(nx=64, ny=20, nz=12, Um=2.25, dt=2e-4),
    dict(nx=40, ny=24, nz=8, Lx=2.2, xcirc=0.2, ycirc=0.2, dt=2e-3),
    dict(nx=96, ny=16, nz=16, Rcirc=0.07, ycirc=0.15, nu=2e-3),
]


@pytest.mark.parametrize("kw", CASES, ids=lambda k: "x".join(str(k[d]) for d in ("nx", "ny", "nz")))
def test_setup_matches_reference_live(ibm, pyoracle, kw):
    if not pyoracle.reference_available():
        pytest.skip("reference checker not built (reference sources absent on this machine)")
    prm = ibm.channel_params(**kw)
    case = ibm.Case(prm)
    ref = pyoracle.ReferenceCase(prm)
    for n in NAMES:
        assert_bitwise(ref.array(n), case.array(n), n)


def test_counts_160x32x32(ibm):
    """Active counts of the 160x32x32 benchmark channel, as the reference's
    geometry code produces them."""
    case = ibm.Case(ibm.channel_params(160, 32, 32))
    c = case.counts
    assert (c["np"], c["nu"], c["nv"], c["nw"]) == (162816, 161536, 157440, 167904)
    assert c["nqu"] + c["nqv"] + c["nqw"] == 487904
    assert c["n_pruned"] == 4


def test_operator_structure(ibm):
    """Inactive rows are identity; momentum rows are 1-norm scaled; the
    pressure rows are -D G (solver_helpers.hpp:66; main.cu:98-103)."""
    case = ibm.Case(ibm.channel_params(48, 16, 16))
    nx, ny, nz = case.shape
    au = case.array("Au_vals").reshape(-1, 7)
    ids = case.array("id_u").reshape(nz, ny, nx + 1)[:, :, 1:nx].ravel()
    act = au[ids > 0]
    assert np.allclose(np.abs(act).sum(axis=1), 1.0, rtol=0, atol=4e-16)
    assert np.all(au[ids == 0, 0] == 1.0) and np.all(au[ids == 0, 1:] == 0.0)
    ap = case.array("Ap_vals").reshape(-1, 7)
    fl = case.array("fluid_p") > 0
    assert np.all(ap[fl, 0] > 0) and np.all(ap[fl, 1:] <= 0)


def test_bad_params_rejected(ibm):
    with pytest.raises(ibm.IBMError):
        ibm.Case(ibm.channel_params(2, 12, 12))

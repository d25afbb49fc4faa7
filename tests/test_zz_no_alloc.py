"""The allocation-free residual entry point (ibm_residual_noalloc) against the
context path: r must equal b - ibm_apply_operator(x) and the norms must match
the norms of that residual and of b, on two calls in a row that share the
library's fixed scratch array (a large operator, then a smaller one).

Device buffers come from torch; the entry point itself allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def rel_err(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def _bind(lib):
    f = lib.ibm_residual_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    f.restype = C.c_int
    return f


def test_residual_noalloc_matches_context_path(ibm):
    torch = pytest.importorskip("torch")
    case = ibm.Case(ibm.channel_params(64, 24, 20, Um=0.8, dt=1e-3))
    solver = ibm.Solver(case)
    f = _bind(solver._lib)
    nx, ny, nz = case.shape
    boxes = [(ibm.FIELD_P, "Ap_vals", (nx, ny, nz)), (ibm.FIELD_U, "Au_vals", (nx - 1, ny, nz))]
    rng = np.random.default_rng(21)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    for field, name, (bx, by, bz) in boxes:
        n = bx * by * bz
        vals = case.array(name)
        assert vals.size == 7 * n
        x = rng.standard_normal(n)
        b = rng.standard_normal(n)
        r_ctx = b - solver.apply_operator(field, x)
        dv = torch.from_numpy(vals.copy()).to(dev)
        dx = torch.from_numpy(x).to(dev)
        db = torch.from_numpy(b).to(dev)
        dr = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        dn = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = f(dv.data_ptr(), bx, by, bz, dx.data_ptr(), db.data_ptr(), dr.data_ptr(), dn.data_ptr(),
               stream.cuda_stream)
        assert rc == 0, rc
        stream.synchronize()
        r = dr.cpu().numpy()
        norms = dn.cpu().numpy()
        assert rel_err(r, r_ctx) <= REL_TOL, name
        assert abs(norms[0] - np.linalg.norm(r_ctx)) <= REL_TOL * np.linalg.norm(r_ctx), name
        assert abs(norms[1] - np.linalg.norm(b)) <= REL_TOL * np.linalg.norm(b), name


def test_residual_noalloc_rejects_bad_arguments(ibm):
    """Size and pointer checks return before any work is queued."""
    torch = pytest.importorskip("torch")
    f = _bind(ibm._native.gpu())
    dev = torch.device("cuda", 0)
    t = torch.zeros(8, dtype=torch.float64, device=dev)
    p = t.data_ptr()
    # 1025 x 1024 x 32 rows: beyond the 2^25 rows the fixed scratch array covers.
    assert f(p, 1025, 1024, 32, p, p, p, p, None) == -7
    assert f(p, 0, 1, 1, p, p, p, p, None) == -1
    host = np.zeros(8)
    assert f(p, 2, 2, 2, host.ctypes.data, p, p, p, None) == -1

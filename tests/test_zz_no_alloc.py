"""The allocation-free residual entry point (ibm_residual_noalloc) against the
context path, for callers that cannot allocate device memory themselves.

r must be bitwise equal to b - ibm_apply_operator(x) (the kernel evaluates the
stencil in the same order), and the norms must match the norms of that
residual and of b. The calls run back to back on the library's one fixed
scratch array: a 30-tile operator first, then 2-tile ones, so a later call
must not pick up partial sums a larger earlier call left behind. Free device
memory must not change across the later calls.

Device buffers come from torch; the entry point itself allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def _bind(lib):
    f = lib.ibm_residual_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    f.restype = C.c_int
    return f


def test_residual_noalloc_matches_context_path(ibm):
    torch = pytest.importorskip("torch")
    big = ibm.Case(ibm.channel_params(64, 24, 20, Um=0.8, dt=1e-3))
    small = ibm.Case(ibm.channel_params(24, 8, 8, Um=0.8, dt=1e-3))
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    calls = []
    for case in (big, small):
        nx, ny, nz = case.shape
        solver = ibm.Solver(case)
        calls.append((solver, case, ibm.FIELD_P, "Ap_vals", (nx, ny, nz)))
        calls.append((solver, case, ibm.FIELD_U, "Au_vals", (nx - 1, ny, nz)))
    # 30720 / 30240 rows (30 tiles of 1024), then 1536 / 1472 rows (2 tiles)
    assert [b[0] * b[1] * b[2] for *_, b in calls] == [30720, 30240, 1536, 1472]
    f = _bind(calls[0][0]._lib)
    rng = np.random.default_rng(21)
    for n_call, (solver, case, field, name, (bx, by, bz)) in enumerate(calls):
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
        free0 = torch.cuda.mem_get_info(0)[0]
        rc = f(dv.data_ptr(), bx, by, bz, dx.data_ptr(), db.data_ptr(), dr.data_ptr(), dn.data_ptr(),
               stream.cuda_stream)
        assert rc == 0, rc
        stream.synchronize()
        if n_call > 0:  # the first call may load the library's module onto the device
            assert torch.cuda.mem_get_info(0)[0] == free0, "the entry point allocated device memory"
        r = dr.cpu().numpy()
        norms = dn.cpu().numpy()
        assert bits_equal(r, r_ctx), name
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
    # r in place of x or b, or norms inside r, would race with the rows that
    # still read them: rejected before any work is queued.
    big = torch.zeros(64, dtype=torch.float64, device=dev)
    v7 = torch.zeros(7 * 8, dtype=torch.float64, device=dev)
    q = big.data_ptr()
    assert f(v7.data_ptr(), 2, 2, 2, q, q + 64, q, q + 256, None) == -1
    assert f(v7.data_ptr(), 2, 2, 2, q, q + 64, q + 128, q + 136, None) == -1

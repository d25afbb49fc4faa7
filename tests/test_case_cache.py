"""The on-disk case cache (include/ibm_host.h: ibm_case_save / ibm_case_load /
ibm_case_build_cached): a saved case loads back bit for bit, a file made for
other parameters or truncated is not used, and build_cached builds once and
loads afterwards."""
import ctypes as C
import os

import numpy as np
import pytest

NAMES = ["Au_vals", "Av_vals", "Aw_vals", "Ap_vals", "active_u", "fluid_p", "id_u", "id_qw", "scale_u", "rhs_u_bc",
         "div_bc_unit", "D_rowptr", "D_col", "D_val", "G_rowptr", "G_col", "G_val", "uin", "beta_p"]


def _arrays(ibm, lib, h):
    out = {}
    for n in NAMES:
        es = C.c_int()
        nb = lib.ibm_case_array_bytes(h, n.encode(), C.byref(es))
        assert nb >= 0, n
        ptr = lib.ibm_case_array(h, n.encode())
        dt = {1: np.uint8, 4: np.int32, 8: np.float64}[es.value]
        out[n] = np.frombuffer((C.c_ubyte * nb).from_address(ptr), dtype=dt).copy() if nb else np.zeros(0, dt)
    return out


@pytest.fixture(scope="module")
def lib(ibm):
    L = ibm._native.host()
    L.ibm_case_save.argtypes = [C.c_void_p, C.c_char_p]
    L.ibm_case_load.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_void_p)]
    L.ibm_case_build_cached.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_void_p)]
    return L


def test_save_load_round_trip(ibm, lib, tmp_path):
    prm = ibm.channel_params(40, 16, 12, Um=0.8, dt=1e-3)
    case = ibm.Case(prm)
    path = str(tmp_path / "case.bin").encode()
    assert lib.ibm_case_save(case._h, path) == 0
    h = C.c_void_p()
    assert lib.ibm_case_load(C.byref(prm), path, C.byref(h)) == 0
    try:
        want, got = _arrays(ibm, lib, case._h), _arrays(ibm, lib, h)
        for n in NAMES:
            assert want[n].dtype == got[n].dtype and np.array_equal(want[n].view(np.uint8), got[n].view(np.uint8)), n
    finally:
        lib.ibm_case_free(h)


def test_other_parameters_or_damage_are_not_loaded(ibm, lib, tmp_path):
    prm = ibm.channel_params(40, 16, 12, Um=0.8, dt=1e-3)
    case = ibm.Case(prm)
    path = tmp_path / "case.bin"
    assert lib.ibm_case_save(case._h, str(path).encode()) == 0
    other = ibm.channel_params(40, 16, 12, Um=0.8, dt=2e-3)
    h = C.c_void_p()
    assert lib.ibm_case_load(C.byref(other), str(path).encode(), C.byref(h)) == 1
    assert lib.ibm_case_load(C.byref(prm), str(tmp_path / "absent.bin").encode(), C.byref(h)) == 1
    data = path.read_bytes()
    path.write_bytes(data[: len(data) // 2])  # truncated file
    rc = lib.ibm_case_load(C.byref(prm), str(path).encode(), C.byref(h))
    assert rc != 0
    if rc == 0:
        lib.ibm_case_free(h)


def test_build_cached_builds_once(ibm, lib, tmp_path):
    prm = ibm.channel_params(40, 16, 12, Um=0.8, dt=1e-3)
    path = tmp_path / "cached.bin"
    h1, h2 = C.c_void_p(), C.c_void_p()
    assert lib.ibm_case_build_cached(C.byref(prm), str(path).encode(), C.byref(h1)) == 0
    assert path.exists()
    mtime = os.path.getmtime(path)
    assert lib.ibm_case_build_cached(C.byref(prm), str(path).encode(), C.byref(h2)) == 0
    assert os.path.getmtime(path) == mtime  # loaded, not rewritten
    try:
        a, b = _arrays(ibm, lib, h1), _arrays(ibm, lib, h2)
        for n in NAMES:
            assert np.array_equal(a[n].view(np.uint8), b[n].view(np.uint8)), n
    finally:
        lib.ibm_case_free(h1)
        lib.ibm_case_free(h2)

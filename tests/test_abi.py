"""The C-ABI libraries load and export every function their headers declare
(no GPU needed: nothing here calls into CUDA)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

LIBS = {
    "ibm_gpu.h": os.path.join(ROOT, "ibm-3d-fpc_gb300", "_build", "libibmgpu.so"),
    "ibm_host.h": os.path.join(ROOT, "ibm-3d-fpc_gb300", "_build", "libibmhost.so"),
}


def declared_functions(header: str):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b(ibm_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.mark.parametrize("header", sorted(LIBS))
def test_library_exports_declared_symbols(header):
    path = LIBS[header]
    assert os.path.exists(path), f"{path} not built"
    lib = ctypes.CDLL(path)
    names = declared_functions(header)
    assert len(names) >= 5
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"{os.path.basename(path)} lacks {missing}"


def test_error_codes_and_defaults(ibm):
    p = ibm.solver_params()
    assert (p.vel_tol, p.vel_maxit, p.vel_kdim, p.vel_jacobi_iters) == (1e-6, 250, 50, 1)
    assert (p.p_tol, p.p_maxit, p.p_kdim, p.p_pc_maxit, p.p_pc_relax_type, p.p_pc_rap_type) == (1e-9, 250, 50, 1, 1, 1)
    assert p.use_zero_initial_guess == 1
    # the reference's FP64 arithmetic by default; the mixed-precision options
    # only act when a mixed form is selected
    assert p.precision == 0 and p.vel_precision == -1 and p.arnoldi_passes == 2
    assert (p.df_residual, p.df_spmv, p.df_rhs, p.row_classes) == (1, 1, 1, 1)


def test_solver_params_struct_matches_header():
    """The ctypes mirror lists the header's ibm_solver_params fields in order."""
    from importlib import import_module
    native = import_module("ibm-3d-fpc_gb300._native")
    text = open(os.path.join(ROOT, "include", "ibm_gpu.h")).read()
    body = re.search(r"typedef struct ibm_solver_params \{(.*?)\} ibm_solver_params;", text, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = [n.strip() for decl in re.findall(r"\b(?:int|double)\s+([\w\s,]+);", body) for n in decl.split(",")]
    assert fields == [n for n, _ in native.SolverParams._fields_]


def test_create_rejects_bad_grid_without_gpu(ibm):
    """Argument checks happen before any CUDA call."""
    from importlib import import_module
    native = import_module("ibm-3d-fpc_gb300._native")
    lib = native.gpu()
    g = native.GridDesc(2, 12, 12, 2.5, 0.41, 0.41, 1.0, 1e-3, 1e-3, 0)
    ctx = ctypes.c_void_p()
    assert lib.ibm_create(ctypes.byref(g), ctypes.byref(ctx)) == -1
    assert b"bad grid" in lib.ibm_last_error(None)

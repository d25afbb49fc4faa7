"""GPU assembly of the momentum and pressure operators (ibm_assemble_momentum,
ibm_assemble_pressure): the row arithmetic checked on the host against the
CPU setup (the same source built for the host, unfused IEEE operations), and
the device kernels against the setup's arrays, bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HERE = os.path.dirname(os.path.abspath(__file__))
HOST_LIB_DIR = os.path.join(ROOT, "ibm-3d-fpc_gb300", "_build")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_assembly_rows_match_the_setup_on_the_host(ibm, tmp_path):
    ibm._native.host()  # builds / loads libibmhost
    exe = tmp_path / "assembly_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                    "-o", str(exe), os.path.join(HERE, "assembly_check.cpp"), "-L" + HOST_LIB_DIR, "-libmhost",
                    "-Wl,-rpath," + HOST_LIB_DIR], check=True)
    for args in (["48", "16", "16"], ["36", "10", "7", "2.25"], ["160", "32", "32", "0.45"],
                 ["96", "32", "16", "1.1", "0.07", "0.17", "2e-3", "5e-4"]):
        out = subprocess.run([str(exe)] + args, capture_output=True, text=True)
        assert out.returncode == 0, out.stdout[-2000:]
        assert "mismatches 0" in out.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(48, 16, 16), (36, 10, 7)])
def test_gpu_assembly_is_the_setup(ibm, shape):
    case = ibm.Case(ibm.channel_params(*shape, Um=1.0))
    s = ibm.Solver(case, ibm.solver_params())
    vals, scales = s.assemble_momentum()
    for f, v, sc in zip("uvw", vals, scales):
        assert np.array_equal(v.view(np.uint64), case.array(f"A{f}_vals").view(np.uint64)), f
        assert np.array_equal(sc.view(np.uint64), case.array(f"scale_{f}").view(np.uint64)), f
    ap = s.assemble_pressure()
    assert np.array_equal(ap.view(np.uint64), case.array("Ap_vals").view(np.uint64))
    # the assembled operators are the context's: a step equals one on the setup's operators
    ref = ibm.Solver(case, ibm.solver_params())
    a, b = s.step(1.0), ref.step(1.0)
    assert a.status == b.status and a.status >= 0
    for x, y, name in zip(s.fields(), ref.fields(), "uvwp"):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), name


@pytest.mark.gpu
def test_gpu_assembly_of_a_moved_body(ibm):
    """A context set up for one body position, re-assembled on the GPU for a
    body moved by 1e-3 (same masks and ids, other cut-cell rows and row
    scales), steps exactly as a context set up for the moved body: the new
    row scales reach the momentum right-hand sides."""
    import ctypes as C
    a = ibm.Case(ibm.channel_params(48, 16, 16, Um=1.0))
    b = ibm.Case(ibm.channel_params(48, 16, 16, Um=1.0, xcirc=0.501))
    for n in ("active_u", "active_v", "active_w", "fluid_p", "id_u", "id_v", "id_w", "id_p", "id_qu", "id_qv",
              "id_qw"):
        assert np.array_equal(a.array(n), b.array(n)), n
    assert not np.array_equal(a.array("scale_u"), b.array("scale_u"))
    s = ibm.Solver(a, ibm.solver_params())
    p = lambda x: C.c_void_p(x.ctypes.data)
    # the moved body's boundary data and projection, the old body's row scales
    s._check(s._lib.ibm_set_aux(s._ctx, *[p(a.array(n)) for n in ("scale_u", "scale_v", "scale_w")],
                                *[p(b.array(n)) for n in ("rhs_u_bc", "rhs_v_bc", "rhs_w_bc", "div_bc_unit",
                                                          "uin")]))
    cnt = b.counts
    s._check(s._lib.ibm_set_projection_csr(s._ctx, p(b.array("D_rowptr")), p(b.array("D_col")),
                                           p(b.array("D_val")), cnt["np"], p(b.array("G_rowptr")),
                                           p(b.array("G_col")), p(b.array("G_val")),
                                           cnt["nqu"] + cnt["nqv"] + cnt["nqw"]))
    s.assemble_pressure(case=b)
    vals, scales = s.assemble_momentum(case=b)
    for f, sc in zip("uvw", scales):
        assert np.array_equal(sc.view(np.uint64), b.array(f"scale_{f}").view(np.uint64)), f
    ref = ibm.Solver(b, ibm.solver_params())
    for _ in range(2):
        x, y = s.step(1.0), ref.step(1.0)
        assert x.status == y.status and x.status >= 0
    for x, y, name in zip(s.fields(), ref.fields(), "uvwp"):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), name

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

"""The C++ driver ibm_run (the reference's main.cu on the two C ABIs):
checkpoints written during a run, and a run restarted from a checkpoint
reproduces the uninterrupted run bit for bit (the step is deterministic);
the case cache is built once and reused."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "ibm-3d-fpc_gb300", "_build", "ibm_run")


def _run(tmp_path, *extra):
    args = [EXE, "-nx", "32", "-ny", "12", "-nz", "12", "-Lx", "2.5", "-xcirc", "0.5", "-ycirc", "0.2",
            "-Rcirc", "0.05", "-Um", "0.45", "-dt", "1e-3", "-nsteps", "6", "-inlet-ramp-steps", "4",
            "-vel-tol", "1e-10", "-p-tol", "1e-10", "-checkpoint-every", "3"] + list(extra)
    out = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    return out.stdout


def _fields(path):
    raw = path.read_bytes()
    hdr = np.frombuffer(raw[:16], dtype=np.int32)
    return hdr, np.frombuffer(raw[24:], dtype=np.float64)


def test_restart_reproduces_uninterrupted_run(tmp_path):
    if not os.path.exists(EXE):
        pytest.skip("ibm_run not built")
    full = tmp_path / "full"
    full.mkdir()
    _run(full, "-checkpoint", "a", "-case-cache", str(tmp_path / "case.bin"))
    assert (tmp_path / "case.bin").exists()
    h3, _ = _fields(full / "a_3.bin")
    assert list(h3) == [32, 12, 12, 3]
    resumed = tmp_path / "resumed"
    resumed.mkdir()
    log = _run(resumed, "-checkpoint", "b", "-restart", str(full / "a_3.bin"), "-case-cache", str(tmp_path / "case.bin"))
    steps = [int(l.split()[0]) for l in log.splitlines() if l[:4].strip().isdigit() and l.count("(") == 2]
    assert steps and steps[0] == 4  # the resumed run starts after the checkpoint
    h6a, fa = _fields(full / "a_6.bin")
    h6b, fb = _fields(resumed / "b_6.bin")
    assert list(h6a) == list(h6b) == [32, 12, 12, 6]
    assert np.array_equal(fa.view(np.uint64), fb.view(np.uint64))


def test_restart_rejects_other_grid(tmp_path):
    if not os.path.exists(EXE):
        pytest.skip("ibm_run not built")
    _run(tmp_path, "-checkpoint", "a")
    args = [EXE, "-nx", "40", "-ny", "12", "-nz", "12", "-nsteps", "5", "-restart", str(tmp_path / "a_3.bin")]
    out = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert out.returncode != 0 and "not a checkpoint" in out.stderr


def test_vtk_output_follows_the_reference_flags(tmp_path, ibm):
    """-write-vtk 1 -vtk-every 4 over 6 steps writes steps 1, 4 and 6 (the
    reference's rule: first, last and every N-th), named stem_%06d.vtk, and
    the last file holds the last checkpoint's fields."""
    if not os.path.exists(EXE):
        pytest.skip("ibm_run not built")
    _run(tmp_path, "-checkpoint", "c", "-write-vtk", "1", "-vtk-every", "4", "-vtk", "flow.vtk")
    names = sorted(f for f in os.listdir(tmp_path) if f.endswith(".vtk"))
    assert names == ["flow_000001.vtk", "flow_000004.vtk", "flow_000006.vtk"]
    _, f6 = _fields(tmp_path / "c_6.bin")
    nx, ny, nz = 32, 12, 12
    nu_, nv_, nw_ = (nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)
    p = f6[nu_ + nv_ + nw_:]
    lines = (tmp_path / "flow_000006.vtk").read_text().splitlines()
    k = lines.index("SCALARS pressure double 1")
    assert np.array_equal(np.array(lines[k + 2:k + 2 + nx * ny * nz], dtype=float), p)

"""Field output in the reference's VTK format: byte-identical to the
reference's own writer (compiled from its sources into the test shim) where
the shim is built, and the format read back otherwise."""
import ctypes as C
import os

import numpy as np
import pytest


def fields(case, seed=0):
    nx, ny, nz = case.shape
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(n) for n in ((nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1), nx * ny * nz)]


def test_vtk_format(ibm, tmp_path):
    case = ibm.Case(ibm.channel_params(16, 8, 6))
    u, v, w, p = fields(case)
    path = str(tmp_path / "f.vtk")
    ibm.write_vtk(path, case, u, v, w, p)
    lines = open(path).read().splitlines()
    nx, ny, nz = case.shape
    n = nx * ny * nz
    assert lines[0] == "# vtk DataFile Version 3.0"
    assert lines[4] == f"DIMENSIONS {nx + 1} {ny + 1} {nz + 1}"
    assert lines[7] == f"CELL_DATA {n}"
    blocks = {}
    i = 8
    while i < len(lines):
        name = lines[i].split()[1]
        blocks[name] = lines[i + 2:i + 2 + n]
        i += 2 + n
    assert list(blocks) == ["ux", "uy", "uz", "pressure", "fluid_mask"]
    U = u.reshape(nz, ny, nx + 1)
    assert np.array_equal(np.array(blocks["ux"], dtype=float), (0.5 * (U[:, :, :-1] + U[:, :, 1:])).ravel())
    W = w.reshape(nz + 1, ny, nx)
    assert np.array_equal(np.array(blocks["uz"], dtype=float), (0.5 * (W[:-1] + W[1:])).ravel())
    assert np.array_equal(np.array(blocks["pressure"], dtype=float), p)
    assert np.array_equal(np.array(blocks["fluid_mask"], dtype=int), (case.array("fluid_p") != 0).astype(int))
    assert ibm.vtk_step_name("a/b.c/st3d.vtk", 7) == "a/b.c/st3d_000007.vtk"
    assert ibm.vtk_step_name("noext", 12) == "noext_000012"


def test_vtk_is_the_reference_writer(ibm, pyoracle, tmp_path):
    if not pyoracle.reference_available():
        pytest.skip("reference checker not built")
    L = C.CDLL(pyoracle.REF_SO)
    L.ref_write_vtk.argtypes = [C.c_char_p] + [C.c_void_p] * 5 + [C.c_int] * 3 + [C.c_double] * 3
    L.ref_vtk_step_name.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_int]
    case = ibm.Case(ibm.channel_params(20, 8, 8))
    u, v, w, p = fields(case, 1)
    ours, ref = str(tmp_path / "ours.vtk"), str(tmp_path / "ref.vtk")
    ibm.write_vtk(ours, case, u, v, w, p)
    fl = np.ascontiguousarray(case.array("fluid_p"), dtype=np.uint8)
    cp = case.params
    L.ref_write_vtk(ref.encode(), *[C.c_void_p(x.ctypes.data) for x in (u, v, w, p, fl)], cp.nx, cp.ny, cp.nz,
                    cp.Lx, cp.Ly, cp.Lz)
    assert open(ours, "rb").read() == open(ref, "rb").read()
    buf = C.create_string_buffer(256)
    for base, step in (("st3d_channel_cylinder_struct_mac_cuda.vtk", 3), ("x/y.z/out", 123456)):
        L.ref_vtk_step_name(base.encode(), step, buf, 256)
        assert ibm.vtk_step_name(base, step) == buf.value.decode()

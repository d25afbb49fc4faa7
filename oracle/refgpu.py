"""The reference's own device kernels, run on the GPU as a checker (test
infrastructure only; the product never imports this module).

``_ref/ref_kernels.cubin`` holds the kernels of the reference's
gpu_dense_ops.hpp compiled from the reference's sources for sm_103a
(``make refcubin``; shim ``ref_shim/ref_kernels.cu``). This module loads it
with the CUDA driver API (cuModuleLoadData, cuModuleGetFunction,
cuLaunchKernel through ctypes) and runs the dense part of one reference
timestep (main.cu:249-357) with the reference's launches (256 threads,
ceil(n / 256) blocks) and its memsets, in its order. The four HYPRE solves
are not part of it: their outputs are taken from the caller, so the stages
can be fed the outputs of the library's own solves and compared stage by
stage. Device buffers come from torch (plumbing only).

The cubin is built where the reference's sources are; it is device code
only, so it loads on any host architecture that has the GPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")
BS = 256


def available() -> bool:
    return os.path.exists(CUBIN)


_cuda = None


def _driver():
    global _cuda
    if _cuda is None:
        _cuda = C.CDLL("libcuda.so.1")
    return _cuda


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what}: CUDA driver error {rc}")


class _Module:
    def __init__(self, path):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # the runtime's primary context is current on this thread
        data = open(path, "rb").read()
        self._data = C.create_string_buffer(data, len(data))
        self.mod = C.c_void_p()
        _check(_driver().cuModuleLoadData(C.byref(self.mod), self._data), "cuModuleLoadData")
        self.fns = {}

    def fn(self, name):
        if name not in self.fns:
            f = C.c_void_p()
            _check(_driver().cuModuleGetFunction(C.byref(f), self.mod, name.encode()), f"cuModuleGetFunction {name}")
            self.fns[name] = f
        return self.fns[name]

    def launch(self, name, n, *args):
        """One launch of kernel `name` over n threads, as main.cu launches
        them: <<<(n + 255) / 256, 256>>> on the default stream."""
        if n <= 0:
            return
        holders = []
        for a in args:
            if isinstance(a, float):
                holders.append(C.c_double(a))
            elif isinstance(a, int):
                holders.append(C.c_int(a))
            elif a is None:
                holders.append(C.c_uint64(0))
            else:  # a torch tensor
                holders.append(C.c_uint64(a.data_ptr()))
        params = (C.c_void_p * len(holders))(*[C.cast(C.pointer(h), C.c_void_p) for h in holders])
        grid = (n + BS - 1) // BS
        _check(_driver().cuLaunchKernel(self.fn(name), C.c_uint(grid), C.c_uint(1), C.c_uint(1), C.c_uint(BS),
                                        C.c_uint(1), C.c_uint(1), C.c_uint(0), C.c_void_p(0), params, C.c_void_p(0)),
               f"cuLaunchKernel {name}")


class ReferenceStep:
    """The reference's dense timestep stages on one case's arrays (any object
    with ``array(name)``, ``params`` and ``shape``, e.g. the package's Case)."""

    def __init__(self, case):
        import torch
        self.torch = torch
        self.m = _Module(CUBIN)
        self.case = case
        cp = case.params
        nx, ny, nz = case.shape
        self.nx, self.ny, self.nz = nx, ny, nz
        self.rho, self.dt = float(cp.rho), float(cp.dt)
        self.dx, self.dy, self.dz = cp.Lx / nx, cp.Ly / ny, cp.Lz / nz  # main.cu:21
        dev = torch.device("cuda")
        self.dev = dev
        up = lambda name: torch.from_numpy(np.ascontiguousarray(case.array(name))).to(dev)
        self.a = {n: up(n) for n in ("active_u", "active_v", "active_w", "fluid_p", "id_u", "id_v", "id_w", "id_p",
                                     "id_qu", "id_qv", "id_qw", "scale_u", "scale_v", "scale_w", "rhs_u_bc",
                                     "rhs_v_bc", "rhs_w_bc", "div_bc_unit", "D_rowptr", "D_col", "D_val",
                                     "G_rowptr", "G_col", "G_val")}
        for n in ("id_u", "id_v", "id_w", "id_p", "id_qu", "id_qv", "id_qw", "D_rowptr", "D_col", "G_rowptr",
                  "G_col"):
            assert self.a[n].dtype == torch.int32, n
        self.uin = np.ascontiguousarray(case.array("uin"))
        self.div_bc_unit = np.ascontiguousarray(case.array("div_bc_unit"))
        self.nqu = int(case.array("id_qu").max())
        self.nqv = int(case.array("id_qv").max())
        self.nqw = int(case.array("id_qw").max())
        self.nq = self.nqu + self.nqv + self.nqw
        self.np_ = int(case.array("id_p").max())
        self.Dn = int(case.array("D_rowptr").size - 1)
        self.Gn = int(case.array("G_rowptr").size - 1)

    def _zeros(self, n):
        return self.torch.zeros(n, dtype=self.torch.float64, device=self.dev)

    def _d(self, x):
        return self.torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to(self.dev)

    def run(self, u, v, w, p, ramp, solve):
        """One reference timestep's dense stages from the state (u, v, w, p)
        with inlet ramp `ramp`. solve(field, rhs) -> x supplies each solve's
        output (field 0..2 = u, v, w momentum, 3 = pressure; rhs and x are
        numpy arrays on the solve box). Returns a dict of numpy arrays: the
        momentum right-hand sides rhs_u/v/w, the pressure right-hand side
        rhs_p, the projected u, v, w, p, and div_l2, umax, vmax, wmax as
        main.cu:352-361 computes them."""
        m, a = self.m, self.a
        nx, ny, nz = self.nx, self.ny, self.nz
        rho, dt = self.rho, self.dt
        nuf, nvf, nwf, npc = (nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1), nx * ny * nz
        nmax = max(nuf, nvf, nwf)
        du, dv, dw, dp = self._d(u), self._d(v), self._d(w), self._d(p)
        duin = self._d(ramp * self.uin)  # main.cu:251, one IEEE product per entry
        m.launch("ref_apply_bc_cleanup", nmax, du, dv, dw, a["active_u"], a["active_v"], a["active_w"], duin, nx, ny,
                 nz)
        conv = [self._zeros(nuf), self._zeros(nvf), self._zeros(nwf)]
        for f, (name, n, act) in enumerate((("ref_conv_u", nuf, "active_u"), ("ref_conv_v", nvf, "active_v"),
                                            ("ref_conv_w", nwf, "active_w"))):
            m.launch(name, n, conv[f], du, dv, dw, a[act], nx, ny, nz, self.dx, self.dy, self.dz)
        pvec, gp = self._zeros(self.np_ + 1), self._zeros(self.nq + 1)
        gpx, gpy, gpz = self._zeros(nuf), self._zeros(nvf), self._zeros(nwf)
        m.launch("ref_pack_pressure_active", npc, pvec, dp, a["fluid_p"], a["id_p"], npc)
        m.launch("ref_spmv_csr_1based", self.Gn, self.Gn, a["G_rowptr"], a["G_col"], a["G_val"], pvec, gp)
        m.launch("ref_unpack_gp_u", nuf, gp, gpx, a["id_qu"], nx, ny, nz)
        m.launch("ref_unpack_gp_v", nvf, gp, gpy, a["id_qv"], nx, ny, nz, self.nqu)
        m.launch("ref_unpack_gp_w", nwf, gp, gpz, a["id_qw"], nx, ny, nz, self.nqu, self.nqv)
        nb = [(nx - 1) * ny * nz, nx * (ny - 1) * nz, nx * ny * (nz - 1)]
        rhs = [self._zeros(n) for n in nb]
        x0 = [self._zeros(n) for n in nb]
        m.launch("ref_build_u_full", nb[0], rhs[0], x0[0], du, conv[0], gpx, a["active_u"], a["id_u"], a["rhs_u_bc"],
                 a["scale_u"], nx, ny, nz, rho, dt, 1)
        m.launch("ref_build_v_full", nb[1], rhs[1], x0[1], dv, conv[1], gpy, a["active_v"], a["id_v"], a["rhs_v_bc"],
                 a["scale_v"], nx, ny, nz, rho, dt, 1)
        m.launch("ref_build_w_full", nb[2], rhs[2], x0[2], dw, conv[2], gpz, a["active_w"], a["id_w"], a["rhs_w_bc"],
                 a["scale_w"], nx, ny, nz, rho, dt, 1)
        self.torch.cuda.synchronize()
        out = {"rhs_u": rhs[0].cpu().numpy(), "rhs_v": rhs[1].cpu().numpy(), "rhs_w": rhs[2].cpu().numpy()}
        xs = [self._d(solve(f, out["rhs_" + "uvw"[f]])) for f in range(3)]
        ut, vt, wt = self._zeros(nuf), self._zeros(nvf), self._zeros(nwf)
        m.launch("ref_scatter_u", nuf, ut, xs[0], du, nx, ny, nz)
        m.launch("ref_scatter_v", nvf, vt, xs[1], dv, nx, ny, nz)
        m.launch("ref_scatter_w", nwf, wt, xs[2], dw, nx, ny, nz)
        m.launch("ref_apply_bc_cleanup", nmax, ut, vt, wt, a["active_u"], a["active_v"], a["active_w"], duin, nx, ny,
                 nz)
        qt = self._zeros(self.nq + 1)
        m.launch("ref_pack_projection_q_u", nuf, qt, ut, a["id_qu"], nx, ny, nz)
        m.launch("ref_pack_projection_q_v", nvf, qt, vt, a["id_qv"], nx, ny, nz, self.nqu)
        m.launch("ref_pack_projection_q_w", nwf, qt, wt, a["id_qw"], nx, ny, nz, self.nqu, self.nqv)
        dqt = self._zeros(self.np_ + 1)
        m.launch("ref_spmv_csr_1based", self.Dn, self.Dn, a["D_rowptr"], a["D_col"], a["D_val"], qt, dqt)
        rhsp, xp0 = self._zeros(npc), self._zeros(npc)
        m.launch("ref_build_pressure_rhs_full", npc, rhsp, xp0, dqt, a["div_bc_unit"], a["fluid_p"], a["id_p"], npc,
                 rho, dt, float(ramp))
        self.torch.cuda.synchronize()
        out["rhs_p"] = rhsp.cpu().numpy()
        xp = self._d(solve(3, out["rhs_p"]))
        phi, gphi = self._zeros(self.np_ + 1), self._zeros(self.nq + 1)
        m.launch("ref_pack_phi_active", npc, phi, xp, a["fluid_p"], a["id_p"], npc)
        m.launch("ref_spmv_csr_1based", self.Gn, self.Gn, a["G_rowptr"], a["G_col"], a["G_val"], phi, gphi)
        m.launch("ref_apply_q_correction", self.nq + 1, qt, gphi, dt / rho, self.nq + 1)
        du.copy_(ut)
        dv.copy_(vt)
        dw.copy_(wt)
        m.launch("ref_unpack_projection_q_u", nuf, qt, du, a["id_qu"], nx, ny, nz)
        m.launch("ref_unpack_projection_q_v", nvf, qt, dv, a["id_qv"], nx, ny, nz, self.nqu)
        m.launch("ref_unpack_projection_q_w", nwf, qt, dw, a["id_qw"], nx, ny, nz, self.nqu, self.nqv)
        m.launch("ref_apply_bc_cleanup", nmax, du, dv, dw, a["active_u"], a["active_v"], a["active_w"], duin, nx, ny,
                 nz)
        m.launch("ref_add_pressure_phi", npc, dp, phi, a["fluid_p"], a["id_p"], npc)
        divv = self._zeros(self.np_ + 1)
        m.launch("ref_spmv_csr_1based", self.Dn, self.Dn, a["D_rowptr"], a["D_col"], a["D_val"], qt, divv)
        self.torch.cuda.synchronize()
        out.update(u=du.cpu().numpy(), v=dv.cpu().numpy(), w=dw.cpu().numpy(), p=dp.cpu().numpy())
        # main.cu:354-361 on the host, in its order
        dv_h = divv.cpu().numpy()
        d = dv_h[1:] + ramp * self.div_bc_unit[1:]
        div2 = float(np.cumsum(d * d)[-1]) if d.size else 0.0  # a running sum, in index order
        out["div_l2"] = float(np.sqrt(div2 / max(1, self.np_)))
        out["umax"] = float(np.abs(out["u"]).max())
        out["vmax"] = float(np.abs(out["v"]).max())
        out["wmax"] = float(np.abs(out["w"]).max())
        return out

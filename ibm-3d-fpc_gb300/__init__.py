"""GB300-native per-timestep solver for the immersed-boundary channel flow.

Python mirror of the reference's driver (main.cu): a :class:`Case` holds the
CPU setup (geometry, masks, ids, embedded operators, CSR projection
operators) produced by ``libibmhost.so``; a :class:`Solver` owns one GPU
context of ``libibmgpu.so`` and advances the state one timestep per
:meth:`Solver.step`, exactly as the reference's step loop (main.cu:249-376).

Both libraries are C ABIs (include/ibm_host.h, include/ibm_gpu.h); this module
is a thin ctypes layer. There is no CPU fallback: without the CUDA library
or a GPU, :class:`Solver` raises.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import Optional

# A batch steps every instance on its own stream. CUDA maps streams onto
# CUDA_DEVICE_MAX_CONNECTIONS hardware work queues (8 unless set), and streams
# that share a queue serialise; 32 queues let the 32-channel ensemble run
# concurrently (1513 -> 2531 instance-steps/s on a GB300). It takes effect
# only if set before the process creates its CUDA context, and a value the
# caller set is kept.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np

from . import _native
from ._native import CaseCounts, CaseParams, GridDesc, SolverParams, SolveStats, StepStats

__all__ = ["CaseParams", "Case", "Solver", "Batch", "SolverParams", "StepStats", "channel_params", "solver_params",
           "IBM_OK", "IBM_NOT_CONVERGED", "IBMError", "FIELD_U", "FIELD_V", "FIELD_W", "FIELD_P"]

IBM_OK = 0
IBM_NOT_CONVERGED = 1
FIELD_U, FIELD_V, FIELD_W, FIELD_P = 0, 1, 2, 3


class IBMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def channel_params(nx: int, ny: int, nz: int, *, Lx: float = 2.5, Ly: float = 0.41, Lz: float = 0.41,
                   rho: float = 1.0, nu: float = 1.0e-3, Um: float = 0.45, dt: float = 1.0e-3,
                   nsub_beta: int = 10, beta_tol: float = 1.0e-8, alpha_tol: float = 1.0e-10,
                   xcirc: float = 0.5, ycirc: float = 0.2, Rcirc: float = 0.05) -> CaseParams:
    """Case parameters; defaults are the benchmark channel (2.5 x 0.41 x 0.41,
    cylinder of diameter 0.1 at (0.5, 0.2)), which differ from the reference's
    built-in defaults (common.hpp:49, 64-66)."""
    return CaseParams(nx, ny, nz, Lx, Ly, Lz, rho, nu, Um, dt, nsub_beta, beta_tol, alpha_tol, xcirc, ycirc, Rcirc)


def solver_params(**kw) -> SolverParams:
    """Solver options starting from the library defaults (the reference's
    defaults, common.hpp:68-80); keyword arguments override fields."""
    p = SolverParams()
    _native.gpu().ibm_solver_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(f"SolverParams has no field {k!r}")
        setattr(p, k, v)
    return p


_DTYPES = {1: np.uint8, 4: np.int32, 8: np.float64}


class Case:
    """CPU setup of one channel case (include/ibm_host.h)."""

    def __init__(self, params: CaseParams):
        self._lib = _native.host()
        self.params = params
        self._h = C.c_void_p()
        rc = self._lib.ibm_case_build(C.byref(params), C.byref(self._h))
        if rc != 0:
            raise IBMError(rc, "ibm_case_build failed (bad parameters)")
        cnt = CaseCounts()
        self._lib.ibm_case_get_counts(self._h, C.byref(cnt))
        self.counts = {f: getattr(cnt, f) for f, _ in CaseCounts._fields_}
        self._cache: dict[str, np.ndarray] = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.ibm_case_free(h)
            self._h = None

    def array(self, name: str) -> np.ndarray:
        """A named setup array (see include/ibm_host.h), as a numpy view."""
        if name not in self._cache:
            es = C.c_int()
            nb = self._lib.ibm_case_array_bytes(self._h, name.encode(), C.byref(es))
            if nb < 0:
                raise KeyError(name)
            ptr = self._lib.ibm_case_array(self._h, name.encode())
            buf = (C.c_ubyte * nb).from_address(ptr) if nb else bytearray()
            self._cache[name] = np.frombuffer(buf, dtype=_DTYPES[es.value]) if nb else np.zeros(0, _DTYPES[es.value])
        return self._cache[name]

    @property
    def shape(self):
        return self.params.nx, self.params.ny, self.params.nz

    def initial_fields(self):
        """The reference's initial state (main.cu:116-126): zero velocity and
        pressure, then the BC cleanup with the unramped inlet profile."""
        nx, ny, nz = self.shape
        u = np.zeros((nz, ny, nx + 1))
        v = np.zeros((nz, ny + 1, nx))
        w = np.zeros((nz + 1, ny, nx))
        p = np.zeros((nz, ny, nx))
        u[:, :, 0] = self.array("uin").reshape(nz, ny)
        return u.ravel(), v.ravel(), w.ravel(), p.ravel()


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Solver:
    """One GPU context running the per-timestep hot path (include/ibm_gpu.h)."""

    def __init__(self, case: Case, params: Optional[SolverParams] = None, device: int = 0, _ctx=None):
        self._lib = _native.gpu()
        self.case = case
        self._owned = _ctx is None
        if _ctx is None:
            g = grid_desc(case, device)
            self._ctx = C.c_void_p()
            rc = self._lib.ibm_create(C.byref(g), C.byref(self._ctx))
            if rc != 0:
                raise IBMError(rc, self._lib.ibm_last_error(None).decode())
        else:
            self._ctx = C.c_void_p(_ctx)
        nx, ny, nz = case.shape
        a = case.array
        self._check(self._lib.ibm_set_operator(self._ctx, FIELD_U, _ptr(a("Au_vals")), nx - 1, ny, nz))
        self._check(self._lib.ibm_set_operator(self._ctx, FIELD_V, _ptr(a("Av_vals")), nx, ny - 1, nz))
        self._check(self._lib.ibm_set_operator(self._ctx, FIELD_W, _ptr(a("Aw_vals")), nx, ny, nz - 1))
        self._check(self._lib.ibm_set_operator(self._ctx, FIELD_P, _ptr(a("Ap_vals")), nx, ny, nz))
        self._check(self._lib.ibm_set_masks(self._ctx, *[_ptr(a(n)) for n in (
            "active_u", "active_v", "active_w", "fluid_p", "active_qu", "active_qv", "active_qw",
            "id_u", "id_v", "id_w", "id_p", "id_qu", "id_qv", "id_qw")]))
        self._check(self._lib.ibm_set_aux(self._ctx, *[_ptr(a(n)) for n in (
            "scale_u", "scale_v", "scale_w", "rhs_u_bc", "rhs_v_bc", "rhs_w_bc", "div_bc_unit", "uin")]))
        cnt = case.counts
        nq = cnt["nqu"] + cnt["nqv"] + cnt["nqw"]
        self._check(self._lib.ibm_set_projection_csr(
            self._ctx, _ptr(a("D_rowptr")), _ptr(a("D_col")), _ptr(a("D_val")), cnt["np"],
            _ptr(a("G_rowptr")), _ptr(a("G_col")), _ptr(a("G_val")), nq))
        # the body, for the cut-surface force (compute_forces = 2)
        cp = case.params
        self._check(self._lib.ibm_set_body(self._ctx, cp.xcirc, cp.ycirc, cp.Rcirc,
                                           _ptr(np.ascontiguousarray(a("alpha_u"), dtype=np.float64)),
                                           _ptr(np.ascontiguousarray(a("alpha_v"), dtype=np.float64))))
        self.set_params(params if params is not None else solver_params())
        self.set_fields(*case.initial_fields())

    def close(self):
        if getattr(self, "_ctx", None):
            if self._owned:
                self._lib.ibm_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        self.close()

    def _check(self, rc: int) -> int:
        if rc < 0:
            raise IBMError(rc, self._lib.ibm_last_error(self._ctx).decode())
        return rc

    def set_params(self, p: SolverParams) -> None:
        self.params = p
        self._check(self._lib.ibm_set_solver_params(self._ctx, C.byref(p)))

    def set_fields(self, u=None, v=None, w=None, p=None) -> None:
        arrs = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, w, p)]
        self._check(self._lib.ibm_set_fields(self._ctx, *[None if x is None else _ptr(x) for x in arrs]))

    def fields(self):
        nx, ny, nz = self.case.shape
        u = np.empty((nx + 1) * ny * nz)
        v = np.empty(nx * (ny + 1) * nz)
        w = np.empty(nx * ny * (nz + 1))
        p = np.empty(nx * ny * nz)
        self._check(self._lib.ibm_get_fields(self._ctx, _ptr(u), _ptr(v), _ptr(w), _ptr(p)))
        return u, v, w, p

    def step(self, ramp: float) -> StepStats:
        st = StepStats()
        self._check(self._lib.ibm_step(self._ctx, C.c_double(ramp), C.byref(st)))
        return st

    def solve(self, field: int, b: np.ndarray, x0: Optional[np.ndarray] = None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        st = SolveStats()
        self._check(self._lib.ibm_solve(self._ctx, field, _ptr(b), _ptr(x), C.byref(st)))
        return x, st

    def apply_operator(self, field: int, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self._check(self._lib.ibm_apply_operator(self._ctx, field, _ptr(x), _ptr(y)))
        return y

    def apply_preconditioner(self, field: int, r: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.empty_like(r)
        self._check(self._lib.ibm_apply_preconditioner(self._ctx, field, _ptr(r), _ptr(z)))
        return z

    def solver_vector(self, field: int, which: int) -> np.ndarray:
        nx, ny, nz = self.case.shape
        n = [(nx - 1) * ny * nz, nx * (ny - 1) * nz, nx * ny * (nz - 1), nx * ny * nz][field]
        out = np.empty(n)
        self._check(self._lib.ibm_get_solver_vector(self._ctx, field, which, _ptr(out)))
        return out

    def launches(self) -> int:
        return int(self._lib.ibm_kernel_launches(self._ctx))

    def profile_reset(self) -> None:
        self._check(self._lib.ibm_profile_reset(self._ctx))

    def profile(self) -> "_native.Profile":
        """Launch accounting since the last profile_reset (ibm_profile)."""
        p = _native.Profile()
        self._check(self._lib.ibm_profile_get(self._ctx, C.byref(p)))
        return p

    def assemble_momentum(self, case: Optional[Case] = None):
        """Assembles the three momentum operators on the GPU from the masks,
        ids and body of ``case`` (default: the solver's own case) with
        ibm_assemble_momentum and sets them on the context; returns their
        row-major values and id-indexed row scales."""
        case = self.case if case is None else case
        nx, ny, nz = case.shape
        cp = case.params
        vals = [np.empty(7 * n) for n in ((nx - 1) * ny * nz, nx * (ny - 1) * nz, nx * ny * (nz - 1))]
        act = [np.ascontiguousarray(case.array(f"active_{f}"), dtype=np.uint8) for f in "uvw"]
        ids = [np.ascontiguousarray(case.array(f"id_{f}"), dtype=np.int32) for f in "uvw"]
        scales = [np.empty(int(i.max()) + 1) for i in ids]
        P = C.c_void_p * 3
        self._check(self._lib.ibm_assemble_momentum(
            self._ctx, cp.xcirc, cp.ycirc, cp.Rcirc, P(*[a.ctypes.data for a in act]),
            P(*[a.ctypes.data for a in ids]), P(*[a.ctypes.data for a in vals]), P(*[a.ctypes.data for a in scales])))
        return vals, scales

    def assemble_pressure(self, case: Optional[Case] = None):
        """Assembles the pressure operator on the GPU from the fractions,
        masks and ids of ``case`` (default: the solver's own case) with
        ibm_assemble_pressure and sets it on the context; returns its
        row-major values."""
        case = self.case if case is None else case
        a = case.array
        nx, ny, nz = case.shape
        vals = np.empty(7 * nx * ny * nz)
        fl = np.ascontiguousarray(a("fluid_p"), dtype=np.uint8)
        idp = np.ascontiguousarray(a("id_p"), dtype=np.int32)
        beta = np.ascontiguousarray(a("beta_p"), dtype=np.float64)
        al = [np.ascontiguousarray(a(f"alpha_{f}"), dtype=np.float64) for f in "uvw"]
        aq = [np.ascontiguousarray(a(f"active_q{f}"), dtype=np.uint8) for f in "uvw"]
        iq = [np.ascontiguousarray(a(f"id_q{f}"), dtype=np.int32) for f in "uvw"]
        P = C.c_void_p * 3
        self._check(self._lib.ibm_assemble_pressure(
            self._ctx, _ptr(fl), _ptr(idp), _ptr(beta), P(*[x.ctypes.data for x in al]),
            P(*[x.ctypes.data for x in aq]), P(*[x.ctypes.data for x in iq]), _ptr(vals)))
        return vals

    # ---------------------------------------------------------- adjoint extension
    def adjoint_setup(self) -> None:
        """Transposed-operator context and inlet weights (ibm_adjoint_setup)."""
        beta = np.ascontiguousarray(self.case.array("beta_p"), dtype=np.float64)
        self._check(self._lib.ibm_adjoint_setup(self._ctx, _ptr(beta)))

    def set_inflow(self, g) -> None:
        """Inflow profile g[ny*nz] (ibm_set_inflow; needs adjoint_setup)."""
        g = np.ascontiguousarray(g, dtype=np.float64)
        self._check(self._lib.ibm_set_inflow(self._ctx, _ptr(g)))

    def step_forward(self, ramp: float) -> StepStats:
        st = StepStats()
        self._check(self._lib.ibm_step_forward(self._ctx, C.c_double(ramp), C.byref(st)))
        return st

    def step_backward(self, ramp: float, weight: float = 0.0) -> StepStats:
        st = StepStats()
        self._check(self._lib.ibm_step_backward(self._ctx, C.c_double(ramp), C.c_double(weight), C.byref(st)))
        return st

    def adjoint_reset(self) -> None:
        self._check(self._lib.ibm_adjoint_reset(self._ctx))

    def adjoint_set(self, lu=None, lv=None, lw=None, lp=None) -> None:
        arrs = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (lu, lv, lw, lp)]
        self._check(self._lib.ibm_adjoint_set(self._ctx, *[None if x is None else _ptr(x) for x in arrs]))

    def adjoint_get(self):
        """(lambda_u, lambda_v, lambda_w, lambda_p, dJ/dg, dJ/dnu)."""
        nx, ny, nz = self.case.shape
        out = [np.empty((nx + 1) * ny * nz), np.empty(nx * (ny + 1) * nz), np.empty(nx * ny * (nz + 1)),
               np.empty(nx * ny * nz), np.empty(ny * nz), np.empty(1)]
        self._check(self._lib.ibm_adjoint_get(self._ctx, *[_ptr(x) for x in out]))
        return out[0], out[1], out[2], out[3], out[4], float(out[5][0])

    def adjoint_solve_stats(self):
        """Stats of the last reverse sweep's transposed solves (u, v, w, p)."""
        out = (SolveStats * 4)()
        self._check(self._lib.ibm_adjoint_solve_stats(self._ctx, out))
        return list(out)

    def tape_depth(self) -> int:
        return self._check(self._lib.ibm_adjoint_tape_depth(self._ctx))

    def checkpoint_save(self, slot: int) -> None:
        self._check(self._lib.ibm_checkpoint_save(self._ctx, slot))

    def checkpoint_load(self, slot: int) -> None:
        self._check(self._lib.ibm_checkpoint_load(self._ctx, slot))

    def checkpoint_clear(self) -> None:
        self._check(self._lib.ibm_checkpoint_clear(self._ctx))

    def drag_gradient(self, ramps, window, checkpoint_every: int = 20):
        """Mean end-of-step drag over the steps in ``window`` (1-based step
        numbers) of len(ramps) steps from the current fields, and its gradient
        with respect to the inflow profile and nu: (J, dJ/dg, dJ/dnu).

        Checkpointing with recomputation: the forward sweep saves the state
        every ``checkpoint_every`` steps; the reverse sweep replays each
        segment from its checkpoint with ibm_step_forward (the tape holds one
        segment) and runs ibm_step_backward over it in reverse. The fields
        are left at the state after the last step."""
        window = set(window)
        n = len(ramps)
        w = 1.0 / len(window)
        p = self.params
        if not p.compute_forces:
            p.compute_forces = 1
            self.set_params(p)
        self.adjoint_reset()
        self.checkpoint_clear()
        J = 0.0
        for k in range(1, n + 1):
            if (k - 1) % checkpoint_every == 0:
                self.checkpoint_save((k - 1) // checkpoint_every)
            st = self.step(ramps[k - 1])
            if k in window:
                J += w * st.force[0]
        end = self.fields()
        for seg in range((n - 1) // checkpoint_every, -1, -1):
            first = seg * checkpoint_every + 1
            last = min(n, first + checkpoint_every - 1)
            self.checkpoint_load(seg)
            for k in range(first, last + 1):
                self.step_forward(ramps[k - 1])
            for k in range(last, first - 1, -1):
                self.step_backward(ramps[k - 1], w if k in window else 0.0)
        self.set_fields(*end)
        *_, dg, dnu = self.adjoint_get()
        return J, dg, dnu

    def run(self, nsteps: int, ramp_steps: int = 200, start: int = 1, callback=None):
        """The reference's step loop (main.cu:249-251): ramp = min(1, step/ramp_steps)."""
        out = []
        for step in range(start, start + nsteps):
            ramp = min(1.0, step / float(ramp_steps))
            st = self.step(ramp)
            out.append(st)
            if callback:
                callback(step, st)
        return out


def write_vtk(path: str, case: Case, u, v, w, p) -> None:
    """Fields in the reference's VTK format (ibm_write_vtk, include/ibm_host.h)."""
    cp = case.params
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, w, p)]
    fluid = np.ascontiguousarray(case.array("fluid_p"), dtype=np.uint8)
    rc = _native.host().ibm_write_vtk(path.encode(), *[_ptr(x) for x in arrs], _ptr(fluid), cp.nx, cp.ny, cp.nz,
                                      cp.Lx, cp.Ly, cp.Lz)
    if rc != 0:
        raise IBMError(rc, f"ibm_write_vtk could not write {path}")


def vtk_step_name(base: str, step: int) -> str:
    """The reference's per-step VTK file name (stem + _%06d + extension)."""
    buf = C.create_string_buffer(4096)
    _native.host().ibm_vtk_step_name(base.encode(), step, buf, len(buf))
    return buf.value.decode()


def grid_desc(case: Case, device: int = 0) -> GridDesc:
    cp = case.params
    return GridDesc(cp.nx, cp.ny, cp.nz, cp.Lx, cp.Ly, cp.Lz, cp.rho, cp.nu, cp.dt, device)


class Batch:
    """Independent channels stepped together (ibm_batch_*, include/ibm_gpu.h).

    ``solvers[i]`` is a Solver on instance i's context (inputs, parameters and
    fields are set per instance); ``step(ramps)`` queues one step of every
    instance before waiting for any, so instances in graph mode run
    concurrently on the GPU."""

    def __init__(self, cases, params=None, device: int = 0):
        self._lib = _native.gpu()
        n = len(cases)
        grids = (GridDesc * n)(*[grid_desc(c, device) for c in cases])
        self._b = C.c_void_p()
        rc = self._lib.ibm_batch_create(n, grids, C.byref(self._b))
        if rc != 0:
            raise IBMError(rc, self._lib.ibm_last_error(None).decode())
        if params is None or isinstance(params, SolverParams):
            params = [params] * n
        self.solvers = [Solver(c, p, device, _ctx=self._lib.ibm_batch_ctx(self._b, i))
                        for i, (c, p) in enumerate(zip(cases, params))]

    def __len__(self):
        return len(self.solvers)

    def step(self, ramps) -> list:
        n = len(self.solvers)
        if isinstance(ramps, (int, float)):
            ramps = [float(ramps)] * n
        r = (C.c_double * n)(*ramps)
        stats = (StepStats * n)()
        rc = self._lib.ibm_batch_step(self._b, r, stats)
        if rc < 0:
            bad = next(i for i in range(n) if stats[i].status < 0)
            raise IBMError(rc, f"instance {bad}: " + self._lib.ibm_last_error(self.solvers[bad]._ctx).decode())
        return list(stats)

    def close(self):
        for s in getattr(self, "solvers", []):
            s.close()
        if getattr(self, "_b", None):
            self._lib.ibm_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        self.close()


def kernel_names() -> list:
    """Names of the kernel classes of ibm_profile, in index order."""
    lib = _native.gpu()
    out = []
    for k in range(64):
        name = lib.ibm_kernel_name(k).decode()
        out.append(name)
        if name == "setup":
            return out
    return out


def force_coefficients(force, params: CaseParams):
    """Drag and lift coefficients of the benchmark channel (Schaefer and Turek
    1996, 3D case with a full-height cylinder): c = 2 F / (rho U^2 D H) with
    the mean inflow velocity U = 4 Um / 9, D = 2 Rcirc, H = Lz."""
    u_mean = 4.0 * params.Um / 9.0
    scale = 2.0 / (params.rho * u_mean * u_mean * 2.0 * params.Rcirc * params.Lz)
    return force[0] * scale, force[1] * scale


def stats_dict(st: StepStats) -> dict:
    d = {"ramp": st.ramp, "div_l2": st.div_l2, "umax": st.umax, "vmax": st.vmax, "wmax": st.wmax,
         "status": st.status, "t_total_ms": st.t_total_ms, "t_rhs_ms": st.t_rhs_ms, "t_mom_ms": st.t_mom_ms,
         "t_p_ms": st.t_p_ms, "t_proj_ms": st.t_proj_ms, "force": tuple(st.force)}
    for f in ("u", "v", "w", "p"):
        s = getattr(st, f)
        d[f"its_{f}"] = s.iters
        d[f"rel_{f}"] = s.rel_res
    return d

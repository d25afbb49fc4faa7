"""ctypes binding of the CPU oracle (test infrastructure only).

Used by the tests, the smoke check and the benchmark's CPU-baseline leg as
the checker; the product never imports it. ``build()`` compiles the oracle
(and, where the reference sources exist, the reference checker) with make.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libibmref.so")
# The reference's source tree, where it is present (it is only needed to build
# the reference checkers; IBM_REFERENCE_DIR overrides the default location).
REFERENCE_DIR = os.environ.get("IBM_REFERENCE_DIR", "/root/reference")


def build(with_reference: bool = True) -> None:
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if with_reference and os.path.isdir(REFERENCE_DIR):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "refcubin", f"REFERENCE={REFERENCE_DIR}"], check=True)


class OracleParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
                ("rho", C.c_double), ("nu", C.c_double), ("dt", C.c_double),
                ("use_zero_initial_guess", C.c_int),
                ("vel_tol", C.c_double), ("vel_maxit", C.c_int), ("vel_kdim", C.c_int), ("vel_jacobi_iters", C.c_int),
                ("p_tol", C.c_double), ("p_maxit", C.c_int), ("p_kdim", C.c_int),
                ("p_pc", C.c_int), ("mg_rap", C.c_int), ("mg_relax", C.c_int), ("mg_nu1", C.c_int),
                ("mg_nu2", C.c_int), ("mg_omega", C.c_double), ("mg_coarse_max", C.c_int), ("mg_max_levels", C.c_int),
                ("mg_group_ratio", C.c_double), ("mg_options", C.c_int),
                ("mg_nu_coarse", C.c_int)]


_IN_FIELDS = ["Au", "Av", "Aw", "Ap", "active_u", "active_v", "active_w", "fluid_p", "active_qu", "active_qv",
              "active_qw", "id_u", "id_v", "id_w", "id_p", "id_qu", "id_qv", "id_qw", "scale_u", "scale_v",
              "scale_w", "rhs_u_bc", "rhs_v_bc", "rhs_w_bc", "div_bc_unit", "D_rowptr", "D_col", "D_val",
              "G_rowptr", "G_col", "G_val", "uin"]


class OracleInputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in _IN_FIELDS]


class OSolve(C.Structure):
    _fields_ = [("iters", C.c_int), ("rel_res", C.c_double), ("status", C.c_int)]


class OStep(C.Structure):
    _fields_ = [("u", OSolve), ("v", OSolve), ("w", OSolve), ("p", OSolve), ("div_l2", C.c_double),
                ("umax", C.c_double), ("vmax", C.c_double), ("wmax", C.c_double), ("status", C.c_int),
                ("force", C.c_double * 3)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_reference=False)
        L = C.CDLL(ORACLE_SO)
        vp, d, i = C.c_void_p, C.c_double, C.c_int
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [C.POINTER(OracleParams), C.POINTER(OracleInputs)]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_fields.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_get_fields.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_step.argtypes = [vp, d, C.POINTER(OStep)]
        L.oracle_forces.argtypes = [vp, vp]
        L.oracle_bc_cleanup.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_convection.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.oracle_momentum_rhs.argtypes = [vp] + [vp] * 7
        L.oracle_pressure_rhs.argtypes = [vp, vp, vp, vp, d, vp]
        L.oracle_tilde.argtypes = [vp, vp, vp, vp, d, vp, vp, vp]
        L.oracle_projection.argtypes = [vp, vp, vp, vp, vp, d, C.POINTER(OStep)]
        L.oracle_apply_operator.argtypes = [vp, i, vp, vp]
        L.oracle_solve.argtypes = [vp, i, vp, vp, C.POINTER(OSolve)]
        L.oracle_mg_levels.argtypes = [vp]
        L.oracle_mg_level_info.argtypes = [vp, i, vp, C.POINTER(i), C.POINTER(i)]
        L.oracle_mg_level_coef.argtypes = [vp, i, vp]
        L.oracle_mg_vcycle.argtypes = [vp, vp, vp]
        L.oracle_step_backward.argtypes = [vp, vp, d, vp, d, vp, vp, vp, vp, vp, vp]
        L.oracle_set_body.argtypes = [vp, d, d, d, vp, vp]
        _lib = L
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Oracle:
    """CPU timestep on a case's arrays (any object with ``array(name)`` and
    ``params``/``shape``, e.g. the package's Case)."""

    def __init__(self, case, *, vel_tol=1e-13, vel_maxit=500, vel_kdim=50, vel_jacobi_iters=1, p_tol=1e-13,
                 p_maxit=500, p_kdim=50, p_pc=1, mg_rap=1, mg_relax=1, mg_nu1=1, mg_nu2=1, mg_omega=2.0 / 3.0,
                 mg_coarse_max=64, mg_max_levels=40, mg_group_ratio=0.0, mg_options=3, mg_nu_coarse=0,
                 use_zero_initial_guess=1, cut_force=False):
        self.L = lib()
        cp = case.params
        self.shape = (cp.nx, cp.ny, cp.nz)
        self.prm = OracleParams(cp.nx, cp.ny, cp.nz, cp.Lx, cp.Ly, cp.Lz, cp.rho, cp.nu, cp.dt,
                                use_zero_initial_guess, vel_tol, vel_maxit, vel_kdim, vel_jacobi_iters, p_tol,
                                p_maxit, p_kdim, p_pc, mg_rap, mg_relax, mg_nu1, mg_nu2, mg_omega, mg_coarse_max,
                                mg_max_levels, mg_group_ratio, mg_options, mg_nu_coarse)
        names = {"Au": "Au_vals", "Av": "Av_vals", "Aw": "Aw_vals", "Ap": "Ap_vals"}
        self._keep = {n: np.ascontiguousarray(case.array(names.get(n, n))) for n in _IN_FIELDS}
        self.inp = OracleInputs(*[_p(self._keep[n]) for n in _IN_FIELDS])
        self.h = self.L.oracle_create(C.byref(self.prm), C.byref(self.inp))
        if cut_force:  # forces (and the adjoint's drag seed) on the cut surface of the cylinder
            self._alpha = [np.ascontiguousarray(case.array(n), dtype=np.float64) for n in ("alpha_u", "alpha_v")]
            self.L.oracle_set_body(self.h, cp.xcirc, cp.ycirc, cp.Rcirc, _p(self._alpha[0]), _p(self._alpha[1]))
        u, v, w, p = case.initial_fields()
        self.set_fields(u, v, w, p)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_destroy(self.h)
            self.h = None

    def sizes(self):
        nx, ny, nz = self.shape
        return (nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1), nx * ny * nz

    def box_sizes(self):
        nx, ny, nz = self.shape
        return (nx - 1) * ny * nz, nx * (ny - 1) * nz, nx * ny * (nz - 1), nx * ny * nz

    def set_fields(self, u, v, w, p):
        self._f = [np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, w, p)]
        self.L.oracle_set_fields(self.h, *[_p(x) for x in self._f])

    def fields(self):
        out = [np.empty(n) for n in self.sizes()]
        self.L.oracle_get_fields(self.h, *[_p(x) for x in out])
        return out

    def forces(self):
        """Force of the fluid on the body from the current fields."""
        out = np.zeros(3)
        self.L.oracle_forces(self.h, _p(out))
        return out

    def step(self, ramp: float) -> OStep:
        st = OStep()
        self.L.oracle_step(self.h, C.c_double(ramp), C.byref(st))
        return st

    def bc_cleanup(self, u, v, w, ramp: float):
        u, v, w = (np.array(x, dtype=np.float64) for x in (u, v, w))
        uin = ramp * self._keep["uin"]
        self.L.oracle_bc_cleanup(self.h, _p(u), _p(v), _p(w), _p(uin))
        return u, v, w

    def convection(self, u, v, w):
        u, v, w = (np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, w))
        out = [np.empty(n) for n in self.sizes()[:3]]
        self.L.oracle_convection(self.h, _p(u), _p(v), _p(w), *[_p(x) for x in out])
        return out

    def momentum_rhs(self, u, v, w, p):
        ins = [np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, w, p)]
        out = [np.empty(n) for n in self.box_sizes()[:3]]
        self.L.oracle_momentum_rhs(self.h, *[_p(x) for x in ins], *[_p(x) for x in out])
        return out

    def tilde(self, xu, xv, xw, ramp):
        ins = [np.ascontiguousarray(x, dtype=np.float64) for x in (xu, xv, xw)]
        out = [np.empty(n) for n in self.sizes()[:3]]
        self.L.oracle_tilde(self.h, *[_p(x) for x in ins], C.c_double(ramp), *[_p(x) for x in out])
        return out

    def pressure_rhs(self, ut, vt, wt, ramp):
        ins = [np.ascontiguousarray(x, dtype=np.float64) for x in (ut, vt, wt)]
        out = np.empty(self.sizes()[3])
        self.L.oracle_pressure_rhs(self.h, *[_p(x) for x in ins], C.c_double(ramp), _p(out))
        return out

    def projection(self, ut, vt, wt, xp, ramp) -> OStep:
        ins = [np.ascontiguousarray(x, dtype=np.float64) for x in (ut, vt, wt, xp)]
        st = OStep()
        self.L.oracle_projection(self.h, *[_p(x) for x in ins], C.c_double(ramp), C.byref(st))
        return st

    def apply_operator(self, field: int, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self.L.oracle_apply_operator(self.h, field, _p(x), _p(y))
        return y

    def solve(self, field: int, b, x0=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        st = OSolve()
        self.L.oracle_solve(self.h, field, _p(b), _p(x), C.byref(st))
        return x, st

    def mg_levels(self):
        n = self.L.oracle_mg_levels(self.h)
        out = []
        for l in range(n):
            dims = np.zeros(3, np.int32)
            cd, ns = C.c_int(), C.c_int()
            self.L.oracle_mg_level_info(self.h, l, _p(dims), C.byref(cd), C.byref(ns))
            out.append((tuple(int(x) for x in dims), cd.value))
        return out

    def mg_level_coef(self, l: int) -> np.ndarray:
        dims, _ = self.mg_levels()[l]
        n = dims[0] * dims[1] * dims[2]
        out = np.empty(n * 27)
        self.L.oracle_mg_level_coef(self.h, l, _p(out))
        return out.reshape(n, 27)

    def mg_vcycle(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        self.L.oracle_mg_vcycle(self.h, _p(b), _p(x))
        return x

    def step_backward(self, ot: "Oracle", ramp: float, beta_p, weight: float, lam, dg) -> float:
        """Reverse sweep of one step (oracle_step_backward): lam (u, v, w, p
        lambdas) and dg are updated in place; returns the step's dJ/dnu."""
        dnu = np.zeros(1)
        beta = np.ascontiguousarray(beta_p, dtype=np.float64)
        rc = self.L.oracle_step_backward(self.h, ot.h, C.c_double(ramp), _p(beta), C.c_double(weight),
                                         *[_p(x) for x in lam], _p(dg), _p(dnu))
        if rc != 0:
            raise RuntimeError(f"oracle_step_backward failed ({rc})")
        return float(dnu[0])


def transpose7(vals, nb):
    """Row-major 7-point operator [n][7] on a box nb = (nbx, nby, nbz) ->
    its transpose in the same layout (slot order C,-x,+x,-y,+y,-z,+z)."""
    nbx, nby, nbz = nb
    A = np.asarray(vals, dtype=np.float64).reshape(nbz, nby, nbx, 7)
    T = np.zeros_like(A)
    T[..., 0] = A[..., 0]
    T[:, :, 1:, 1] = A[:, :, :-1, 2]
    T[:, :, :-1, 2] = A[:, :, 1:, 1]
    T[:, 1:, :, 3] = A[:, :-1, :, 4]
    T[:, :-1, :, 4] = A[:, 1:, :, 3]
    T[1:, :, :, 5] = A[:-1, :, :, 6]
    T[:-1, :, :, 6] = A[1:, :, :, 5]
    return T.ravel()


class TransposedCase:
    """A case view whose four operators are transposed."""

    def __init__(self, case):
        self.base = case
        self.params = case.params
        nx, ny, nz = case.shape
        boxes = {"Au_vals": (nx - 1, ny, nz), "Av_vals": (nx, ny - 1, nz), "Aw_vals": (nx, ny, nz - 1),
                 "Ap_vals": (nx, ny, nz)}
        self._t = {n: transpose7(case.array(n), b) for n, b in boxes.items()}

    @property
    def shape(self):
        return self.base.shape

    def array(self, name):
        return self._t[name] if name in self._t else self.base.array(name)

    def initial_fields(self):
        return self.base.initial_fields()


def drag_gradient(case, ramps, window, **oracle_kw):
    """Objective J = mean over the steps in ``window`` (1-based step numbers)
    of the end-of-step drag F_x, for len(ramps) steps from the case's initial
    fields; returns (J, dJ/dg, dJ/dnu) by the oracle's reverse sweep (every
    step-start state kept)."""
    o = Oracle(case, **oracle_kw)
    ot = Oracle(TransposedCase(case), **oracle_kw)
    states, J = [], 0.0
    w = 1.0 / len(window)
    for n, ramp in enumerate(ramps, start=1):
        states.append(o.fields())
        o.step(ramp)
        if n in window:
            J += w * o.forces()[0]
    lam = [np.zeros(s) for s in o.sizes()]
    nx, ny, nz = case.shape
    dg = np.zeros(ny * nz)
    dnu = 0.0
    beta = case.array("beta_p")
    for n in range(len(ramps), 0, -1):
        o.set_fields(*states[n - 1])
        dnu += o.step_backward(ot, ramps[n - 1], beta, w if n in window else 0.0, lam, dg)
    return J, dg, dnu, lam


def drag_objective(case, ramps, window, **oracle_kw):
    o = Oracle(case, **oracle_kw)
    J = 0.0
    for n, ramp in enumerate(ramps, start=1):
        o.step(ramp)
        if n in window:
            J += o.forces()[0] / len(window)
    return J


class RefParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int)] + \
        [(n, C.c_double) for n in "Lx Ly Lz rho nu Um dt".split()] + [("nsub_beta", C.c_int)] + \
        [(n, C.c_double) for n in "beta_tol alpha_tol xcirc ycirc Rcirc".split()]


def reference_available() -> bool:
    return os.path.exists(REF_SO)


class ReferenceCase:
    """The reference's own CPU setup (compiled from its sources into _ref/)."""

    def __init__(self, params):
        self.L = C.CDLL(REF_SO)
        L = self.L
        L.ref_case_build.restype = C.c_void_p
        L.ref_case_build.argtypes = [C.POINTER(RefParams)]
        L.ref_case_array_bytes.restype = C.c_long
        L.ref_case_array_bytes.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_int)]
        L.ref_case_array_get.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p, C.c_long]
        L.ref_case_free.argtypes = [C.c_void_p]
        L.ref_enforce_bc.argtypes = [C.c_void_p] * 7 + [C.c_int] * 3
        L.ref_convection.argtypes = [C.c_void_p] * 9 + [C.c_int] * 3 + [C.c_double] * 3
        cp = params
        self.params = params
        rp = RefParams(cp.nx, cp.ny, cp.nz, cp.Lx, cp.Ly, cp.Lz, cp.rho, cp.nu, cp.Um, cp.dt, cp.nsub_beta,
                       cp.beta_tol, cp.alpha_tol, cp.xcirc, cp.ycirc, cp.Rcirc)
        self.h = L.ref_case_build(C.byref(rp))
        self._cache = {}

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_case_free(self.h)
            self.h = None

    def array(self, name: str) -> np.ndarray:
        if name not in self._cache:
            e = C.c_int()
            n = self.L.ref_case_array_bytes(self.h, name.encode(), C.byref(e))
            if n < 0:
                raise KeyError(name)
            dt = {1: np.uint8, 4: np.int32, 8: np.float64}[e.value]
            a = np.empty(n // e.value, dt)
            self.L.ref_case_array_get(self.h, name.encode(), _p(a), n)
            self._cache[name] = a
        return self._cache[name]

    def enforce_bc(self, u, v, w, uin_step):
        nx, ny, nz = self.params.nx, self.params.ny, self.params.nz
        u, v, w = (np.array(x, dtype=np.float64) for x in (u, v, w))
        uin_step = np.ascontiguousarray(uin_step, dtype=np.float64)
        self.L.ref_enforce_bc(_p(u), _p(v), _p(w), _p(self.array("active_u")), _p(self.array("active_v")),
                              _p(self.array("active_w")), _p(uin_step), nx, ny, nz)
        return u, v, w

    def convection(self, u, v, w):
        cp = self.params
        nx, ny, nz = cp.nx, cp.ny, cp.nz
        u, v, w = (np.ascontiguousarray(x, dtype=np.float64) for x in (u, v, w))
        out = [np.empty((nx + 1) * ny * nz), np.empty(nx * (ny + 1) * nz), np.empty(nx * ny * (nz + 1))]
        self.L.ref_convection(*[_p(x) for x in out], _p(u), _p(v), _p(w), _p(self.array("active_u")),
                              _p(self.array("active_v")), _p(self.array("active_w")), nx, ny, nz,
                              cp.Lx / nx, cp.Ly / ny, cp.Lz / nz)
        return out

"""ctypes bindings of the package's two C-ABI libraries.

``libibmhost.so`` — CPU setup (include/ibm_host.h).
``libibmgpu.so``  — the per-timestep solver on one GB300 (include/ibm_gpu.h).

Both are built in-tree under ``_build/`` by :mod:`build`. Loading fails loudly
when a library is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
HOST_LIB = os.path.join(BUILD_DIR, "libibmhost.so")
GPU_LIB = os.path.join(BUILD_DIR, "libibmgpu.so")


class CaseParams(C.Structure):
    """ibm_case_params (include/ibm_host.h)."""

    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
                ("rho", C.c_double), ("nu", C.c_double), ("Um", C.c_double), ("dt", C.c_double),
                ("nsub_beta", C.c_int), ("beta_tol", C.c_double), ("alpha_tol", C.c_double),
                ("xcirc", C.c_double), ("ycirc", C.c_double), ("Rcirc", C.c_double)]


class CaseCounts(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nu", "nv", "nw", "np", "nqu", "nqv", "nqw", "n_pruned")]


class GridDesc(C.Structure):
    """ibm_grid_desc (include/ibm_gpu.h)."""

    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
                ("rho", C.c_double), ("nu", C.c_double), ("dt", C.c_double),
                ("device", C.c_int)]


class SolverParams(C.Structure):
    """ibm_solver_params (include/ibm_gpu.h)."""

    _fields_ = [("vel_tol", C.c_double), ("vel_maxit", C.c_int), ("vel_kdim", C.c_int),
                ("vel_jacobi_iters", C.c_int),
                ("p_tol", C.c_double), ("p_maxit", C.c_int), ("p_kdim", C.c_int),
                ("p_pc", C.c_int), ("p_pc_maxit", C.c_int), ("p_pc_relax_type", C.c_int),
                ("p_pc_rap_type", C.c_int),
                ("mg_nu1", C.c_int), ("mg_nu2", C.c_int), ("mg_omega", C.c_double),
                ("mg_coarse_max", C.c_int), ("mg_max_levels", C.c_int),
                ("use_zero_initial_guess", C.c_int), ("precision", C.c_int), ("use_graph", C.c_int),
                ("vel_inner_sweeps", C.c_int), ("mg_group_ratio", C.c_double), ("mg_options", C.c_int),
                ("mg_nu_coarse", C.c_int), ("cycle_rtol32", C.c_double), ("compute_forces", C.c_int),
                ("row_classes", C.c_int), ("mg_quads", C.c_int),
                ("df_residual", C.c_int), ("mg_fused_coarse", C.c_int),
                ("mg_fused_sweep", C.c_int), ("vel_precision", C.c_int),
                ("df_spmv", C.c_int), ("df_rhs", C.c_int), ("arnoldi_passes", C.c_int)]


class Profile(C.Structure):
    """ibm_profile: per kernel class launches, algorithmic bytes, timed ms."""
    _fields_ = [("nkernels", C.c_int), ("launches", C.c_longlong * 32), ("bytes", C.c_double * 32),
                ("time_ms", C.c_double * 32), ("timed_launches", C.c_longlong * 32),
                ("phase_bytes", C.c_double * 5)]


class SolveStats(C.Structure):
    _fields_ = [("iters", C.c_int), ("rel_res", C.c_double), ("status", C.c_int)]


class StepStats(C.Structure):
    _fields_ = [("ramp", C.c_double), ("u", SolveStats), ("v", SolveStats), ("w", SolveStats),
                ("p", SolveStats), ("div_l2", C.c_double), ("umax", C.c_double),
                ("vmax", C.c_double), ("wmax", C.c_double),
                ("t_rhs_ms", C.c_double), ("t_mom_ms", C.c_double), ("t_p_ms", C.c_double),
                ("t_proj_ms", C.c_double), ("t_total_ms", C.c_double), ("status", C.c_int),
                ("force", C.c_double * 3)]


_host = None
_gpu = None


def _load(path: str) -> C.CDLL:
    if not os.path.exists(path):
        raise RuntimeError(f"{os.path.basename(path)} is not built: run __graft_entry__.build() "
                           "(or python -m build inside the package directory)")
    return C.CDLL(path)


def host() -> C.CDLL:
    global _host
    if _host is None:
        lib = _load(HOST_LIB)
        vp = C.c_void_p
        lib.ibm_case_params_default.argtypes = [C.POINTER(CaseParams)]
        lib.ibm_case_build.argtypes = [C.POINTER(CaseParams), C.POINTER(vp)]
        lib.ibm_case_free.argtypes = [vp]
        lib.ibm_case_get_counts.argtypes = [vp, C.POINTER(CaseCounts)]
        lib.ibm_case_array_bytes.argtypes = [vp, C.c_char_p, C.POINTER(C.c_int)]
        lib.ibm_case_array_bytes.restype = C.c_long
        lib.ibm_case_array.argtypes = [vp, C.c_char_p]
        lib.ibm_case_array.restype = vp
        lib.ibm_host_check_sum_order.argtypes = [C.c_int, C.c_uint]
        lib.ibm_write_vtk.argtypes = [C.c_char_p] + [vp] * 5 + [C.c_int] * 3 + [C.c_double] * 3
        lib.ibm_vtk_step_name.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_int]
        _host = lib
    return _host


def gpu() -> C.CDLL:
    global _gpu
    if _gpu is None:
        lib = _load(GPU_LIB)
        vp = C.c_void_p
        P = C.POINTER
        d = C.c_double
        i = C.c_int
        lib.ibm_create.argtypes = [P(GridDesc), P(vp)]
        lib.ibm_destroy.argtypes = [vp]
        lib.ibm_last_error.argtypes = [vp]
        lib.ibm_last_error.restype = C.c_char_p
        lib.ibm_set_operator.argtypes = [vp, i, vp, i, i, i]
        lib.ibm_set_masks.argtypes = [vp] + [vp] * 7 + [vp] * 7
        lib.ibm_set_aux.argtypes = [vp] + [vp] * 7 + [vp]
        lib.ibm_set_projection_csr.argtypes = [vp, vp, vp, vp, i, vp, vp, vp, i]
        lib.ibm_set_body.argtypes = [vp, d, d, d, vp, vp]
        lib.ibm_set_solver_params.argtypes = [vp, P(SolverParams)]
        lib.ibm_get_solver_params.argtypes = [vp, P(SolverParams)]
        lib.ibm_solver_params_default.argtypes = [P(SolverParams)]
        lib.ibm_set_fields.argtypes = [vp, vp, vp, vp, vp]
        lib.ibm_get_fields.argtypes = [vp, vp, vp, vp, vp]
        lib.ibm_step.argtypes = [vp, d, P(StepStats)]
        lib.ibm_solve.argtypes = [vp, i, vp, vp, P(SolveStats)]
        lib.ibm_apply_operator.argtypes = [vp, i, vp, vp]
        lib.ibm_get_solver_vector.argtypes = [vp, i, i, vp]
        lib.ibm_apply_preconditioner.argtypes = [vp, i, vp, vp]
        lib.ibm_profile_reset.argtypes = [vp]
        lib.ibm_profile_time_kernel.argtypes = [vp, i]
        lib.ibm_profile_get.argtypes = [vp, P(Profile)]
        lib.ibm_batch_create.argtypes = [i, P(GridDesc), P(vp)]
        lib.ibm_batch_destroy.argtypes = [vp]
        lib.ibm_batch_size.argtypes = [vp]
        lib.ibm_batch_ctx.argtypes = [vp, i]
        lib.ibm_batch_ctx.restype = vp
        lib.ibm_batch_step.argtypes = [vp, P(d), P(StepStats)]
        lib.ibm_kernel_name.argtypes = [i]
        lib.ibm_kernel_name.restype = C.c_char_p
        lib.ibm_synchronize.argtypes = [vp]
        lib.ibm_stream.argtypes = [vp]
        lib.ibm_stream.restype = vp
        lib.ibm_kernel_launches.argtypes = [vp]
        lib.ibm_kernel_launches.restype = C.c_longlong
        lib.ibm_device_query.argtypes = [i, C.c_char_p, i]
        lib.ibm_assemble_momentum.argtypes = [vp, d, d, d, vp * 3, vp * 3, vp * 3, vp * 3]
        lib.ibm_assemble_pressure.argtypes = [vp, vp, vp, vp, vp * 3, vp * 3, vp * 3, vp]
        lib.ibm_adjoint_setup.argtypes = [vp, vp]
        lib.ibm_set_inflow.argtypes = [vp, vp]
        lib.ibm_step_forward.argtypes = [vp, d, P(StepStats)]
        lib.ibm_step_backward.argtypes = [vp, d, d, P(StepStats)]
        lib.ibm_adjoint_reset.argtypes = [vp]
        lib.ibm_adjoint_set.argtypes = [vp, vp, vp, vp, vp]
        lib.ibm_adjoint_get.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        lib.ibm_adjoint_tape_depth.argtypes = [vp]
        lib.ibm_adjoint_solve_stats.argtypes = [vp, P(SolveStats)]
        lib.ibm_checkpoint_save.argtypes = [vp, i]
        lib.ibm_checkpoint_load.argtypes = [vp, i]
        lib.ibm_checkpoint_clear.argtypes = [vp]
        _gpu = lib
    return _gpu

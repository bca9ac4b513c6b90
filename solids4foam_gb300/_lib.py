"""ctypes binding of libs4g.so (the C ABI declared in include/s4g.h).

The library is built in-tree by solids4foam_gb300/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback for the solver.
"""
from __future__ import annotations

import ctypes as ct
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libs4g.so")

# s4g_status
OK, BAD_ARG, OOM, NOT_CONVERGED, NAN_DETECTED, INDEFINITE, TIMEOUT, CUDA_ERROR, NO_DEVICE, \
    ADMISSION_REJECTED, PENDING, CANCELLED, NOT_BUILT = range(13)
# enums
RENUMBER_NONE, RENUMBER_RCM, RENUMBER_TILED = 0, 1, 2
LINEAR_ELASTIC, NEO_HOOKEAN = 0, 1
FIXED_DISPLACEMENT, SOLID_TRACTION = 0, 1
PRECOND_DIC, PRECOND_DIAGONAL = 0, 1
FP64, FP32_REFINE = 0, 1
LIN_GEOM_TOTAL_DISP, NONLIN_GEOM_TOTAL_LAG, NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP = 0, 1, 2


class CtxOpts(ct.Structure):
    _fields_ = [("device", ct.c_int), ("verbose", ct.c_int), ("profile", ct.c_int),
                ("no_graphs", ct.c_int), ("spin_limit", ct.c_int)]


# kernel kinds of the per-kernel timers (S4G_K_*)
KERNEL_KINDS = ("rhs", "post", "sweep_fwd", "sweep_bwd", "diag", "p_update", "spmv", "update",
                "loc_precond", "loc_spmv")


class MeshDesc(ct.Structure):
    _fields_ = [
        ("n_cells", ct.c_int), ("n_faces", ct.c_int), ("n_internal_faces", ct.c_int),
        ("owner", ct.c_void_p), ("neighbour", ct.c_void_p),
        ("C", ct.c_void_p), ("V", ct.c_void_p), ("Cf", ct.c_void_p), ("Sf", ct.c_void_p),
        ("n_patches", ct.c_int), ("patch_start", ct.c_void_p), ("patch_size", ct.c_void_p),
    ]


class MeshOpts(ct.Structure):
    _fields_ = [("renumber", ct.c_int), ("part_size", ct.c_int),
                ("ls_boundary_delta", ct.c_int), ("dic_subdomains", ct.c_int),
                ("no_autotune", ct.c_int), ("empty_direction", ct.c_int),
                ("part_of_cell", ct.c_void_p)]


class MeshInfo(ct.Structure):
    _fields_ = [("n_cells", ct.c_int), ("n_internal_faces", ct.c_int),
                ("n_boundary_faces", ct.c_int), ("n_parts", ct.c_int),
                ("part_depth", ct.c_int), ("max_local_levels", ct.c_int),
                ("n_levels_global", ct.c_int), ("device_bytes", ct.c_longlong),
                ("n_local_entries", ct.c_longlong), ("local_slots", ct.c_int)]


class Law(ct.Structure):
    _fields_ = [("type", ct.c_int), ("use_mu_K", ct.c_int), ("E", ct.c_double),
                ("nu", ct.c_double), ("mu", ct.c_double), ("K", ct.c_double),
                ("rho", ct.c_double)]


class LinSolver(ct.Structure):
    _fields_ = [("preconditioner", ct.c_int), ("tolerance", ct.c_double),
                ("rel_tol", ct.c_double), ("max_iter", ct.c_int)]


class Outer(ct.Structure):
    _fields_ = [("n_correctors", ct.c_int), ("solution_tol", ct.c_double),
                ("alternative_tol", ct.c_double), ("material_tol", ct.c_double),
                ("stab_scale", ct.c_double), ("info_frequency", ct.c_int),
                ("field_relaxation", ct.c_double), ("relaxation_method", ct.c_int)]


class ServerOpts(ct.Structure):
    _fields_ = [("device", ct.c_int), ("max_slots", ct.c_int), ("memory_budget", ct.c_longlong),
                ("dry_run", ct.c_int), ("dry_run_us_per_kcell", ct.c_double)]


class Request(ct.Structure):
    _fields_ = [("mesh", ct.c_void_p), ("mesh_opts", MeshOpts), ("law", Law), ("n_bc", ct.c_int),
                ("bc_patch", ct.c_void_p), ("bc_type", ct.c_void_p), ("bc_vec3", ct.c_void_p),
                ("bc_pressure", ct.c_void_p), ("lin", LinSolver), ("outer", Outer),
                ("precision", ct.c_int), ("model", ct.c_int), ("n_increments", ct.c_int),
                ("bc_relaxation", ct.c_void_p)]


class ServerStats(ct.Structure):
    _fields_ = [("submitted", ct.c_longlong), ("completed", ct.c_longlong),
                ("rejected", ct.c_longlong), ("cancelled", ct.c_longlong),
                ("running", ct.c_int), ("queued", ct.c_int),
                ("bytes_in_use", ct.c_longlong), ("memory_budget", ct.c_longlong),
                ("p50_ms", ct.c_double), ("p99_ms", ct.c_double), ("mean_ms", ct.c_double),
                ("solves_per_s", ct.c_double)]


class Perf(ct.Structure):
    _fields_ = [
        ("n_correctors", ct.c_int), ("converged", ct.c_int),
        ("total_lin_iters", ct.c_longlong), ("last_max_lin_iters", ct.c_int),
        ("initial_residual", ct.c_double), ("rel_residual", ct.c_double),
        ("solve_ms", ct.c_double), ("h2d_ms", ct.c_double), ("d2h_ms", ct.c_double),
        ("kernel_launches", ct.c_longlong), ("enforce_linear", ct.c_int),
        ("device_status", ct.c_int), ("part_threads", ct.c_int), ("spmv_unroll", ct.c_int),
        ("tune_us", ct.c_double * 6),
        ("kernel_ms", ct.c_double * len(KERNEL_KINDS)),
        ("kernel_launches_by", ct.c_longlong * len(KERNEL_KINDS)),
        ("device_loop", ct.c_int),
    ]

    def as_dict(self):
        d = {f[0]: getattr(self, f[0]) for f in self._fields_[:-3]}
        d["device_loop"] = self.device_loop
        d["tune_us"] = list(self.tune_us)
        d["kernel_ms"] = dict(zip(KERNEL_KINDS, list(self.kernel_ms)))
        d["kernel_launches_by"] = dict(zip(KERNEL_KINDS, list(self.kernel_launches_by)))
        return d


# every symbol declared in include/s4g.h, with its ctypes signature
_SIGS = {
    "s4g_status_str": (ct.c_char_p, [ct.c_int]),
    "s4g_abi_version": (ct.c_int, []),
    "s4g_last_error": (ct.c_char_p, []),
    "s4g_ctx_create": (ct.c_int, [ct.POINTER(ct.c_void_p), ct.POINTER(CtxOpts)]),
    "s4g_ctx_destroy": (ct.c_int, [ct.c_void_p]),
    "s4g_mesh_upload": (ct.c_int, [ct.c_void_p, ct.POINTER(MeshDesc), ct.POINTER(MeshOpts),
                                   ct.POINTER(ct.c_void_p)]),
    "s4g_mesh_plan": (ct.c_int, [ct.POINTER(MeshDesc), ct.POINTER(MeshOpts), ct.c_void_p,
                                 ct.POINTER(MeshInfo)]),
    "s4g_mesh_get_permutation": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "s4g_mesh_get_parts": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "s4g_mesh_get_info": (ct.c_int, [ct.c_void_p, ct.POINTER(MeshInfo)]),
    "s4g_mesh_destroy": (ct.c_int, [ct.c_void_p]),
    "s4g_material_set": (ct.c_int, [ct.c_void_p, ct.POINTER(Law)]),
    "s4g_bc_set": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p]),
    "s4g_bc_set_relaxation": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_double]),
    "s4g_solver_set": (ct.c_int, [ct.c_void_p, ct.POINTER(LinSolver), ct.POINTER(Outer), ct.c_int]),
    "s4g_default_controls": (None, [ct.POINTER(LinSolver), ct.POINTER(Outer)]),
    "s4g_solve": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p,
                             ct.POINTER(Perf)]),
    "s4g_solve_step": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p,
                                  ct.POINTER(Perf)]),
    "s4g_state_reset": (ct.c_int, [ct.c_void_p]),
    "s4g_get_gradD": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "s4g_solve_batch": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "s4g_mesh_set_points": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p,
                                       ct.c_void_p]),
    "s4g_get_pointD": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "s4g_op_matrix": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "s4g_server_create": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "s4g_server_submit": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.POINTER(ct.c_uint64)]),
    "s4g_server_poll": (ct.c_int, [ct.c_void_p, ct.c_uint64, ct.c_int, ct.c_void_p, ct.c_void_p,
                                   ct.c_void_p]),
    "s4g_server_cancel": (ct.c_int, [ct.c_void_p, ct.c_uint64]),
    "s4g_server_get_stats": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "s4g_server_destroy": (ct.c_int, [ct.c_void_p]),
    "s4g_solve_cases": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p,
                                   ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "s4g_op_amul": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p]),
    "s4g_op_amul_dot_noalloc": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p,
                                           ct.c_void_p]),
    "s4g_op_precondition": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p]),
    "s4g_box_mesh_sizes": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int] + [ct.POINTER(ct.c_int)] * 4),
    "s4g_box_mesh_build": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int, ct.c_double, ct.c_double,
                                      ct.c_double, ct.c_double, ct.c_uint64] + [ct.c_void_p] * 9),
    "s4g_box_mesh_faces": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p]),
    "s4g_point_cells": (ct.c_int, [ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int,
                                   ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "s4g_point_interpolate": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                         ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                         ct.c_void_p]),
    "s4g_derived_fields": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                      ct.c_void_p, ct.c_void_p]),
    "s4g_traction_sngrad": (ct.c_int, [ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                       ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_double,
                                       ct.c_void_p]),
    "s4g_foam_read_mesh": (ct.c_int, [ct.c_char_p, ct.POINTER(ct.c_void_p)]),
    "s4g_foam_mesh_desc": (ct.c_int, [ct.c_void_p, ct.POINTER(MeshDesc), ct.POINTER(ct.c_int)]),
    "s4g_foam_mesh_points": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_void_p),
                                        ct.POINTER(ct.c_void_p), ct.POINTER(ct.c_void_p)]),
    "s4g_foam_patch_name": (ct.c_char_p, [ct.c_void_p, ct.c_int]),
    "s4g_foam_patch_type": (ct.c_char_p, [ct.c_void_p, ct.c_int]),
    "s4g_foam_read_d": (ct.c_int, [ct.c_void_p, ct.c_char_p]),
    "s4g_foam_bc": (ct.c_int, [ct.c_void_p, ct.c_int, ct.POINTER(ct.c_int),
                               ct.POINTER(ct.c_void_p), ct.POINTER(ct.c_void_p),
                               ct.POINTER(ct.c_double)]),
    "s4g_foam_apply_bcs": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "s4g_foam_load_ramp": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_double),
                                      ct.POINTER(ct.c_int)]),
    "s4g_foam_read_time": (ct.c_int, [ct.c_char_p] + [ct.POINTER(ct.c_double)] * 3),
    "s4g_foam_series_kind": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_int)]),
    "s4g_foam_bc_at": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_double, ct.POINTER(ct.c_int),
                                  ct.c_void_p, ct.c_void_p, ct.POINTER(ct.c_double)]),
    "s4g_foam_apply_bcs_at": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_double]),
    "s4g_foam_read_relaxation": (ct.c_int, [ct.c_char_p, ct.c_char_p, ct.POINTER(ct.c_double),
                                            ct.POINTER(ct.c_double)]),
    "s4g_foam_read_grad_scheme": (ct.c_int, [ct.c_char_p, ct.c_char_p, ct.POINTER(ct.c_int)]),
    "s4g_foam_read_controls": (ct.c_int, [ct.c_char_p, ct.POINTER(ct.c_int), ct.POINTER(Law),
                                          ct.POINTER(LinSolver), ct.POINTER(Outer)]),
    "s4g_foam_free": (None, [ct.c_void_p]),
    "s4g_foam_boundary_D": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "s4g_foam_write_field": (ct.c_int, [ct.c_void_p, ct.c_char_p, ct.c_char_p, ct.c_int,
                                        ct.c_char_p, ct.c_void_p, ct.c_void_p]),
    "s4g_foam_write_mesh": (ct.c_int, [ct.c_char_p, ct.c_int, ct.c_void_p, ct.c_int, ct.c_void_p,
                                       ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int,
                                       ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "s4g_foam_empty_direction": (ct.c_int, [ct.c_void_p]),
    "s4g_foam_write_point_field": (ct.c_int, [ct.c_void_p, ct.c_char_p, ct.c_char_p, ct.c_char_p,
                                              ct.c_void_p]),
}

_lib = None


class S4GError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = lib().s4g_last_error().decode(errors="replace")
        name = lib().s4g_status_str(status).decode()
        super().__init__(f"{where}: {name} ({msg})")


def lib():
    """Loads libs4g.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
                f"g.build()\"` (or solids4foam_gb300/build.py); the solver has no CPU fallback")
        _lib = ct.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def check(status: int, where: str, allow=(OK,)):
    if status not in allow:
        raise S4GError(status, where)
    return status


def declared_symbols():
    return list(_SIGS)

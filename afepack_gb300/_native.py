"""ctypes binding of libafepack_gb300.so (the C ABI in include/afepack_gb300.h).

The library is loaded from the package's ``_lib`` directory; it is built by
``afepack_gb300.build`` (``__graft_entry__.build()``).  There is no fallback:
if the library is missing or cannot run, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB

c_i32p = C.POINTER(C.c_int32)
c_i64p = C.POINTER(C.c_int64)
c_f64p = C.POINTER(C.c_double)
c_void_pp = C.POINTER(C.c_void_p)

AFP_PRECISION_FP64 = 0
AFP_PRECISION_MIXED = 1
AFP_ERR_INVALID = 1
AFP_ERR_NOT_CONVERGED = 5
AFP_ERR_BREAKDOWN = 6
AFP_ERR_TIMEOUT = 8


class AFPError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where}: status {status} ({message})")


class AssembleOpts(C.Structure):
    _fields_ = [("acc_stiff", C.c_int), ("acc_mass", C.c_int), ("coef", c_f64p)]


class AMGOpts(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("smooth_step", C.c_int), ("max_coarse", C.c_int),
                ("min_density", C.c_double), ("alpha", C.c_double), ("precision", C.c_int),
                ("dense_tail", C.c_int), ("max_colors", C.c_int), ("symmetric", C.c_int),
                ("coarse_colors", C.c_int), ("interp_bf16", C.c_int),
                ("fused_vcycle", C.c_int), ("wait_limit_s", C.c_double), ("inject_barrier_stall", C.c_int), ("gpu_coarsen", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("initial_residual", C.c_double),
                ("final_residual", C.c_double), ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerOpts(C.Structure):
    _fields_ = [("workers", C.c_int), ("hbm_budget_bytes", C.c_int64), ("precision", C.c_int), ("tol", C.c_double),
                ("maxit", C.c_int), ("dense_tail", C.c_int)]


class Request(C.Structure):
    _fields_ = [("dim", C.c_int), ("degree", C.c_int), ("acc_stiff", C.c_int), ("acc_mass", C.c_int),
                ("n_vertex", C.c_int64), ("coords", C.c_void_p), ("n_cell", C.c_int64), ("cells", C.c_void_p),
                ("n_dof", C.c_int64), ("elem_dof", C.c_void_p), ("dirichlet", C.c_void_p), ("coef", C.c_void_p),
                ("f", C.c_void_p)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("rel_residual", C.c_double),
                ("queue_seconds", C.c_double), ("setup_seconds", C.c_double), ("latency_seconds", C.c_double),
                ("device_seconds", C.c_double), ("estimate_bytes", C.c_int64), ("measured_bytes", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchOpts(C.Structure):
    _fields_ = [("width", C.c_int), ("tol", C.c_double), ("maxit", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("failed", C.c_int64), ("queued", C.c_int64), ("p50_seconds", C.c_double),
                ("p99_seconds", C.c_double), ("solves_per_second", C.c_double), ("budget_bytes", C.c_int64),
                ("in_use_bytes", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# (name, argtypes) of every exported entry point; the restype is afp_status
# (c_int) unless noted in _RESTYPES.
SIGNATURES = {
    "afp_version": [],
    "afp_status_string": [C.c_int],
    "afp_last_error": [],
    "afp_context_create": [C.c_int, c_void_pp],
    "afp_context_destroy": [C.c_void_p],
    "afp_context_synchronize": [C.c_void_p],
    "afp_context_launch_count": [C.c_void_p, c_i64p],
    "afp_context_stream": [C.c_void_p, c_void_pp],
    "afp_space_create": [C.c_void_p, C.c_int, C.c_int, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                         C.c_void_p, c_void_pp],
    "afp_space_create_numbered": [C.c_void_p, C.c_int, C.c_int, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                  C.c_void_p, C.c_void_p],
    "afp_space_info": [C.c_void_p, C.c_void_p, C.c_void_p],
    "afp_space_download_dofs": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "afp_quadrature_points": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "afp_l2_discretize": [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_void_p],
    "afp_space_destroy": [C.c_void_p],
    "afp_assemble": [C.c_void_p, C.POINTER(AssembleOpts), c_void_pp, c_void_pp],
    "afp_matrix_create_csr": [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                              c_void_pp],
    "afp_matrix_info": [C.c_void_p, c_i64p, c_i64p, c_i64p],
    "afp_matrix_set_values": [C.c_void_p, C.c_void_p],
    "afp_matrix_download": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
    "afp_matrix_vmult": [C.c_void_p, C.c_void_p, C.c_void_p],
    "afp_matrix_vmult_noalloc": [C.c_void_p, C.c_void_p, C.c_void_p],
    "afp_matrix_destroy": [C.c_void_p],
    "afp_apply_dirichlet": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int],
    "afp_amg_default_opts": [C.POINTER(AMGOpts)],
    "afp_amg_setup": [C.c_void_p, C.POINTER(AMGOpts), c_void_pp],
    "afp_amg_setup_lazy": [C.c_void_p, C.POINTER(AMGOpts), c_void_pp],
    "afp_amg_lazy_reinit": [C.c_void_p, C.c_void_p],
    "afp_amg_destroy": [C.c_void_p],
    "afp_amg_num_levels": [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "afp_amg_level_info": [C.c_void_p, C.c_int, c_i64p, c_i64p, C.POINTER(C.c_int)],
    "afp_amg_download_level": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p],
    "afp_amg_download_projection": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p],
    "afp_amg_solve": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int64, C.c_int, C.POINTER(SolveInfo)],
    "afp_amg_precondition": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int],
    "afp_amg_time_kernel": [C.c_void_p, C.c_int, C.c_int, C.c_int, c_f64p, c_f64p],
    "afp_pcg_solve": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.POINTER(SolveInfo)],
    "afp_pcg_solve_multi": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int,
                            C.POINTER(SolveInfo)],
    "afp_host_coarsen": [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, c_i64p,
                         C.POINTER(c_i32p), C.POINTER(c_i32p), C.POINTER(c_f64p)],
    "afp_host_free": [C.c_void_p],
    "afp_server_default_opts": [C.POINTER(ServerOpts)],
    "afp_server_create": [C.c_int, C.POINTER(ServerOpts), c_void_pp],
    "afp_server_submit": [C.c_void_p, C.POINTER(Request), c_i64p],
    "afp_server_wait": [C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(RequestResult)],
    "afp_server_poll": [C.c_void_p, C.c_int64, C.POINTER(C.c_int)],
    "afp_server_get_stats": [C.c_void_p, C.POINTER(ServerStats)],
    "afp_server_reset_stats": [C.c_void_p],
    "afp_server_destroy": [C.c_void_p],
    "afp_batch_default_opts": [C.POINTER(BatchOpts)],
    "afp_batch_server_create": [C.c_void_p, C.POINTER(BatchOpts), c_void_pp],
    "afp_batch_server_submit": [C.c_void_p, C.c_void_p, c_i64p],
    "afp_batch_server_wait": [C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(RequestResult)],
    "afp_batch_server_get_stats": [C.c_void_p, C.POINTER(ServerStats)],
    "afp_batch_server_reset_stats": [C.c_void_p],
    "afp_batch_server_destroy": [C.c_void_p],
}
_RESTYPES = {"afp_version": C.c_int, "afp_status_string": C.c_char_p, "afp_last_error": C.c_char_p,
             "afp_amg_default_opts": None, "afp_host_free": None, "afp_server_default_opts": None,
             "afp_batch_default_opts": None}

_lib = None


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} is missing: build it with `python -m afepack_gb300.build`")
        L = C.CDLL(LIB)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPES.get(name, C.c_int)
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != 0:
        msg = lib().afp_last_error()
        raise AFPError(status, where, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args), name)


def ptr(a, dtype=None):
    """Address of a numpy array or of a CUDA torch tensor (no copy)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if dtype is not None:
        assert a.dtype == dtype, f"expected {dtype}, got {a.dtype}"
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)

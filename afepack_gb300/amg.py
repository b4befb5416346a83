"""Python mirror of AFEPack's AMGSolver / AMGPreconditioner over the C ABI.

Constructor arguments and methods follow include/AFEPack/AMGSolver.h:67-196:
``AMGSolver(M, tol=1e-12, s=3, nmpo=50, nmpsd=0.382, alp=0.25)``,
``reinit(M)``, ``solve(x, r, tol=0.0, step=20, mode=0)`` (step+1 V-cycles),
``tolerence()``, ``smoothStep()``; ``AMGPreconditioner(M, is=5, s=3).vmult(x, b)``.
The GB300 options (precision, dense tail, colour cap, symmetric smoothing)
are keyword-only.  ``pcg`` is the outer preconditioned CG of the reference's
example solvers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .fem import SparseMatrix

FP64 = N.AFP_PRECISION_FP64
MIXED = N.AFP_PRECISION_MIXED


def default_opts() -> N.AMGOpts:
    o = N.AMGOpts()
    N.lib().afp_amg_default_opts(C.byref(o))
    return o


class AMGSolver:
    def __init__(self, M: SparseMatrix | None = None, tol: float = 1.0e-12, s: int = 3, nmpo: int = 50,
                 nmpsd: float = 0.382, alp: float = 0.25, *, precision: int = FP64, dense_tail: int | None = None,
                 max_colors: int | None = None, symmetric: bool = True, coarse_colors: int | None = None,
                 interp_bf16: bool | None = None, fused_vcycle: bool | None = None, gpu_coarsen: bool | None = None):
        self.opts = default_opts()
        self.opts.tolerance = tol
        self.opts.smooth_step = s
        self.opts.max_coarse = nmpo
        self.opts.min_density = nmpsd
        self.opts.alpha = alp
        self.opts.precision = precision
        if dense_tail is not None:
            self.opts.dense_tail = dense_tail
        if max_colors is not None:
            self.opts.max_colors = max_colors
        self.opts.symmetric = int(symmetric)
        if coarse_colors is not None:
            self.opts.coarse_colors = coarse_colors
        if interp_bf16 is not None:
            self.opts.interp_bf16 = int(interp_bf16)
        if fused_vcycle is not None:
            self.opts.fused_vcycle = int(fused_vcycle)
        if gpu_coarsen is not None:
            self.opts.gpu_coarsen = int(gpu_coarsen)
        self.handle = None
        self.matrix = None
        if M is not None:
            self.reinit(M)

    # accessors of the reference
    def tolerence(self):
        return self.opts.tolerance

    def smoothStep(self):
        return self.opts.smooth_step

    def reinit(self, M: SparseMatrix):
        self.clear()
        h = C.c_void_p()
        N.call("afp_amg_setup", M.handle, C.byref(self.opts), C.byref(h))
        self.handle = h
        self.matrix = M

    def clear(self):
        if self.handle:
            N.lib().afp_amg_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass

    # hierarchy inspection
    def n_project(self) -> int:
        a, b = C.c_int(), C.c_int()
        N.call("afp_amg_num_levels", self.handle, C.byref(a), C.byref(b))
        return a.value

    def solve_levels(self) -> int:
        a, b = C.c_int(), C.c_int()
        N.call("afp_amg_num_levels", self.handle, C.byref(a), C.byref(b))
        return b.value

    def level_info(self, level: int):
        n, nnz, colors = C.c_int64(), C.c_int64(), C.c_int()
        N.call("afp_amg_level_info", self.handle, level, C.byref(n), C.byref(nnz), C.byref(colors))
        return n.value, nnz.value, colors.value

    def level_matrix(self, level: int):
        """Galerkin matrix of a level (0 = fine) in the reference's layout."""
        n = self.level_info(level)[0]
        rp = np.empty(n + 1, dtype=np.int32)
        N.call("afp_amg_download_level", self.handle, level, N.ptr(rp), None, None)
        ci = np.empty(int(rp[-1]), dtype=np.int32)
        va = np.empty(int(rp[-1]))
        N.call("afp_amg_download_level", self.handle, level, None, N.ptr(ci), N.ptr(va))
        return rp, ci, va

    def projection(self, level: int):
        """P_level (n_{level+1} x n_level) in the reference's layout."""
        n_c = self.level_info(level + 1)[0]
        rp = np.empty(n_c + 1, dtype=np.int32)
        N.call("afp_amg_download_projection", self.handle, level, N.ptr(rp), None, None)
        ci = np.empty(int(rp[-1]), dtype=np.int32)
        va = np.empty(int(rp[-1]))
        N.call("afp_amg_download_projection", self.handle, level, None, N.ptr(ci), N.ptr(va))
        return rp, ci, va

    def time_kernel(self, kind: int, level: int = 0, reps: int = 20):
        """(mean ms, algorithmic bytes) of one unit: 0 GS sweep, 1 residual,
        2 V-cycle, 3 FP64 fine SpMV (CUDA events on the library stream)."""
        ms, nb = C.c_double(), C.c_double()
        N.call("afp_amg_time_kernel", self.handle, kind, level, reps, C.byref(ms), C.byref(nb))
        return ms.value, nb.value

    # solving
    def solve(self, x, r, tol: float = 0.0, step: int = 20, mode: int = 0):
        """step+1 V-cycles from x, in place (AMGSolver::solve)."""
        info = N.SolveInfo()
        N.call("afp_amg_solve", self.handle, N.ptr(x), N.ptr(r), tol, step, mode, C.byref(info))
        return info.as_dict()

    def pcg(self, b, tol: float = 1e-10, maxit: int = 500, x=None):
        """CG preconditioned by one V-cycle per iteration; returns (x, info)."""
        if x is None:
            if hasattr(b, "data_ptr"):
                import torch
                x = torch.zeros_like(b)
            else:
                x = np.zeros_like(np.asarray(b, dtype=np.float64))
        if not hasattr(b, "data_ptr"):
            b = np.ascontiguousarray(b, dtype=np.float64)
        info = N.SolveInfo()
        st = N.lib().afp_pcg_solve(self.handle, N.ptr(x), N.ptr(b), tol, maxit, C.byref(info))
        if st != N.AFP_ERR_NOT_CONVERGED:  # the iteration limit is reported in info, as the reference prints it
            N.check(st, "afp_pcg_solve")
        return x, info.as_dict()

    def pcg_multi(self, B, tol: float = 1e-8, maxit: int = 500, X=None):
        """nrhs systems at once; B is n x nrhs row-major."""
        nrhs = B.shape[1]
        if X is None:
            if hasattr(B, "data_ptr"):
                import torch
                X = torch.zeros_like(B)
            else:
                X = np.zeros_like(np.asarray(B, dtype=np.float64))
        if not hasattr(B, "data_ptr"):
            B = np.ascontiguousarray(B, dtype=np.float64)
        infos = (N.SolveInfo * nrhs)()
        st = N.lib().afp_pcg_solve_multi(self.handle, N.ptr(X), N.ptr(B), nrhs, tol, maxit, infos)
        if st != N.AFP_ERR_NOT_CONVERGED:
            N.check(st, "afp_pcg_solve_multi")
        return X, [i.as_dict() for i in infos]


    def lazyReinit(self, M: SparseMatrix):
        """AMGSolver::lazyReinit: the lazyProject hierarchy on first use, then
        numeric re-setup for new values on the same pattern."""
        if self.handle is None:
            h = C.c_void_p()
            N.call("afp_amg_setup_lazy", M.handle, C.byref(self.opts), C.byref(h))
            self.handle = h
        else:
            N.call("afp_amg_lazy_reinit", self.handle, M.handle)
        self.matrix = M


class AMGPreconditioner(AMGSolver):
    """AMGPreconditioner(M, is=5, s=3): lazy hierarchy; vmult(x, b) runs is+1 V-cycles from x."""

    def __init__(self, M: SparseMatrix | None = None, iterate_step: int = 5, s: int = 3, **kw):
        self.iterate_step = iterate_step
        super().__init__(None, s=s, **kw)
        if M is not None:
            self.lazyReinit(M)

    def reinit(self, M: SparseMatrix, iterate_step: int = 5):
        self.lazyReinit(M)
        self.iterate_step = iterate_step

    def vmult(self, x, b):
        N.call("afp_amg_precondition", self.handle, N.ptr(x), N.ptr(b), self.iterate_step)


def host_coarsen(rowptr, cols, vals, alpha: float = 0.25):
    """Project() on the host through the C ABI: (cf flags, P rowptr, cols, vals)."""
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    m = rowptr.shape[0] - 1
    cf = np.empty(m, dtype=np.int32)
    nc = C.c_int64()
    prp, pci, pva = N.c_i32p(), N.c_i32p(), N.c_f64p()
    N.call("afp_host_coarsen", m, N.ptr(rowptr), N.ptr(cols), N.ptr(vals), alpha, N.ptr(cf), C.byref(nc),
           C.byref(prp), C.byref(pci), C.byref(pva))
    n_c = nc.value
    rp = np.ctypeslib.as_array(prp, (n_c + 1,)).copy()
    nnz = int(rp[-1])
    ci = np.ctypeslib.as_array(pci, (max(nnz, 1),))[:nnz].copy()
    va = np.ctypeslib.as_array(pva, (max(nnz, 1),))[:nnz].copy()
    for p in (prp, pci, pva):
        N.lib().afp_host_free(C.cast(p, C.c_void_p))
    return cf, rp, ci, va

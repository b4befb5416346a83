"""ctypes front end of the CPU oracle (oracle/afp_oracle.c) -- TEST INFRASTRUCTURE.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; it is the checker, never the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_i64p = C.POINTER(C.c_int64)
_f64p = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)


class _CSR(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("rowptr", _i64p), ("cols", _i64p), ("vals", _f64p)]


class _AMG(C.Structure):
    _fields_ = [("n_level", C.c_int), ("most_project_full", C.c_int), ("A", C.POINTER(_CSR)),
                ("P", C.POINTER(_CSR)), ("n_coarse", C.c_int64), ("coarse_inv", _f64p),
                ("smooth_step", C.c_int), ("alpha", C.c_double), ("Pt", C.POINTER(_CSR))]


def build() -> str:
    """Compile liboracle.so with gcc (a second or two)."""
    src = os.path.join(HERE, "afp_oracle.c")
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "afp_oracle.h"))):
        base = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"]
        if subprocess.run(base + ["-fopenmp"], capture_output=True).returncode != 0:
            subprocess.check_call(base)  # serial build where OpenMP is unavailable
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.orc_assemble.argtypes = [C.c_int, C.c_int, _f64p, C.c_int64, _i64p, _i32p, C.c_int64, C.c_int,
                                      C.c_int, _f64p, C.POINTER(_CSR), _f64p]
        _lib.orc_vmult.argtypes = [C.POINTER(_CSR), _f64p, _f64p]
        _lib.orc_apply_dirichlet.argtypes = [C.POINTER(_CSR), _f64p, _i32p, _f64p]
        _lib.orc_amg_setup.argtypes = [C.POINTER(_CSR), C.c_int, C.c_int64, C.c_double, C.c_double,
                                       C.POINTER(_AMG)]
        _lib.orc_amg_free.argtypes = [C.POINTER(_AMG)]
        _lib.orc_amg_from_levels.argtypes = [C.c_int, C.POINTER(_CSR), C.POINTER(_CSR), C.c_int, C.c_int,
                                             C.POINTER(_AMG)]
        _lib.orc_amg_set_coarse_inverse.argtypes = [C.POINTER(_AMG), _f64p]
        _lib.orc_project.argtypes = [C.POINTER(_CSR), C.c_double, C.POINTER(_CSR), _i32p]
        _lib.orc_rap.argtypes = [C.POINTER(_CSR), C.POINTER(_CSR), C.POINTER(_CSR)]
        _lib.orc_amg_vcycles.argtypes = [C.POINTER(_AMG), _f64p, _f64p, C.c_int]
        _lib.orc_pcg.argtypes = [C.POINTER(_CSR), C.POINTER(_AMG), _f64p, _f64p, C.c_double, C.c_int, _f64p]
        _lib.orc_pcg.restype = C.c_int
        _lib.orc_csr_free.argtypes = [C.POINTER(_CSR)]
        _lib.orc_amg_setup_lazy.argtypes = [C.POINTER(_CSR), C.c_int, C.c_int64, C.c_double, C.POINTER(_AMG)]
        _lib.orc_amg_lazy_reinit.argtypes = [C.POINTER(_AMG), C.POINTER(_CSR)]
        _lib.orc_quadrature_points.argtypes = [C.c_int, _f64p, C.c_int64, _i64p, C.c_int, _f64p]
        _lib.orc_l2_discretize.argtypes = [C.c_int, C.c_int, _f64p, C.c_int64, _i64p, _i32p, C.c_int64, C.c_int,
                                           _f64p, _f64p, _f64p]
    return _lib


def _ptr(a, t):
    return a.ctypes.data_as(t)


class CSR:
    """Host CSR in the reference layout (int64 rowptr/cols, float64 vals)."""

    def __init__(self, rowptr, cols, vals, shape):
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        self.cols = np.ascontiguousarray(cols, dtype=np.int64)
        self.vals = np.ascontiguousarray(vals, dtype=np.float64)
        self.shape = tuple(int(s) for s in shape)

    @classmethod
    def _from_c(cls, c: _CSR):
        m = c.m
        nnz = c.rowptr[m]
        out = cls(np.ctypeslib.as_array(c.rowptr, (m + 1,)).copy(),
                  np.ctypeslib.as_array(c.cols, (max(nnz, 1),))[:nnz].copy(),
                  np.ctypeslib.as_array(c.vals, (max(nnz, 1),))[:nnz].copy(), (m, c.n))
        return out

    def _c(self) -> _CSR:
        return _CSR(self.shape[0], self.shape[1], _ptr(self.rowptr, _i64p), _ptr(self.cols, _i64p),
                    _ptr(self.vals, _f64p))

    @property
    def nnz(self):
        return int(self.rowptr[-1])

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.shape[0])
        c = self._c()
        lib().orc_vmult(C.byref(c), _ptr(x, _f64p), _ptr(y, _f64p))
        return y

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.vals, self.cols, self.rowptr), shape=self.shape)


def assemble(space, acc_stiff, acc_mass, coef=None):
    """(stiffness CSR, mass values in the same pattern) of a FESpace."""
    mesh = space.mesh
    coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    cells = np.ascontiguousarray(mesh.cells, dtype=np.int64)
    ed = np.ascontiguousarray(space.elem_dof, dtype=np.int32)
    out = _CSR()
    nnz_guess = None
    cf = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
    # first pass gives the pattern; mass values need the nnz, so assemble twice
    rc = lib().orc_assemble(mesh.dim, space.degree, _ptr(coords, _f64p), mesh.n_cell, _ptr(cells, _i64p),
                            _ptr(ed, _i32p), space.n_dof, acc_stiff, acc_mass,
                            None if cf is None else _ptr(cf, _f64p), C.byref(out), None)
    if rc != 0:
        raise RuntimeError(f"orc_assemble failed ({rc})")
    K = CSR._from_c(out)
    lib().orc_csr_free(C.byref(out))
    mass = np.empty(K.nnz)
    out = _CSR()
    rc = lib().orc_assemble(mesh.dim, space.degree, _ptr(coords, _f64p), mesh.n_cell, _ptr(cells, _i64p),
                            _ptr(ed, _i32p), space.n_dof, acc_stiff, acc_mass,
                            None if cf is None else _ptr(cf, _f64p), C.byref(out), _ptr(mass, _f64p))
    if rc != 0:
        raise RuntimeError(f"orc_assemble failed ({rc})")
    lib().orc_csr_free(C.byref(out))
    del nnz_guess
    return K, mass


def quadrature_points(space, acc):
    """[n_cell, nq, dim] global quadrature points of the rule of accuracy acc."""
    mesh = space.mesh
    coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    cells = np.ascontiguousarray(mesh.cells, dtype=np.int64)
    nq = lib().orc_quadrature_points(mesh.dim, _ptr(coords, _f64p), mesh.n_cell, _ptr(cells, _i64p), acc, None)
    if nq < 0:
        raise RuntimeError("orc_quadrature_points failed")
    pts = np.empty((mesh.n_cell, nq, mesh.dim))
    lib().orc_quadrature_points(mesh.dim, _ptr(coords, _f64p), mesh.n_cell, _ptr(cells, _i64p), acc,
                                _ptr(pts, _f64p))
    return pts


def l2_discretize(space, acc, fq=None, u=None):
    """Operator::L2Discretize of point values fq [n_cell, nq] or of a FEM function u [n_dof]."""
    mesh = space.mesh
    coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    cells = np.ascontiguousarray(mesh.cells, dtype=np.int64)
    ed = np.ascontiguousarray(space.elem_dof, dtype=np.int32)
    f1 = np.empty(space.n_dof)
    fq = None if fq is None else np.ascontiguousarray(fq, dtype=np.float64)
    u = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
    rc = lib().orc_l2_discretize(mesh.dim, space.degree, _ptr(coords, _f64p), mesh.n_cell, _ptr(cells, _i64p),
                                 _ptr(ed, _i32p), space.n_dof, acc, None if fq is None else _ptr(fq, _f64p),
                                 None if u is None else _ptr(u, _f64p), _ptr(f1, _f64p))
    if rc != 0:
        raise RuntimeError(f"orc_l2_discretize failed ({rc})")
    return f1


def apply_dirichlet(A: CSR, f, dirichlet, g=None):
    """In place on A.vals and f (BoundaryConditionAdmin::apply)."""
    d = np.ascontiguousarray(dirichlet, dtype=np.int32)
    gg = None if g is None else np.ascontiguousarray(g, dtype=np.float64)
    c = A._c()
    lib().orc_apply_dirichlet(C.byref(c), _ptr(f, _f64p), _ptr(d, _i32p), None if gg is None else _ptr(gg, _f64p))


def project(A: CSR, alpha=0.25):
    cf = np.empty(A.shape[0], dtype=np.int32)
    out = _CSR()
    lib().orc_project(C.byref(A._c()), alpha, C.byref(out), _ptr(cf, _i32p))
    P = CSR._from_c(out)
    lib().orc_csr_free(C.byref(out))
    return P, cf


def rap(P: CSR, A: CSR) -> CSR:
    out = _CSR()
    lib().orc_rap(C.byref(P._c()), C.byref(A._c()), C.byref(out))
    R = CSR._from_c(out)
    lib().orc_csr_free(C.byref(out))
    return R


class AMG:
    """AMGSolver::reinit + solve, restated in C."""

    def __init__(self, A: CSR, smooth_step=3, max_coarse=50, min_density=0.382, alpha=0.25):
        self._A = A
        self._h = _AMG()
        rc = lib().orc_amg_setup(C.byref(A._c()), smooth_step, max_coarse, min_density, alpha, C.byref(self._h))
        if rc != 0:
            raise RuntimeError("orc_amg_setup failed (singular coarsest matrix)")

    @classmethod
    def lazy(cls, A: CSR, smooth_step=3, max_coarse=50, min_density=0.382):
        """lazyInit: the hierarchy AMGPreconditioner builds."""
        self = cls.__new__(cls)
        self._A = A
        self._h = _AMG()
        if lib().orc_amg_setup_lazy(C.byref(A._c()), smooth_step, max_coarse, min_density, C.byref(self._h)):
            raise RuntimeError("singular coarsest matrix")
        return self

    def lazy_reinit(self, A: CSR):
        self._A = A
        if lib().orc_amg_lazy_reinit(C.byref(self._h), C.byref(A._c())):
            raise RuntimeError("lazy re-setup failed")

    @classmethod
    def from_levels(cls, A_levels, P_levels, most_project_full=True, smooth_step=3, coarse_inv=None):
        """A hierarchy built elsewhere: A_levels[0..L], P_levels[0..L-1] (CSR).
        coarse_inv (row-major, n_L x n_L) replaces the oracle's own inverse of
        the coarsest level, for coarsest levels too large for it."""
        self = cls.__new__(cls)
        self._A = A_levels[0]
        L = len(P_levels)
        As = (_CSR * (L + 1))(*[a._c() for a in A_levels])
        Ps = (_CSR * max(L, 1))(*[p._c() for p in P_levels]) if L else (_CSR * 1)()
        self._h = _AMG()
        full = int(most_project_full) if coarse_inv is None else 0
        rc = lib().orc_amg_from_levels(L, As, Ps, full, smooth_step, C.byref(self._h))
        if rc != 0:
            raise RuntimeError("singular coarsest matrix")
        if coarse_inv is not None:
            inv = np.ascontiguousarray(coarse_inv, dtype=np.float64)
            if lib().orc_amg_set_coarse_inverse(C.byref(self._h), _ptr(inv, _f64p)) != 0:
                raise RuntimeError("coarse inverse")
        return self

    def __del__(self):
        if getattr(self, "_h", None) is not None and lib is not None:
            try:
                lib().orc_amg_free(C.byref(self._h))
            except Exception:
                pass

    @property
    def n_level(self):
        return self._h.n_level

    def level(self, l) -> CSR:
        return CSR._from_c(self._h.A[l])

    def projection(self, l) -> CSR:
        return CSR._from_c(self._h.P[l])

    def coarse_inverse(self):
        n = self._h.n_coarse
        return np.ctypeslib.as_array(self._h.coarse_inv, (n * n,)).reshape(n, n).copy()

    def vcycles(self, x, r, cycles):
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        r = np.ascontiguousarray(r, dtype=np.float64)
        lib().orc_amg_vcycles(C.byref(self._h), _ptr(x, _f64p), _ptr(r, _f64p), cycles)
        return x

    def pcg(self, b, tol=1e-10, maxit=500, x0=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.ascontiguousarray(x0, dtype=np.float64).copy()
        rel = C.c_double()
        it = lib().orc_pcg(C.byref(self._A._c()), C.byref(self._h), _ptr(b, _f64p), _ptr(x, _f64p), tol, maxit,
                           C.byref(rel))
        return x, it, rel.value

"""Python mirror of AFEPack's discretisation interface over the C ABI.

Names and argument meaning follow the reference classes:
``StiffMatrix`` / ``MassMatrix`` (include/AFEPack/BilinearOperator.h:74-224:
``algebricAccuracy()``, ``build()``), ``BoundaryConditionAdmin``
(include/AFEPack/FEMSpace.h, ``add`` / ``apply``) and the CSR
``SparseMatrix`` (include/AFEPack/SparseMatrix.h: ``m()``, ``n()``,
``n_nonzero_elements()``, ``vmult``).  All computation happens in
libafepack_gb300 on the GPU; these classes own handles and move arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .mesh import FESpace as HostSpace


class Context:
    """One GPU and one CUDA stream (afp_context)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        N.call("afp_context_create", device, C.byref(h))
        self.handle = h

    def synchronize(self):
        N.call("afp_context_synchronize", self.handle)

    def stream(self) -> int:
        """The library's cudaStream_t as an integer handle."""
        s = C.c_void_p()
        N.call("afp_context_stream", self.handle, C.byref(s))
        return s.value or 0

    def launch_count(self) -> int:
        v = C.c_int64()
        N.call("afp_context_launch_count", self.handle, C.byref(v))
        return v.value

    def close(self):
        if self.handle:
            N.lib().afp_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SparseMatrix:
    """Device CSR in AFEPack's layout (diagonal first in each row)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    @classmethod
    def from_csr(cls, ctx: Context, rowptr, cols, vals, shape=None):
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        m = rowptr.shape[0] - 1
        n = shape[1] if shape is not None else m
        h = C.c_void_p()
        N.call("afp_matrix_create_csr", ctx.handle, m, n, int(rowptr[-1]), N.ptr(rowptr), N.ptr(cols),
               N.ptr(vals), C.byref(h))
        return cls(ctx, h)

    def info(self):
        m, n, nnz = C.c_int64(), C.c_int64(), C.c_int64()
        N.call("afp_matrix_info", self.handle, C.byref(m), C.byref(n), C.byref(nnz))
        return m.value, n.value, nnz.value

    def m(self):
        return self.info()[0]

    def n(self):
        return self.info()[1]

    def n_nonzero_elements(self):
        return self.info()[2]

    def download(self):
        m, _, nnz = self.info()
        rp = np.empty(m + 1, dtype=np.int32)
        ci = np.empty(nnz, dtype=np.int32)
        va = np.empty(nnz, dtype=np.float64)
        N.call("afp_matrix_download", self.handle, N.ptr(rp), N.ptr(ci), N.ptr(va))
        return rp, ci, va

    def set_values(self, vals):
        """Overwrite the stored values (pattern unchanged)."""
        if not hasattr(vals, "data_ptr"):
            vals = np.ascontiguousarray(vals, dtype=np.float64)
        N.call("afp_matrix_set_values", self.handle, N.ptr(vals))

    def values(self):
        _, _, nnz = self.info()
        va = np.empty(nnz, dtype=np.float64)
        N.call("afp_matrix_download", self.handle, None, None, N.ptr(va))
        return va

    def vmult(self, x):
        m, n, _ = self.info()
        if hasattr(x, "data_ptr"):
            import torch
            y = torch.empty(m, dtype=torch.float64, device=x.device)
        else:
            x = np.ascontiguousarray(x, dtype=np.float64)
            y = np.empty(m)
        N.call("afp_matrix_vmult", self.handle, N.ptr(x), N.ptr(y))
        return y

    def close(self):
        if self.handle:
            N.lib().afp_matrix_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Space:
    """Device copy of a P1/P2 space: mesh, cells and AFEPack's DOF map."""

    def __init__(self, ctx: Context, host: HostSpace):
        self.ctx = ctx
        self.host = host
        self.mesh = mesh = host.mesh
        coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
        cells = np.ascontiguousarray(mesh.cells, dtype=np.int32)
        ed = np.ascontiguousarray(host.elem_dof, dtype=np.int32)
        h = C.c_void_p()
        N.call("afp_space_create", ctx.handle, mesh.dim, host.degree, mesh.n_vertex, N.ptr(coords), mesh.n_cell,
               N.ptr(cells), host.n_dof, N.ptr(ed), C.byref(h))
        self.handle = h

    @classmethod
    def numbered(cls, ctx: Context, mesh, degree: int) -> "Space":
        """FEMSpace::buildDof on the device: the DOF map, boundary marks and
        interpolation points computed from the mesh alone."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.host = None
        coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
        cells = np.ascontiguousarray(mesh.cells, dtype=np.int32)
        bm = np.ascontiguousarray(mesh.bmask, dtype=np.int32)
        h = C.c_void_p()
        N.call("afp_space_create_numbered", ctx.handle, mesh.dim, degree, mesh.n_vertex, N.ptr(coords), mesh.n_cell,
               N.ptr(cells), N.ptr(bm), C.byref(h))
        self.handle = h
        self.mesh = mesh
        return self

    def dofs(self):
        """(elem_dof [n_cell, nd], dof_bmark [n_dof], dof_point [n_dof, dim]) of a numbered space."""
        n, nd = C.c_int64(), C.c_int()
        N.call("afp_space_info", self.handle, C.byref(n), C.byref(nd))
        mesh = self.mesh
        ed = np.empty((mesh.n_cell, nd.value), dtype=np.int32)
        bm = np.empty(n.value, dtype=np.int32)
        pt = np.empty((n.value, mesh.dim))
        N.call("afp_space_download_dofs", self.handle, N.ptr(ed), N.ptr(bm), N.ptr(pt))
        return ed, bm, pt

    @property
    def n_dof(self):
        if self.host is None:
            n = C.c_int64()
            N.call("afp_space_info", self.handle, C.byref(n), None)
            return n.value
        return self.host.n_dof

    def close(self):
        if self.handle:
            N.lib().afp_space_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def assemble(space: Space, acc_stiff: int, acc_mass: int | None = None, coef=None):
    """Stiffness (scaled per cell by coef) and, when acc_mass is given, the
    mass matrix in the same pattern: StiffMatrix::build + MassMatrix::build."""
    cf = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
    opts = N.AssembleOpts(acc_stiff, acc_mass if acc_mass is not None else 0,
                          cf.ctypes.data_as(N.c_f64p) if cf is not None else None)
    K, M = C.c_void_p(), C.c_void_p()
    N.call("afp_assemble", space.handle, C.byref(opts), C.byref(K), C.byref(M) if acc_mass is not None else None)
    km = SparseMatrix(space.ctx, K)
    mm = SparseMatrix(space.ctx, M) if acc_mass is not None else None
    return km, mm


SOURCE_POINT_VALUES, SOURCE_FEM_FUNCTION, SOURCE_GAUSSIANS = 0, 1, 2


def quadrature_points(space: Space, acc: int) -> np.ndarray:
    """[n_cell, n_q, dim] global quadrature points of the rule of accuracy acc."""
    nq = C.c_int()
    N.call("afp_quadrature_points", space.handle, acc, C.byref(nq), None)
    pts = np.empty((space.mesh.n_cell, nq.value, space.mesh.dim))
    N.call("afp_quadrature_points", space.handle, acc, C.byref(nq), N.ptr(pts))
    return pts


class Gaussians:
    """f(x) = sum_g amp_g exp(-|x - c_g|^2 / (2 s_g^2)), evaluated on the device."""

    def __init__(self, centres, widths, amps=None):
        centres = np.atleast_2d(np.asarray(centres, dtype=np.float64))
        widths = np.asarray(widths, dtype=np.float64).reshape(-1, 1)
        amps = np.ones_like(widths) if amps is None else np.asarray(amps, dtype=np.float64).reshape(-1, 1)
        self.data = np.ascontiguousarray(np.concatenate([centres, widths, amps], axis=1))


def L2Discretize(f, space: Space, acc: int) -> np.ndarray:
    """Operator::L2Discretize(f, fem_space, f1, algebric_accuracy) on the GPU.

    f: a callable of points [..., dim] (evaluated on the host at the device's
    quadrature points, as the reference evaluates its function pointer), the
    DOF values of a FEM function on `space`, or `Gaussians` (evaluated on the
    device)."""
    if isinstance(f, Gaussians):
        src, data = SOURCE_GAUSSIANS, f.data
    elif callable(f):
        src, data = SOURCE_POINT_VALUES, np.ascontiguousarray(f(quadrature_points(space, acc)), dtype=np.float64)
    else:
        src, data = SOURCE_FEM_FUNCTION, np.ascontiguousarray(f, dtype=np.float64)
    out = np.empty(space.n_dof)
    N.call("afp_l2_discretize", space.handle, acc, src, N.ptr(data), data.size, N.ptr(out))
    return out


class StiffMatrix:
    """StiffMatrix<DIM,double>(fem_space): set algebricAccuracy, then build()."""

    def __init__(self, space: Space, coef=None):
        self.space = space
        self.algebricAccuracy = 2 if space.mesh.dim == 3 else 4
        self.coef = coef
        self.matrix: SparseMatrix | None = None

    def build(self) -> SparseMatrix:
        self.matrix, _ = assemble(self.space, self.algebricAccuracy, None, self.coef)
        return self.matrix


class MassMatrix:
    """MassMatrix<DIM,double>(fem_space): set algebricAccuracy, then build()."""

    def __init__(self, space: Space):
        self.space = space
        self.algebricAccuracy = 4
        self.matrix: SparseMatrix | None = None

    def build(self) -> SparseMatrix:
        _, self.matrix = assemble(self.space, 1, self.algebricAccuracy)
        return self.matrix


class BoundaryConditionAdmin:
    """Dirichlet conditions by boundary mark, applied as AFEPack does
    (FEMSpace.templates.h:1305-1366)."""

    def __init__(self, host: HostSpace):
        self.host = host
        self.conditions: dict[int, object] = {}

    def add(self, mark: int, value=0.0):
        """value: a constant or a function of the interpolation points [n, dim]."""
        if mark < 0:
            raise ValueError("a boundary mark must be a positive number")
        if mark in self.conditions:
            raise ValueError(f"there is a boundary condition for mark {mark} already")
        self.conditions[mark] = value

    def arrays(self):
        bm = self.host.dof_bmark
        dirichlet = np.zeros(self.host.n_dof, dtype=np.int32)
        g = np.zeros(self.host.n_dof)
        for mark, val in self.conditions.items():
            sel = bm == mark
            dirichlet[sel] = 1
            g[sel] = val(self.host.dof_point[sel]) if callable(val) else float(val)
        return dirichlet, g

    def apply(self, A: SparseMatrix, f, preserve_symmetry: bool = True):
        """In place on A and on f (a float64 numpy array or CUDA tensor)."""
        dirichlet, g = self.arrays()
        if hasattr(f, "data_ptr"):
            import torch
            dirichlet = torch.from_numpy(dirichlet).to(f.device)
            g = torch.from_numpy(g).to(f.device)
        N.call("afp_apply_dirichlet", A.handle, N.ptr(f), N.ptr(dirichlet), N.ptr(g), int(preserve_symmetry))

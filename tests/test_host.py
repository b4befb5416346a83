"""Host-side logic: DOF numbering, quadrature tables, C/F coarsening, C ABI."""
import os
import re

import numpy as np
import pytest

import oracle as O
from conftest import ROOT, golden_csr, golden_names, load_golden
from afepack_gb300.mesh import FESpace, cube_mesh, square_mesh


CASE_MESH = {
    "tri_p1_8": lambda: square_mesh(8, 0.2, 0),
    "tri_p1_16_coef": lambda: square_mesh(16, 0.2, 5),
    "tri_p2_6": lambda: square_mesh(6, 0.2, 1),
    "tet_p1_4": lambda: cube_mesh(4, 0.15, 2),
    "tet_p2_2": lambda: cube_mesh(2, 0.15, 3),
}


@pytest.mark.parametrize("name", golden_names())
def test_dof_numbering_matches_reference(name):
    g = load_golden(name)
    mesh = CASE_MESH[name]()
    assert np.array_equal(mesh.coords, g["coords"]) and np.array_equal(mesh.cells, g["cells"])
    sp = FESpace(mesh, int(g["degree"]))
    assert np.array_equal(sp.elem_dof, g["elem_dof"])
    assert np.array_equal(sp.dof_bmark, g["dof_bmark"])


def test_meshes_positively_oriented():
    for mesh in (square_mesh(12), cube_mesh(5)):
        x = mesh.coords[mesh.cells]
        if mesh.dim == 2:
            a, b = x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]
            vol = a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]
        else:
            vol = np.einsum("ij,ij->i", np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]), x[:, 3] - x[:, 0])
        assert (vol > 0).all()


def test_quadrature_tables():
    from afepack_gb300.csrc import gen_quadrature as G  # noqa: F401  (module imports cleanly)
    text = open(os.path.join(ROOT, "afepack_gb300", "csrc", "quadrature_tables.h")).read()
    for name, dim in (("AFP_TRI_QUAD", 2), ("AFP_TET_QUAD", 3)):
        offs = [int(v) for v in re.search(name + r"_OFFSET\[\d+\] = \{([^}]*)\}", text).group(1).split(",")]
        body = re.search(name + r"_POINTS\[\d+\]\[\d\] = \{(.*?)\n\};", text, re.S).group(1)
        pts = np.array([[float(v) for v in row.split(",") if v.strip()] for row in re.findall(r"\{([^}]*)\}", body)])
        for a, b in zip(offs[:-1], offs[1:]):
            assert abs(pts[a:b, dim].sum() - 1.0) < 2e-7  # weights of each rule sum to one
    import refpath
    tdir = refpath.template_dir()
    if tdir is not None:
        tri = G.parse(os.path.join(tdir, "triangle", "triangle.tmp_geo"), 2)
        assert len(tri[4]) == 6 and tri[4][0][0] == 0.445948490915965


@pytest.mark.parametrize("name", golden_names())
def test_host_coarsen_matches_reference(native, name):
    from afepack_gb300.amg import host_coarsen
    g = load_golden(name)
    A = golden_csr(g, "system")
    for l in range(int(g["n_project"])):
        cf, rp, ci, va = host_coarsen(A.rowptr, A.cols, A.vals)
        P = golden_csr(g, f"P{l}")
        assert np.array_equal(rp, P.rowptr) and np.array_equal(ci, P.cols) and np.array_equal(va, P.vals)
        assert int((cf == -1).sum()) == P.shape[0]
        A = golden_csr(g, f"A{l + 1}")


def test_host_coarsen_larger(native):
    from afepack_gb300.amg import host_coarsen
    from afepack_gb300 import workloads as W
    wl = W.poisson2d_p1(64)
    K, mass = O.assemble(wl.space, 4, 4)
    b = O.CSR(K.rowptr, K.cols, mass, K.shape).matvec(wl.f)
    O.apply_dirichlet(K, b, wl.space.dof_bmark)
    A = K
    for _ in range(3):
        P, cf_o = O.project(A)
        cf, rp, ci, va = host_coarsen(A.rowptr, A.cols, A.vals)
        assert np.array_equal(cf, cf_o)
        assert np.array_equal(rp, P.rowptr) and np.array_equal(ci, P.cols) and np.array_equal(va, P.vals)
        A = O.rap(P, A)


def test_abi_exports_every_declared_symbol(native):
    header = open(os.path.join(ROOT, "include", "afepack_gb300.h")).read()
    declared = sorted(set(re.findall(r"\b(afp_[a-z0-9_]+)\s*\(", header)))
    assert len(declared) >= 25
    from afepack_gb300 import _native
    for name in declared:
        assert hasattr(native, name), name
        assert name in _native.SIGNATURES, name
    assert native.afp_version() == 1
    assert native.afp_status_string(5) == b"not converged"


def test_errors_without_gpu_are_reported(native):
    # no GPU here (or a GPU): a bad device index is an invalid argument, never a crash
    import ctypes as C
    h = C.c_void_p()
    st = native.afp_context_create(10_000, C.byref(h))
    assert st in (1, 3)


def test_null_arguments_are_invalid_without_a_gpu(native):
    """Entry points check their arguments before touching a device: NULL
    handles and pointers are AFP_ERR_INVALID (1), on any machine."""
    import ctypes as C
    out = C.c_void_p()
    assert native.afp_space_create_numbered(None, 2, 1, 4, None, 2, None, None, C.byref(out)) == 1
    assert native.afp_space_info(None, None, None) == 1
    assert native.afp_space_download_dofs(None, None, None, None) == 1
    assert native.afp_quadrature_points(None, 4, None, None) == 1
    assert native.afp_l2_discretize(None, 4, 0, None, 0, None) == 1
    assert native.afp_batch_server_submit(None, None, None) == 1


def test_amg_default_options():
    """Defaults of afp_amg_opts as set by afp_amg_default_opts (host only):
    the reference's AMGSolver parameters plus the GB300-side choices."""
    from afepack_gb300.amg import default_opts
    o = default_opts()
    assert (o.tolerance, o.smooth_step, o.max_coarse) == (1e-12, 3, 50)
    assert (o.min_density, o.alpha) == (0.382, 0.25)
    assert o.precision == 0 and o.symmetric == 1
    assert (o.dense_tail, o.max_colors, o.coarse_colors) == (4096, 32, 4)
    assert o.interp_bf16 == 0 and o.fused_vcycle == 0
    assert o.wait_limit_s == 2.0 and o.inject_barrier_stall == 0 and o.gpu_coarsen == 1

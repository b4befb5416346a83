"""GPU assembly and Dirichlet elimination against the reference (golden
fixtures from AFEPack itself) and against the oracle at larger sizes.

Contract: CSR pattern bit-exact; values within 1e-13 of the reference,
row-scaled (|da_ij| <= 1e-13 max_k |a_ik|).  The kernels repeat the
reference's arithmetic, so equality is in fact bitwise and is asserted too.
"""
import numpy as np
import pytest

import oracle as O
from conftest import golden_csr, golden_names, golden_space, load_golden

pytestmark = pytest.mark.gpu
TOL = 1e-13


def row_scaled_err(rp, a, b):
    rows = np.repeat(np.arange(rp.shape[0] - 1), np.diff(rp))
    scale = np.maximum.reduceat(np.abs(b), rp[:-1]) if b.size else b
    return float((np.abs(a - b) / np.maximum(scale[rows], 1e-300)).max()) if b.size else 0.0


def gpu_assemble(ctx, sp, acc_s, acc_m, coef=None):
    from afepack_gb300.fem import Space, assemble
    space = Space(ctx, sp)
    K, M = assemble(space, acc_s, acc_m, coef)
    return space, K, M


@pytest.mark.parametrize("name", golden_names())
def test_assembly_matches_reference(ctx, name):
    g = load_golden(name)
    sp = golden_space(g)
    _, K, M = gpu_assemble(ctx, sp, int(g["acc_stiff"]), int(g["acc_mass"]), g.get("coef"))
    rp, ci, va = K.download()
    ref = golden_csr(g, "stiff")
    assert np.array_equal(rp, ref.rowptr) and np.array_equal(ci, ref.cols)
    assert row_scaled_err(rp, va, ref.vals) <= TOL
    assert row_scaled_err(rp, M.values(), g["mass_vals"]) <= TOL
    assert np.array_equal(va, ref.vals) and np.array_equal(M.values(), g["mass_vals"])


@pytest.mark.parametrize("name", golden_names())
def test_dirichlet_matches_reference(ctx, name):
    from afepack_gb300.fem import BoundaryConditionAdmin
    g = load_golden(name)
    sp = golden_space(g)
    _, K, M = gpu_assemble(ctx, sp, int(g["acc_stiff"]), int(g["acc_mass"]), g.get("coef"))
    b = M.vmult(g["f"])
    assert np.allclose(b, g["rhs_mass"], rtol=1e-14, atol=1e-16)
    bca = BoundaryConditionAdmin(sp)
    bca.add(1, 0.0)
    b = g["rhs_mass"].copy()
    bca.apply(K, b)
    assert np.array_equal(K.values(), g["system_vals"])
    assert np.array_equal(b, g["rhs"])


@pytest.mark.parametrize("dim,degree,n", [(2, 1, 256), (2, 2, 48), (3, 1, 24), (3, 2, 10)])
def test_assembly_matches_oracle_large(ctx, dim, degree, n):
    from afepack_gb300.mesh import FESpace, cube_mesh, square_mesh
    from afepack_gb300.workloads import ACC
    mesh = square_mesh(n, 0.2, 7) if dim == 2 else cube_mesh(n, 0.15, 7)
    sp = FESpace(mesh, degree)
    acc_s, acc_m = ACC[(dim, degree)]
    coef = np.exp(np.random.default_rng(n).standard_normal(mesh.n_cell))
    _, K, M = gpu_assemble(ctx, sp, acc_s, acc_m, coef)
    Ko, mo = O.assemble(sp, acc_s, acc_m, coef)
    rp, ci, va = K.download()
    assert np.array_equal(rp, Ko.rowptr) and np.array_equal(ci, Ko.cols)
    assert row_scaled_err(rp, va, Ko.vals) <= TOL
    assert row_scaled_err(rp, M.values(), mo) <= TOL


def test_nonzero_dirichlet_data(ctx):
    from afepack_gb300.fem import BoundaryConditionAdmin
    from afepack_gb300.mesh import FESpace, square_mesh
    sp = FESpace(square_mesh(20, 0.2, 3), 2)
    _, K, M = gpu_assemble(ctx, sp, 4, 4)
    Ko, mo = O.assemble(sp, 4, 4)
    g = lambda p: np.sin(3 * p[:, 0]) + p[:, 1] ** 2
    f = np.random.default_rng(1).uniform(-1, 1, sp.n_dof)
    bca = BoundaryConditionAdmin(sp)
    bca.add(1, g)
    bo = O.CSR(Ko.rowptr, Ko.cols, mo, Ko.shape).matvec(f)
    b = M.vmult(f)
    assert np.allclose(b, bo, rtol=1e-13, atol=1e-16 * np.abs(bo).max())  # SpMV: rounding order differs
    b = bo.copy()  # same right-hand side into both eliminations
    bca.apply(K, b)
    d, gv = bca.arrays()
    O.apply_dirichlet(Ko, bo, d, gv)
    assert np.array_equal(K.values(), Ko.vals)
    assert np.array_equal(b, bo)


def test_bad_input_is_an_error_not_a_fault(ctx):
    from afepack_gb300 import _native as N
    from afepack_gb300.fem import Space
    from afepack_gb300.mesh import FESpace, square_mesh
    sp = FESpace(square_mesh(4), 1)
    sp.elem_dof = sp.elem_dof.copy()
    sp.elem_dof[3, 1] = sp.n_dof + 5  # out of range: rejected before any kernel uses it
    with pytest.raises(N.AFPError) as e:
        Space(ctx, sp)
    assert e.value.status == 1


@pytest.mark.parametrize("dim,degree,n", [(2, 1, 64), (2, 2, 40), (3, 1, 12), (3, 2, 7)])
def test_device_dof_numbering_matches_buildDof(ctx, dim, degree, n):
    """afp_space_create_numbered: the DOF map, boundary marks and points equal
    the host numbering of FEMSpace::buildDof's order, and so do the matrices."""
    from afepack_gb300.fem import Space, assemble
    from afepack_gb300.mesh import FESpace, cube_mesh, square_mesh
    mesh = square_mesh(n, 0.2, 3) if dim == 2 else cube_mesh(n, 0.15, 3)
    host = FESpace(mesh, degree)
    dev = Space.numbered(ctx, mesh, degree)
    ed, bm, pt = dev.dofs()
    assert dev.n_dof == host.n_dof
    assert np.array_equal(ed, host.elem_dof)
    assert np.array_equal(bm, host.dof_bmark)
    assert np.array_equal(pt, host.dof_point)
    acc = {(2, 1): (4, 4), (2, 2): (4, 4), (3, 1): (2, 4), (3, 2): (4, 4)}[(dim, degree)]
    K1, _ = assemble(dev, *acc)
    K2, _ = assemble(Space(ctx, host), *acc)
    for a, b in zip(K1.download(), K2.download()):
        assert np.array_equal(a, b)


def _poly(pts):
    x, y = pts[..., 0], pts[..., 1]
    return 1.0 + x * y - 2.0 * y * y


@pytest.mark.parametrize("name", golden_names())
def test_l2_discretize_matches_reference(ctx, name):
    """Operator::L2Discretize on the GPU, bitwise against AFEPack: a point
    function at the device's quadrature points, and a FEM function."""
    from afepack_gb300.fem import L2Discretize, Space, quadrature_points
    g = load_golden(name)
    host = golden_space(g)
    sp = Space(ctx, host)
    acc = int(g["acc_mass"])
    assert np.array_equal(quadrature_points(sp, acc), O.quadrature_points(host, acc))
    assert np.array_equal(L2Discretize(_poly, sp, acc), g["l2_fun"])
    assert np.array_equal(L2Discretize(g["f"], sp, acc), g["l2_fem"])


@pytest.mark.parametrize("dim,degree,n", [(2, 2, 96), (3, 1, 40), (3, 2, 8)])
def test_l2_discretize_matches_oracle(ctx, dim, degree, n):
    """Larger meshes against the oracle: bitwise for point values and FEM
    functions (3D P1 40^3 has 384,000 cells, more than one 256 MB chunk of
    terms, so the per-DOF sums continue across chunks); device-evaluated
    Gaussians within 1e-14 of the oracle fed numpy's values."""
    from afepack_gb300.fem import Gaussians, L2Discretize, Space
    from afepack_gb300.mesh import FESpace, cube_mesh, square_mesh
    mesh = square_mesh(n, 0.2, 4) if dim == 2 else cube_mesh(n, 0.15, 4)
    host = FESpace(mesh, degree)
    sp = Space(ctx, host)
    acc = 4
    pts = O.quadrature_points(host, acc)
    assert np.array_equal(L2Discretize(_poly, sp, acc), O.l2_discretize(host, acc, fq=_poly(pts)))
    u = np.random.default_rng(7).uniform(-1, 1, host.n_dof)
    assert np.array_equal(L2Discretize(u, sp, acc), O.l2_discretize(host, acc, u=u))
    rng = np.random.default_rng(8)
    c, s = rng.uniform(0.2, 0.8, (8, dim)), rng.uniform(0.05, 0.2, 8)
    fq = np.zeros(pts.shape[:2])
    for cc, ss in zip(c, s):
        fq += np.exp(-np.sum((pts - cc) ** 2, axis=-1) / (2.0 * ss * ss))
    ref = O.l2_discretize(host, acc, fq=fq)
    got = L2Discretize(Gaussians(c, s), sp, acc)
    assert np.max(np.abs(got - ref)) <= 1e-14 * np.max(np.abs(ref))

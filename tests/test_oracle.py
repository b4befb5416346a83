"""The CPU oracle (plain-C restatement) against the reference's own outputs.

Golden fixtures come from AFEPack compiled from its sources
(tests/golden/make_golden.py).  The restatement must agree bit for bit on
assembly, Dirichlet elimination, every AMG level and the V-cycle iterate.
"""
import numpy as np
import pytest

import oracle as O
from conftest import golden_csr, golden_names, golden_space, load_golden


@pytest.mark.parametrize("name", golden_names())
def test_assembly_bitwise(name):
    g = load_golden(name)
    sp = golden_space(g)
    K, mass = O.assemble(sp, int(g["acc_stiff"]), int(g["acc_mass"]), g.get("coef"))
    ref = golden_csr(g, "stiff")
    assert np.array_equal(K.rowptr, ref.rowptr) and np.array_equal(K.cols, ref.cols)
    assert np.array_equal(K.vals, ref.vals)
    assert np.array_equal(mass, g["mass_vals"])
    b = O.CSR(K.rowptr, K.cols, mass, K.shape).matvec(g["f"])
    assert np.array_equal(b, g["rhs_mass"])


@pytest.mark.parametrize("name", golden_names())
def test_dirichlet_and_hierarchy_bitwise(name):
    g = load_golden(name)
    sp = golden_space(g)
    K, mass = O.assemble(sp, int(g["acc_stiff"]), int(g["acc_mass"]), g.get("coef"))
    b = O.CSR(K.rowptr, K.cols, mass, K.shape).matvec(g["f"])
    O.apply_dirichlet(K, b, sp.dof_bmark != 0)
    assert np.array_equal(K.vals, g["system_vals"])
    assert np.array_equal(b, g["rhs"])
    amg = O.AMG(K)
    assert amg.n_level == int(g["n_project"])
    for l in range(amg.n_level):
        P, A = amg.projection(l), amg.level(l + 1)
        Pr, Ar = golden_csr(g, f"P{l}"), golden_csr(g, f"A{l + 1}")
        for mine, ref in ((P, Pr), (A, Ar)):
            assert np.array_equal(mine.rowptr, ref.rowptr)
            assert np.array_equal(mine.cols, ref.cols)
            assert np.array_equal(mine.vals, ref.vals)
    # two V-cycles: only the dense coarse inverse (LAPACK there) may differ in rounding
    x = amg.vcycles(np.zeros_like(b), b, 2)
    assert np.allclose(x, g["x_vcycle"], rtol=1e-12, atol=1e-14 * np.abs(g["x_vcycle"]).max())
    x, it, rel = amg.pcg(b, 1e-10)
    assert rel <= 1e-10 and abs(it - int(g["pcg_iters"])) <= 1
    assert np.abs(x - g["x_pcg"]).max() <= 1e-9 * np.abs(g["x_pcg"]).max()


@pytest.mark.parametrize("name", golden_names())
def test_lazy_hierarchy_bitwise(name):
    """lazyInit / lazyReinit (AMGPreconditioner) restated against the reference."""
    g = load_golden(name)
    S = golden_csr(g, "system")
    amg = O.AMG.lazy(S)
    assert amg.n_level == int(g["lazy_n_project"])
    for l in range(amg.n_level):
        for mine, ref in ((amg.projection(l), golden_csr(g, f"LP{l}")), (amg.level(l + 1), golden_csr(g, f"LA{l + 1}"))):
            assert np.array_equal(mine.rowptr, ref.rowptr) and np.array_equal(mine.cols, ref.cols)
            assert np.array_equal(mine.vals, ref.vals)
    x = amg.vcycles(np.zeros_like(g["rhs"]), g["rhs"], 3)  # vmult with iterate_step 2
    assert np.allclose(x, g["x_lazy"], rtol=1e-11, atol=1e-13 * np.abs(g["x_lazy"]).max())
    S2 = O.CSR(S.rowptr, S.cols, S.vals * 1.5, S.shape)
    amg.lazy_reinit(S2)
    for l in range(amg.n_level):
        ref = golden_csr(g, f"LRA{l + 1}")
        assert np.array_equal(amg.level(l + 1).vals, ref.vals)
    x2 = amg.vcycles(np.zeros_like(g["rhs"]), g["rhs"], 3)
    assert np.allclose(x2, g["x_lazy2"], rtol=1e-11, atol=1e-13 * np.abs(g["x_lazy2"]).max())


def test_from_levels_with_given_coarse_inverse():
    """A hierarchy rebuilt from its levels, truncated above the coarsest level
    and given that level's inverse from LAPACK, runs the same CG as the
    oracle's own hierarchy truncated there (used for the timed CPU sample)."""
    g = load_golden("tri_p1_16_coef")
    S = golden_csr(g, "system")
    amg = O.AMG(S)
    L = min(2, amg.n_level)
    A = [amg.level(l) for l in range(L + 1)]
    P = [amg.projection(l) for l in range(L)]
    own = O.AMG.from_levels(A, P)
    inv = np.linalg.inv(A[-1].to_scipy().toarray())
    given = O.AMG.from_levels(A, P, coarse_inv=inv)
    b = g["rhs"]
    x1, it1, _ = own.pcg(b, 1e-10)
    x2, it2, _ = given.pcg(b, 1e-10)
    assert it1 == it2
    assert np.abs(x1 - x2).max() <= 1e-10 * np.abs(x1).max()


def poly_source(pts):
    """The fixture's point function, 1 + x y - 2 y^2, in the driver's operation order."""
    x, y = pts[..., 0], pts[..., 1]
    return 1.0 + x * y - 2.0 * y * y


@pytest.mark.parametrize("name", golden_names())
def test_l2_discretize_matches_reference(name):
    """Operator::L2Discretize of a point function (evaluated at the oracle's
    quadrature points) and of a FEM function, bitwise against AFEPack."""
    g = load_golden(name)
    sp = golden_space(g)
    acc = int(g["acc_mass"])
    fq = poly_source(O.quadrature_points(sp, acc))
    assert np.array_equal(O.l2_discretize(sp, acc, fq=fq), g["l2_fun"])
    assert np.array_equal(O.l2_discretize(sp, acc, u=g["f"]), g["l2_fem"])

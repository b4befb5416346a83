"""Parity at the benchmark sizes, against solvers independent of this
library: the 64^3 P1 Poisson system (274,625 DOFs) in FP64 and mixed
precision against SciPy's CG with a diagonal preconditioner run to 1e-14,
and the FP32 V-cycle with BF16 interpolation (interp_bf16) on the 32^3
system against SuperLU.  The bar is the metric's: 1e-8 relative error."""
import numpy as np
import pytest
import scipy.sparse as sps
import scipy.sparse.linalg as spla

pytestmark = pytest.mark.gpu


def system(ctx, wl):
    from afepack_gb300.fem import BoundaryConditionAdmin, Space, assemble
    space = Space(ctx, wl.space)
    K, M = assemble(space, wl.acc_stiff, wl.acc_mass, wl.coef)
    b = M.vmult(wl.f)
    bca = BoundaryConditionAdmin(wl.space)
    bca.add(1, 0.0)
    bca.apply(K, b)
    return K, b


def scipy_matrix(K):
    rp, ci, va = K.download()
    return sps.csr_matrix((va, ci, rp), shape=(rp.shape[0] - 1,) * 2)


def jacobi_cg(A, b, rtol=1e-14):
    d = A.diagonal()
    Mp = spla.LinearOperator(A.shape, matvec=lambda v: v / d)
    x, info = spla.cg(A, b, rtol=rtol, atol=0.0, maxiter=20000, M=Mp)
    assert info == 0
    return x


def test_poisson3d_p1_64_both_precisions(ctx):
    from afepack_gb300 import workloads as W
    from afepack_gb300.amg import FP64, MIXED, AMGSolver
    wl = W.poisson3d_p1(64)
    K, b = system(ctx, wl)
    A = scipy_matrix(K)
    xr = jacobi_cg(A, b)
    assert np.linalg.norm(b - A @ xr) <= 1e-11 * np.linalg.norm(b)  # SciPy stops near 1e-12
    for precision in (FP64, MIXED):
        amg = AMGSolver(K, precision=precision)
        x, info = amg.pcg(b, 1e-10, 300)
        assert info["converged"] and info["iterations"] <= 30, info
        assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr), precision


def test_bf16_interpolation_reaches_the_direct_solution(ctx):
    from afepack_gb300 import workloads as W
    from afepack_gb300.amg import FP64, MIXED, AMGSolver
    wl = W.poisson3d_p1(32)
    K, b = system(ctx, wl)
    xd = spla.splu(scipy_matrix(K).tocsc()).solve(b)
    it = {}
    for name, kw in (("fp64", dict(precision=FP64)), ("bf16", dict(precision=MIXED, interp_bf16=True))):
        amg = AMGSolver(K, **kw)
        x, info = amg.pcg(b, 1e-10, 300)
        assert info["converged"], (name, info)
        assert np.linalg.norm(x - xd) <= 1e-8 * np.linalg.norm(xd), name
        it[name] = info["iterations"]
    # BF16 interpolation weights cost iterations, within a bound
    assert it["bf16"] <= 2 * it["fp64"] + 5, it

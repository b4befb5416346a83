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


def test_elliptic2d_p2_512_mixed_against_direct(ctx):
    """2D P2 on the 512^2 split grid (1,050,625 DOFs), coefficient contrast
    1e4: the mixed-precision solve against SuperLU."""
    from afepack_gb300 import workloads as W
    from afepack_gb300.amg import MIXED, AMGSolver
    wl = W.elliptic2d_p2(512)
    K, b = system(ctx, wl)
    amg = AMGSolver(K, precision=MIXED)
    x, info = amg.pcg(b, 1e-10, 2000)
    assert info["converged"], info
    xd = spla.splu(scipy_matrix(K).tocsc()).solve(b)
    assert np.linalg.norm(x - xd) <= 1e-8 * np.linalg.norm(xd)


def test_poisson3d_p2_48_batched_against_oracle(ctx):
    """3D P2 on the 48^3 Kuhn cube (912,673 DOFs), 64 right-hand sides, the
    reference's lazyProject hierarchy: batched mixed-precision CG against the
    oracle's FP64 CG (the reference algorithm in C, on its own lazy
    hierarchy) for two of the columns."""
    import oracle as O
    import torch
    from afepack_gb300 import workloads as W
    from afepack_gb300.amg import MIXED, AMGSolver
    from afepack_gb300.fem import BoundaryConditionAdmin, Space, assemble
    wl = W.poisson3d_p2_multi(48, 64)
    K, M = assemble(Space(ctx, wl.space), wl.acc_stiff, wl.acc_mass)
    d = wl.space.dof_bmark != 0
    Bm = np.stack([M.vmult(np.ascontiguousarray(wl.f[:, c])) for c in range(64)], axis=1)
    bca = BoundaryConditionAdmin(wl.space)
    bca.add(1, 0.0)
    bca.apply(K, np.ascontiguousarray(Bm[:, 0]).copy())
    Bm[d] = 0.0
    amg = AMGSolver(precision=MIXED)
    amg.lazyReinit(K)
    X, infos = amg.pcg_multi(torch.from_numpy(np.ascontiguousarray(Bm)).to("cuda:0"), 1e-10, 500)
    assert all(i["converged"] for i in infos)
    X = X.cpu().numpy()
    rp, ci, va = K.download()
    ref = O.AMG.lazy(O.CSR(rp, ci, va, (rp.shape[0] - 1,) * 2))
    for c in (0, 63):
        xo, it, rel = ref.pcg(np.ascontiguousarray(Bm[:, c]), 1e-12, 500)
        assert rel <= 1e-12
        assert np.linalg.norm(X[:, c] - xo) <= 1e-8 * np.linalg.norm(xo), c

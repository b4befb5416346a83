"""Failure paths of the solve path, all injected from the host: a poisoned
right-hand side, an iteration limit that is too small, and one bad request in
a server that is serving others.  Each must come back as a status code with
the context still usable; no GPU fault is provoked."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BREAKDOWN, NOT_CONVERGED, TIMEOUT = 6, 5, 8


def _poisson(ctx, n=24, precision=0):
    from afepack_gb300 import workloads as W
    from afepack_gb300.amg import AMGSolver
    from afepack_gb300.fem import BoundaryConditionAdmin, Space, assemble
    wl = W.poisson2d_p1(n)
    K, M = assemble(Space(ctx, wl.space), wl.acc_stiff, wl.acc_mass)
    b = M.vmult(wl.f)
    bca = BoundaryConditionAdmin(wl.space)
    bca.add(1, 0.0)
    bca.apply(K, b)
    return K, b, AMGSolver(K, precision=precision)


def _pcg_status(native, amg, b, tol, maxit):
    from afepack_gb300 import _native as N
    x = np.zeros_like(b)
    info = N.SolveInfo()
    st = native.afp_pcg_solve(amg.handle, N.ptr(x), N.ptr(b), tol, maxit, C.byref(info))
    return st, x, info.as_dict()


@pytest.mark.parametrize("precision", [0, 1])
def test_nan_rhs_is_a_breakdown_and_the_solver_stays_usable(native, ctx, precision):
    K, b, amg = _poisson(ctx, precision=precision)
    bad = b.copy()
    bad[len(b) // 3] = np.nan
    st, _, _ = _pcg_status(native, amg, bad, 1e-10, 100)
    assert st == BREAKDOWN, native.afp_last_error()
    assert b"non-finite" in native.afp_last_error()
    st, x, info = _pcg_status(native, amg, b, 1e-10, 200)  # same solver, good data
    assert st == 0 and info["converged"] == 1


def test_iteration_limit_is_reported_as_not_converged(native, ctx):
    K, b, amg = _poisson(ctx)
    st, x, info = _pcg_status(native, amg, b, 1e-12, 2)
    assert st == NOT_CONVERGED
    assert info["iterations"] == 2 and info["converged"] == 0
    assert info["final_residual"] < info["initial_residual"]  # x holds the last iterate
    assert np.isfinite(x).all() and np.abs(x).max() > 0
    # the Python mirror reports it in info, as the reference prints it
    _, info2 = amg.pcg(b, 1e-12, 2)
    assert info2["converged"] == 0 and info2["iterations"] == 2


def test_multi_rhs_nan_column_is_a_breakdown(native, ctx):
    from afepack_gb300 import _native as N
    K, b, amg = _poisson(ctx)
    B = np.stack([b, 2 * b, -b], axis=1).copy()
    B[5, 1] = np.inf
    X = np.zeros_like(B)
    infos = (N.SolveInfo * 3)()
    st = native.afp_pcg_solve_multi(amg.handle, N.ptr(X), N.ptr(B), 3, 1e-10, 100, infos)
    assert st == BREAKDOWN
    X, infos = amg.pcg_multi(np.stack([b, 2 * b], axis=1).copy(), 1e-10, 200)
    assert all(i["converged"] for i in infos)


def test_one_poisoned_request_fails_alone_in_the_server(ctx):
    """A request whose data are NaN fails with a breakdown status; the requests
    served beside it finish with bitwise the solutions they get alone."""
    from afepack_gb300 import workloads as W
    from afepack_gb300.serve import Server
    reqs = [W.request_workload(W.Request(i, n, var, 7100 + i))
            for i, (n, var) in enumerate([(40, False), (72, True), (56, False)])]
    poison = W.request_workload(W.Request(9, 64, True, 7199))
    poison.f = poison.f.copy()
    poison.f[10] = np.nan
    with Server(workers=1) as alone:
        solo = [alone.wait(alone.submit(wl)) for wl in reqs]
    with Server(workers=4) as mix:
        tickets = [mix.submit(wl) for wl in (reqs[0], poison, reqs[1], reqs[2])]
        out = [mix.wait(t) for t in tickets]
        st = mix.stats()
    assert out[1][1]["status"] == BREAKDOWN
    assert st["failed"] == 1 and st["completed"] == 3
    for (x, r), (xm, rm) in zip(solo, [out[0], out[2], out[3]]):
        assert r["status"] == 0 and rm["status"] == 0
        assert np.array_equal(x, xm)


def test_one_poisoned_column_fails_alone_in_the_batch_server(ctx):
    """Continuous batching against one hierarchy: a NaN right-hand side
    retires with a breakdown status after its first iteration; the columns
    beside it finish with bitwise the solutions they get alone, and the
    server keeps serving."""
    from afepack_gb300.amg import MIXED
    from afepack_gb300.serve import BatchServer
    _, b, amg = _poisson(ctx, 48, MIXED)
    rng = np.random.default_rng(3)
    good = [b * (1.0 + 0.2 * rng.standard_normal()) for _ in range(5)]
    bad = b.copy()
    bad[7] = np.nan
    with BatchServer(amg, width=4) as alone:
        solo = [alone.wait(alone.submit(v)) for v in good]
    with BatchServer(amg, width=4) as srv:
        tickets = [srv.submit(v) for v in (good[0], good[1], bad, good[2], good[3], good[4])]
        out = [srv.wait(t) for t in tickets]
        after = srv.wait(srv.submit(good[0]))
        st = srv.stats()
    assert out[2][1]["status"] == BREAKDOWN and out[2][1]["iterations"] == 1
    assert st["failed"] == 1 and st["completed"] == 6
    for (x, r), (xm, rm) in zip(solo, [out[0], out[1], out[3], out[4], out[5]]):
        assert r["status"] == 0 and rm["status"] == 0
        assert np.array_equal(x, xm)
    assert np.array_equal(after[0], solo[0][0])


def test_stalled_grid_barrier_times_out_and_the_context_stays_usable(native, ctx):
    """Fault injection on the GPU without a fault: the persistent V-cycle's
    first grid barrier waits for one arrival more than the grid has (a count
    that nothing completes); every bounded wait gives up after 50 ms, the
    kernel returns, and the call reports AFP_ERR_TIMEOUT.  The same context
    then solves normally."""
    from afepack_gb300.amg import MIXED, AMGSolver
    K, b, _ = _poisson(ctx, n=48)
    amg = AMGSolver(K, precision=MIXED, fused_vcycle=True)
    amg.opts.wait_limit_s = 0.05
    amg.opts.inject_barrier_stall = 1
    amg.reinit(K)
    st, _, _ = _pcg_status(native, amg, b, 1e-10, 50)
    assert st == TIMEOUT, native.afp_last_error()
    assert b"bounded wait" in native.afp_last_error()
    good = AMGSolver(K, precision=MIXED, fused_vcycle=True)
    st, x, info = _pcg_status(native, good, b, 1e-10, 200)
    assert st == 0 and info["converged"] == 1

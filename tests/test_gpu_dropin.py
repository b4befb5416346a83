"""The drop-in boundary executed on the GPU.  AFEPack itself cannot be built
where the GPU is (its sources are not there), so the test builds the
drop-in's core -- everything AMGSolver_gb300.cpp does apart from reading
AFEPack's classes -- with a C++ driver that replays AFEPack's calls, runs it,
and checks what comes back against the reference's own outputs (the
fixtures): the lazy hierarchy bitwise, its numeric re-setup bitwise, the
refusal of another pattern, and AMGSolver::solve / AMGPreconditioner::vmult
against the same calls made directly through the C ABI."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_csr, golden_names, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(native, tmp_path_factory):
    from afepack_gb300.build import LIB
    exe = tmp_path_factory.mktemp("dropin") / "dropin_driver"
    cxx = shutil.which("g++") or "g++"
    libdir = os.path.dirname(LIB)
    cmd = [cxx, "-std=c++17", "-O1", os.path.join(ROOT, "tests", "dropin_driver.cpp"),
           os.path.join(ROOT, "afepack_gb300", "dropin", "dropin_core.cpp"), "-I" + os.path.join(ROOT, "include"),
           "-L" + libdir, "-lafepack_gb300", "-Wl,-rpath," + libdir, "-pthread", "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    return str(exe)


def _read(d, name, dtype):
    return np.fromfile(os.path.join(d, name), dtype=dtype)


@pytest.mark.parametrize("name", golden_names())
def test_dropin_core_against_reference(driver, ctx, tmp_path, name):
    from afepack_gb300.amg import AMGPreconditioner, AMGSolver
    from afepack_gb300.fem import SparseMatrix
    g = load_golden(name)
    S = golden_csr(g, "system")
    m = S.shape[0]
    with open(tmp_path / "system.bin", "wb") as f:
        np.array([m, S.nnz], dtype=np.int64).tofile(f)
        S.rowptr.astype(np.int32).tofile(f)
        S.cols.astype(np.int32).tofile(f)
        S.vals.astype(np.float64).tofile(f)
        g["rhs"].astype(np.float64).tofile(f)
    env = dict(os.environ, AFP_DENSE_TAIL="0")
    res = subprocess.run([driver, str(tmp_path)], capture_output=True, text=True, env=env, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    d = str(tmp_path)
    # lazyInit: the reference's lazyProject hierarchy, bitwise
    np_lazy = int(open(os.path.join(d, "lazy_levels.txt")).read())
    assert np_lazy == int(g["lazy_n_project"])
    for l in range(1, np_lazy + 1):
        A = golden_csr(g, f"LA{l}")
        assert np.array_equal(_read(d, f"lazy{l}_rp.bin", np.int32), A.rowptr)
        assert np.array_equal(_read(d, f"lazy{l}_ci.bin", np.int32), A.cols)
        assert np.array_equal(_read(d, f"lazy{l}_va.bin", np.float64), A.vals)
        # lazyReinit on the same pattern with values x 1.5: the reference's re-setup
        assert np.array_equal(_read(d, f"relazy{l}_va.bin", np.float64), golden_csr(g, f"LRA{l}").vals)
    assert "same sparsity pattern" in open(os.path.join(d, "refused.txt")).read()
    # solve / vmult equal the same calls made through the C ABI directly
    K = SparseMatrix.from_csr(ctx, S.rowptr, S.cols, S.vals)
    direct = AMGSolver(K, dense_tail=0, symmetric=False)
    x = np.zeros(m)
    direct.solve(x, g["rhs"], 1e-8, 4, 1)
    assert np.array_equal(_read(d, "x_solve.bin", np.float64), x)
    K2 = SparseMatrix.from_csr(ctx, S.rowptr, S.cols, S.vals * 1.5)
    pre = AMGPreconditioner(K2, 2, 3, dense_tail=0, symmetric=False)
    xv = np.zeros(m)
    pre.vmult(xv, g["rhs"])
    assert np.array_equal(_read(d, "x_vmult.bin", np.float64), xv)

"""The C++ drop-ins (afepack_gb300/dropin/AMGSolver_gb300.cpp and
BilinearOperator_gb300.cpp) compile against AFEPack's unchanged headers and
link with the rest of AFEPack and libafepack_gb300.so in place of
src/AMGSolver.cpp and src/BilinearOperator.cpp.  Needs the reference sources
(skipped where they are not mounted); nothing is run."""
import glob
import os
import subprocess

import pytest

from conftest import ROOT

import refpath

REF = refpath.source() or ""
OBJ = os.path.join(ROOT, "oracle", "_ref", "obj")

MAIN = r"""
#include <AFEPack/AMGSolver.h>
#include <AFEPack/BilinearOperator.h>
#include "VarCoeffStiffMatrix.h"
using namespace AFEPack;
int main(int argc, char**) {
  SparsityPattern sp(1, 1, (size_t)1);
  sp.compress();
  SparseMatrix<double> A(sp);
  AMGSolver solver;   // construct only: reinit/solve/build would need a GPU
  Vector<double> x(1), r(1);
  if (argc > 99) {
    solver.reinit(A);
    solver.solve(x, r, 1e-8, 200);
    FEMSpace<double, 2> fs2;
    StiffMatrix<2, double> K2(fs2);
    MassMatrix<2, double> M2(fs2);
    K2.build();
    M2.build();
    FEMSpace<double, 3> fs3;
    StiffMatrix<3, double> K3(fs3);
    K3.build();
    std::vector<double> coef(1, 2.0);
    VarCoeffStiffMatrix<2> C2(fs2, coef);
    C2.build();
  }
  return 0;
}
"""


@pytest.mark.skipif(not REF, reason="AFEPack sources not available")
def test_dropin_links_into_afepack(native, tmp_path):
    if not os.path.exists(os.path.join(OBJ, "BilinearOperator.o")):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "-j8", f"REF={REF}"],
                              stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    flags = ["-std=c++20", "-O1", "-w", "-I" + os.path.join(ROOT, "oracle", "shim"), "-I" + os.path.join(REF, "include"),
             "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "afepack_gb300", "dropin")]
    drops = []
    for src in ("AMGSolver_gb300.cpp", "BilinearOperator_gb300.cpp", "dropin_core.cpp"):
        obj = tmp_path / src.replace(".cpp", ".o")
        subprocess.check_call(["g++", *flags, "-c", os.path.join(ROOT, "afepack_gb300", "dropin", src), "-o", str(obj)])
        drops.append(str(obj))
    main = tmp_path / "main.cpp"
    main.write_text(MAIN)
    objs = [o for o in glob.glob(os.path.join(OBJ, "*.o"))
            if not o.endswith(("AMGSolver.o", "BilinearOperator.o", "ref_driver.o"))]
    libdir = os.path.join(ROOT, "afepack_gb300", "_lib")
    openblas = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-p", "-n"], capture_output=True,
                              text=True).stdout
    blas = [l.split(":=", 1)[1].strip() for l in openblas.splitlines() if l.startswith("OPENBLAS :=")]
    blas_lib = [b for b in blas if b and os.path.exists(b)]
    exe = tmp_path / "poisson_gpu"
    cmd = ["g++", *flags, str(main), *drops, *objs, *blas_lib, "-L" + libdir, "-lafepack_gb300",
           "-Wl,-rpath," + libdir, "-ldl", "-pthread", "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    assert exe.exists()

"""Shared fixtures.  Tests marked `gpu` need a GB300; the rest run on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103)")


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def golden_csr(g, name):
    import oracle as O
    return O.CSR(g[f"{name}_rowptr"], g[f"{name}_cols"], g[f"{name}_vals"], g[f"{name}_shape"])


def golden_space(g):
    from afepack_gb300.mesh import FESpace, Mesh
    mesh = Mesh(int(g["dim"]), 0, g["coords"], g["cells"], np.zeros(g["coords"].shape[0], np.uint8))
    sp = FESpace.__new__(FESpace)
    sp.mesh, sp.degree = mesh, int(g["degree"])
    sp.elem_dof = g["elem_dof"].astype(np.int32)
    sp.dof_bmark = g["dof_bmark"].astype(np.int32)
    sp.dof_point = np.zeros((sp.dof_bmark.shape[0], mesh.dim))
    return sp


@pytest.fixture(scope="session")
def native():
    from afepack_gb300 import _native, build
    build.build()
    return _native.lib()


@pytest.fixture(scope="session")
def ctx(native):
    from afepack_gb300.fem import Context
    c = Context(0)
    yield c
    c.close()

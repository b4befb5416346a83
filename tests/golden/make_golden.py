"""Regenerates the golden fixtures of tests/golden from AFEPack itself.

AFEPack is compiled unchanged from its sources by ``make -C oracle ref``
(the reference tree must be mounted); this script writes each case's mesh in
the reference's Mesh format, runs oracle/_ref/ref_driver (the reference's own
FEMSpace -> StiffMatrix/MassMatrix::build -> BoundaryConditionAdmin::apply ->
AMGSolver::reinit/solve call sequence) and stores its outputs as one .npz
per case.  The reference publishes no golden vectors for this path, so these
outputs are the pins.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from afepack_gb300.mesh import FESpace, cube_mesh, square_mesh, write_reference_mesh  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
TPL = os.path.join(ROOT, "oracle", "_ref", "tpl")

# name: (mesh factory, degree, acc_stiff, acc_mass, coefficient?, levels?)
CASES = {
    "tri_p1_8": (lambda: square_mesh(8, 0.2, 0), 1, 4, 4, False, True),
    "tri_p1_16_coef": (lambda: square_mesh(16, 0.2, 5), 1, 4, 4, True, True),
    "tri_p2_6": (lambda: square_mesh(6, 0.2, 1), 2, 4, 4, True, True),
    "tet_p1_4": (lambda: cube_mesh(4, 0.15, 2), 1, 2, 4, False, True),
    "tet_p2_2": (lambda: cube_mesh(2, 0.15, 3), 2, 4, 4, True, True),
}


def load_csr(d, name):
    return {f"{name}_{k}": np.load(os.path.join(d, f"{name}_{k}.npy")) for k in ("rowptr", "cols", "vals", "shape")}


def make(name, spec):
    factory, deg, acc_s, acc_m, with_coef, levels = spec
    mesh = factory()
    sp = FESpace(mesh, deg)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    f = rng.uniform(-1.0, 1.0, sp.n_dof)
    coef = np.exp(rng.standard_normal(mesh.n_cell)) if with_coef else None
    with tempfile.TemporaryDirectory() as d:
        write_reference_mesh(mesh, os.path.join(d, "m.mesh"))
        f.tofile(os.path.join(d, "f.bin"))
        args = [DRIVER, f"mesh={d}/m.mesh", f"dim={mesh.dim}", f"deg={deg}", f"out={d}", f"f={d}/f.bin",
                f"acc_stiff={acc_s}", f"acc_mass={acc_m}", "amg=1", f"dump_levels={int(levels)}", "vcycles=2",
                "pcg_tol=1e-10", "lazy=1"]
        if coef is not None:
            coef.tofile(os.path.join(d, "coef.bin"))
            args.append(f"coef={d}/coef.bin")
        res = subprocess.run(args, cwd=TPL, capture_output=True, text=True, check=True)
        meta = json.loads(res.stdout.strip().splitlines()[-1])
        out = {"coords": mesh.coords, "cells": mesh.cells, "f": f, "dim": mesh.dim, "degree": deg,
               "acc_stiff": acc_s, "acc_mass": acc_m,
               "elem_dof": np.load(os.path.join(d, "elem_dof.npy")),
               "dof_bmark": np.load(os.path.join(d, "dof_bmark.npy")),
               "rhs_mass": np.load(os.path.join(d, "rhs_mass.npy")), "rhs": np.load(os.path.join(d, "rhs.npy")),
               "l2_fun": np.load(os.path.join(d, "l2_fun.npy")), "l2_fem": np.load(os.path.join(d, "l2_fem.npy")),
               "x_vcycle": np.load(os.path.join(d, "x_vcycle.npy")), "x_pcg": np.load(os.path.join(d, "x_pcg.npy")),
               "n_project": meta["n_project"], "pcg_iters": meta["pcg_iters"]}
        if coef is not None:
            out["coef"] = coef
        for nm in ("stiff", "mass", "system"):
            out.update(load_csr(d, nm))
        for l in range(meta["n_project"]):
            out.update(load_csr(d, f"P{l}"))
            out.update(load_csr(d, f"A{l + 1}"))
        out["lazy_n_project"] = meta["lazy_n_project"]
        out["x_lazy"] = np.load(os.path.join(d, "x_lazy.npy"))
        out["x_lazy2"] = np.load(os.path.join(d, "x_lazy2.npy"))
        for l in range(meta["lazy_n_project"]):
            out.update(load_csr(d, f"LP{l}"))
            out.update(load_csr(d, f"LPt{l}"))
            out.update(load_csr(d, f"LA{l + 1}"))
            out.update(load_csr(d, f"LRA{l + 1}"))
        inv = os.path.join(d, "coarse_inverse.npy")
        if os.path.exists(inv):
            out["coarse_inverse"] = np.load(inv)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, "n_dof", sp.n_dof, "levels", meta["n_project"], "pcg", meta["pcg_iters"])


def main():
    if not os.path.exists(DRIVER):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "-j8"])
    for name, spec in CASES.items():
        make(name, spec)


if __name__ == "__main__":
    main()

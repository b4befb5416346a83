"""Seeded synthetic workloads for the elliptic-solve path.

Each workload is a mesh, a P1/P2 Lagrange space with AFEPack's DOF numbering,
an optional per-element coefficient and the nodal data f whose mass-matrix
image b = M f is the right-hand side (zero Dirichlet data on the boundary).

  poisson2d_p1(n=256)      unit square, n x n split cells, jitter 0.2h, seed 0,
                           f ~ U[-1,1] per DOF
  poisson3d_p1(n=64)       unit cube, Kuhn split, jitter 0.15h, seed 1,
                           f = sum of 8 Gaussians (centres U[0.2,0.8]^3,
                           widths U[0.05,0.2])
  elliptic2d_p2(n=512)     unit square, P2, jitter 0.2h, seed 2, log a a
                           squared-exponential Gaussian random field (length
                           0.05) per cell, rescaled to contrast 1e4; f = 1
  poisson3d_p2_multi(n=48) unit cube, Kuhn split, P2, seed 3, 64 right-hand
                           sides f ~ N(0,1) per DOF
  request_stream(count)    independent 2D P1 requests, n log-uniform in
                           [32, 1024], half Poisson, half log a ~ N(0,1) per
                           element, f ~ U[-1,1], seed 4

Mesh jitter draws from ``default_rng(seed)``; the data (f, a) draw from
``default_rng(1000 + seed)`` so a mesh does not depend on how much data is
drawn.  These inputs stand in for no public data set: they are the benchmark.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .mesh import FESpace, Mesh, cube_mesh, square_mesh

# quadrature accuracies (algebraic degree) used for each operator; these are
# the ones AFEPack's own examples use (2D: 4, 3D P1 stiffness: 2) and the
# ones that integrate the P2 stiffness/mass integrands exactly.
ACC = {
    (2, 1): (4, 4),
    (2, 2): (4, 4),
    (3, 1): (2, 4),
    (3, 2): (4, 4),
}


@dataclass
class Workload:
    name: str
    space: FESpace
    coef: np.ndarray | None      # [n_cell] per-element coefficient, or None
    f: np.ndarray                # [n_dof] or [n_dof, k] nodal data
    acc_stiff: int
    acc_mass: int

    @property
    def mesh(self) -> Mesh:
        return self.space.mesh


def _make(name, mesh, degree, coef, f):
    sp = FESpace(mesh, degree)
    acc_s, acc_m = ACC[(mesh.dim, degree)]
    return Workload(name, sp, coef, f, acc_s, acc_m)


def poisson2d_p1(n: int = 256, seed: int = 0) -> Workload:
    mesh = square_mesh(n, 0.2, seed)
    sp = FESpace(mesh, 1)
    f = np.random.default_rng(1000 + seed).uniform(-1.0, 1.0, sp.n_dof)
    return Workload(f"poisson2d_p1_{n}", sp, None, f, *ACC[(2, 1)])


def poisson3d_p1(n: int = 64, seed: int = 1) -> Workload:
    mesh = cube_mesh(n, 0.15, seed)
    sp = FESpace(mesh, 1)
    rng = np.random.default_rng(1000 + seed)
    centres = rng.uniform(0.2, 0.8, size=(8, 3))
    widths = rng.uniform(0.05, 0.2, size=8)
    x = sp.dof_point
    f = np.zeros(sp.n_dof)
    for c, s in zip(centres, widths):
        f += np.exp(-np.sum((x - c) ** 2, axis=1) / (2.0 * s * s))
    return Workload(f"poisson3d_p1_{n}", sp, None, f, *ACC[(3, 1)])


def gaussian_sources(space: FESpace, count: int, seed: int = 5, device=None):
    """Nodal data of `count` requests on one space, each drawn like the 64^3
    Poisson workload's f: a sum of 8 Gaussians with centres U[0.2,0.8]^d and
    widths U[0.05,0.2], request j from default_rng([seed, j]).  Returns an
    n x count array, or a torch tensor on `device` (evaluated there)."""
    if device is None:
        x = space.dof_point
        out = np.zeros((space.n_dof, count))
    else:
        import torch
        x = torch.from_numpy(np.ascontiguousarray(space.dof_point)).to(device)
        out = torch.zeros((space.n_dof, count), dtype=torch.float64, device=device)
    for j in range(count):
        rng = np.random.default_rng([seed, j])
        centres = rng.uniform(0.2, 0.8, size=(8, space.dof_point.shape[1]))
        widths = rng.uniform(0.05, 0.2, size=8)
        for c, s in zip(centres, widths):
            if device is None:
                out[:, j] += np.exp(-np.sum((x - c) ** 2, axis=1) / (2.0 * s * s))
            else:
                ct = torch.as_tensor(c, dtype=torch.float64, device=device)
                out[:, j] += torch.exp(-((x - ct) ** 2).sum(dim=1) / (2.0 * s * s))
    return out


def gaussian_field(n: int, length: float, rng: np.random.Generator) -> np.ndarray:
    """Squared-exponential Gaussian random field on the n x n cell-centre grid
    of the unit square, sampled by circulant embedding on a 2n x 2n torus."""
    m = 2 * n
    h = 1.0 / n
    d = np.minimum(np.arange(m), m - np.arange(m)) * h
    r2 = d[:, None] ** 2 + d[None, :] ** 2
    cov = np.exp(-r2 / (2.0 * length * length))
    lam = np.maximum(np.fft.fft2(cov).real, 0.0)
    xi = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    field = np.fft.fft2(np.sqrt(lam / (m * m)) * xi).real
    return field[:n, :n]


def contrast_coefficient(logf: np.ndarray, contrast: float) -> np.ndarray:
    """exp of an affine map of ``logf`` onto [0, ln contrast]: min 1, max = contrast."""
    lo, hi = logf.min(), logf.max()
    return np.exp((logf - lo) / (hi - lo) * np.log(contrast))


def elliptic2d_p2(n: int = 512, seed: int = 2, contrast: float = 1.0e4) -> Workload:
    mesh = square_mesh(n, 0.2, seed)
    rng = np.random.default_rng(1000 + seed)
    cell = contrast_coefficient(gaussian_field(n, 0.05, rng), contrast)  # [j, i] by cell row
    coef = np.repeat(cell.reshape(-1), 2)  # both triangles of a cell share it
    sp = FESpace(mesh, 2)
    f = np.ones(sp.n_dof)
    return Workload(f"elliptic2d_p2_{n}", sp, coef, f, *ACC[(2, 2)])


def poisson3d_p2_multi(n: int = 48, nrhs: int = 64, seed: int = 3) -> Workload:
    mesh = cube_mesh(n, 0.15, seed)
    sp = FESpace(mesh, 2)
    f = np.random.default_rng(1000 + seed).standard_normal((sp.n_dof, nrhs))
    return Workload(f"poisson3d_p2_{n}_x{nrhs}", sp, None, f, *ACC[(3, 2)])


@dataclass
class Request:
    index: int
    n: int
    variable: bool
    seed: int


def request_stream(count: int = 2000, seed: int = 4, n_min: int = 32, n_max: int = 1024):
    """The request mix of the served stream: sizes and types only; each
    request's mesh and data are made by ``request_workload``."""
    rng = np.random.default_rng(seed)
    ns = np.rint(np.exp(rng.uniform(np.log(n_min), np.log(n_max), count))).astype(int)
    var = rng.random(count) < 0.5
    return [Request(i, int(ns[i]), bool(var[i]), seed * 100000 + i) for i in range(count)]


def request_workload(req: Request) -> Workload:
    mesh = square_mesh(req.n, 0.2, req.seed)
    sp = FESpace(mesh, 1)
    rng = np.random.default_rng(1000 + req.seed)
    coef = np.exp(rng.standard_normal(mesh.n_cell)) if req.variable else None
    f = rng.uniform(-1.0, 1.0, sp.n_dof)
    return Workload(f"request{req.index}_n{req.n}", sp, coef, f, *ACC[(2, 1)])

"""Seeded synthetic simplex meshes and the AFEPack degree-of-freedom numbering.

Two mesh families cover every workload of this package:

* ``square_mesh(n)`` -- the unit square cut into an n x n grid whose cells are
  split along the (i,j)->(i+1,j+1) diagonal into two counter-clockwise
  triangles;
* ``cube_mesh(n)`` -- the unit cube cut into n^3 cubes, each Kuhn-split into six
  positively oriented tetrahedra along its main diagonal.

Interior nodes are jittered uniformly; the random draws are taken from
``numpy.random.default_rng(seed)`` in row-major node order, x before y before z.

``FESpace`` numbers the degrees of freedom exactly as AFEPack's
``FEMSpace::buildDof`` does (include/AFEPack/FEMSpace.templates.h:884-1003):
elements are visited in order, and inside an element the template geometries
are visited dimension by dimension (vertices, then edges), each geometry getting
the next free number the first time it is touched.  The element-local order of
the DOFs is the template order (``triangle.2.tmp_dof`` / ``tetrahedron.2.tmp_dof``),
and the edge basis functions are attached to template edges the way the
``.bas_fun`` files attach them (``TemplateElement.h:506-531``).  This numbering
fixes the CSR row order, so it is the contract that makes the sparsity pattern
comparable entry by entry with the reference.

``write_reference_mesh`` writes the reference's ``Mesh<DIM,DOW>`` text format
(include/AFEPack/Geometry.templates.h:471-493) so that the same mesh can be fed
to AFEPack itself.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# Template edges, as (local vertex a, local vertex b) in template order.
# triangle.tmp_geo lists edge j as the one opposite vertex j.
TRI_EDGES = np.array([[1, 2], [0, 2], [0, 1]], dtype=np.int64)
# tetrahedron.tmp_geo: 0:(0,1) 1:(0,2) 2:(0,3) 3:(2,3) 4:(1,3) 5:(1,2)
TET_EDGES = np.array([[0, 1], [0, 2], [0, 3], [2, 3], [1, 3], [1, 2]], dtype=np.int64)


@dataclass
class Mesh:
    """A conforming simplex mesh of the unit square or cube.

    coords   [n_vertex, dim] float64
    cells    [n_cell, dim+1] int64, positively oriented
    bmask    [n_vertex] uint8 bit mask of the boundary lines/planes a vertex
             lies on (bit 2*a for x_a = 0, bit 2*a+1 for x_a = 1)
    """

    dim: int
    n: int
    coords: np.ndarray
    cells: np.ndarray
    bmask: np.ndarray

    @property
    def n_vertex(self) -> int:
        return self.coords.shape[0]

    @property
    def n_cell(self) -> int:
        return self.cells.shape[0]


def _boundary_mask(ijk: np.ndarray, n: int) -> np.ndarray:
    mask = np.zeros(ijk.shape[0], dtype=np.uint8)
    for a in range(ijk.shape[1]):
        mask |= (ijk[:, a] == 0).astype(np.uint8) << (2 * a)
        mask |= (ijk[:, a] == n).astype(np.uint8) << (2 * a + 1)
    return mask


def square_mesh(n: int, jitter: float = 0.2, seed: int = 0) -> Mesh:
    """n x n split-square triangulation of [0,1]^2 (2 n^2 triangles)."""
    h = 1.0 / n
    m = n + 1
    j, i = np.divmod(np.arange(m * m, dtype=np.int64), m)
    ij = np.stack([i, j], axis=1)
    coords = ij.astype(np.float64) * h
    interior = np.all((ij > 0) & (ij < n), axis=1)
    rng = np.random.default_rng(seed)
    if jitter != 0.0:
        coords[interior] += rng.uniform(-jitter * h, jitter * h, size=(int(interior.sum()), 2))
    cj, ci = np.divmod(np.arange(n * n, dtype=np.int64), n)
    a = cj * m + ci
    b = a + 1
    c = a + m
    d = c + 1
    cells = np.empty((2 * n * n, 3), dtype=np.int64)
    cells[0::2] = np.stack([a, b, d], axis=1)
    cells[1::2] = np.stack([a, d, c], axis=1)
    return Mesh(2, n, coords, cells, _boundary_mask(ij, n))


# Kuhn paths: for each permutation of the axes (itertools.permutations order)
# the tetrahedron walks from the cube's low corner to its high corner.
_KUHN_PERMS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


def cube_mesh(n: int, jitter: float = 0.15, seed: int = 1) -> Mesh:
    """n^3 cube Kuhn-split into 6 n^3 tetrahedra."""
    h = 1.0 / n
    m = n + 1
    node = np.arange(m ** 3, dtype=np.int64)
    k, rem = np.divmod(node, m * m)
    j, i = np.divmod(rem, m)
    ijk = np.stack([i, j, k], axis=1)
    coords = ijk.astype(np.float64) * h
    interior = np.all((ijk > 0) & (ijk < n), axis=1)
    rng = np.random.default_rng(seed)
    if jitter != 0.0:
        coords[interior] += rng.uniform(-jitter * h, jitter * h, size=(int(interior.sum()), 3))
    ck, crem = np.divmod(np.arange(n ** 3, dtype=np.int64), n * n)
    cj, ci = np.divmod(crem, n)
    base = np.stack([ci, cj, ck], axis=1)
    stride = np.array([1, m, m * m], dtype=np.int64)
    cells = np.empty((6 * n ** 3, 4), dtype=np.int64)
    for p, perm in enumerate(_KUHN_PERMS):
        c = base.copy()
        verts = [c @ stride]
        for ax in perm:
            c[:, ax] += 1
            verts.append(c @ stride)
        cells[p::6] = np.stack(verts, axis=1)
    # orientation: swap the last two vertices of negatively oriented tets
    x = coords[cells]
    vol = np.einsum("ij,ij->i", np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]), x[:, 3] - x[:, 0])
    neg = vol < 0
    cells[neg, 2], cells[neg, 3] = cells[neg, 3].copy(), cells[neg, 2].copy()
    return Mesh(3, n, coords, cells, _boundary_mask(ijk, n))


def _edge_keys(mesh: Mesh) -> np.ndarray:
    """[n_cell, n_edge] int64 key min*nv+max of each template edge."""
    tmpl = TRI_EDGES if mesh.dim == 2 else TET_EDGES
    a = mesh.cells[:, tmpl[:, 0]]
    b = mesh.cells[:, tmpl[:, 1]]
    nv = mesh.n_vertex
    return np.minimum(a, b) * nv + np.maximum(a, b)


@dataclass
class FESpace:
    """Lagrange P1/P2 space on ``mesh`` with AFEPack's DOF numbering.

    elem_dof  [n_cell, nd] int32 -- global DOF of each template DOF
    dof_bmark [n_dof] int32      -- boundary mark (1 on the boundary, else 0)
    dof_point [n_dof, dim]       -- interpolation point of each DOF
    """

    mesh: Mesh
    degree: int
    elem_dof: np.ndarray = field(init=False)
    dof_bmark: np.ndarray = field(init=False)
    dof_point: np.ndarray = field(init=False)

    def __post_init__(self):
        mesh = self.mesh
        nv = mesh.n_vertex
        cells = mesh.cells
        if self.degree == 1:
            keys = cells.copy()
        elif self.degree == 2:
            keys = np.concatenate([cells, nv + _edge_keys(mesh)], axis=1)
        else:
            raise ValueError("only P1 and P2 Lagrange elements are provided")
        flat = keys.ravel()
        uniq, first = np.unique(flat, return_index=True)
        order = np.argsort(first, kind="stable")
        rank = np.empty(uniq.shape[0], dtype=np.int64)
        rank[order] = np.arange(uniq.shape[0], dtype=np.int64)
        dof = rank[np.searchsorted(uniq, flat)]
        self.elem_dof = dof.reshape(keys.shape).astype(np.int32)
        n_dof = uniq.shape[0]
        # boundary mark and interpolation point per DOF
        bm = np.zeros(n_dof, dtype=np.int32)
        pt = np.zeros((n_dof, mesh.dim), dtype=np.float64)
        nvx = mesh.dim + 1
        vdof = self.elem_dof[:, :nvx].ravel()
        vid = cells.ravel()
        bm[vdof] = (mesh.bmask[vid] != 0).astype(np.int32)
        pt[vdof] = mesh.coords[vid]
        if self.degree == 2:
            tmpl = TRI_EDGES if mesh.dim == 2 else TET_EDGES
            edof = self.elem_dof[:, nvx:].ravel()
            va = cells[:, tmpl[:, 0]].ravel()
            vb = cells[:, tmpl[:, 1]].ravel()
            bm[edof] = ((mesh.bmask[va] & mesh.bmask[vb]) != 0).astype(np.int32)
            pt[edof] = 0.5 * (mesh.coords[va] + mesh.coords[vb])
        self.dof_bmark = bm
        self.dof_point = pt

    @property
    def n_dof(self) -> int:
        return self.dof_bmark.shape[0]

    @property
    def n_element_dof(self) -> int:
        return self.elem_dof.shape[1]


def _fmt_rows(prefix: str, arr: np.ndarray) -> str:
    """Rows of integers as '<prefix> a b c' lines."""
    cols = [arr[:, c].astype(str) for c in range(arr.shape[1])]
    out = np.char.add(prefix, cols[0])
    for c in cols[1:]:
        out = np.char.add(np.char.add(out, " "), c)
    return "\n".join(out.tolist())


def _geometry_block(idx: np.ndarray, verts: np.ndarray, bnds: np.ndarray, bmark: np.ndarray) -> str:
    n = idx.shape[0]
    vline = _fmt_rows(f"{verts.shape[1]} ", verts).split("\n")
    bline = _fmt_rows(f"{bnds.shape[1]} ", bnds).split("\n")
    lines = [f"{n}"]
    ids = idx.astype(str).tolist()
    bms = bmark.astype(str).tolist()
    for q in range(n):
        lines.append(ids[q])
        lines.append(vline[q])
        lines.append(bline[q])
        lines.append(bms[q])
    return "\n".join(lines) + "\n\n"


def write_reference_mesh(mesh: Mesh, path: str) -> None:
    """Write ``mesh`` in AFEPack's internal ``Mesh<DIM,DIM>`` text format.

    Layout (Geometry.templates.h:471-493): the point count and coordinates,
    then for every dimension d = 0..DIM the geometry count followed by, per
    geometry, its index, its vertex list, its boundary list and its boundary
    mark.  A triangle's boundaries are its edges opposite v0, v1, v2; a
    tetrahedron's are its faces opposite v0..v3; a face's are its edges
    opposite its three vertices.
    """
    nv = mesh.n_vertex
    dim = mesh.dim
    parts = [f"{nv}\n"]
    fmt = " ".join(["%.17e"] * dim)
    parts.append("\n".join(fmt % tuple(r) for r in mesh.coords.tolist()) + "\n\n")
    vid = np.arange(nv, dtype=np.int64)
    vb = (mesh.bmask != 0).astype(np.int64)
    parts.append(_geometry_block(vid, vid[:, None], vid[:, None], vb))
    # edges
    ek = _edge_keys(mesh)
    ekeys, einv = np.unique(ek.ravel(), return_inverse=True)
    einv = einv.reshape(ek.shape)
    ea, eb = np.divmod(ekeys, nv)
    evert = np.stack([ea, eb], axis=1)
    ebm = ((mesh.bmask[ea] & mesh.bmask[eb]) != 0).astype(np.int64)
    parts.append(_geometry_block(np.arange(ekeys.shape[0]), evert, evert, ebm))
    eid_of = lambda a, b: np.searchsorted(ekeys, np.minimum(a, b) * nv + np.maximum(a, b))
    if dim == 2:
        # template edge j is opposite vertex j, which is the TRI_EDGES order
        parts.append(_geometry_block(np.arange(mesh.n_cell), mesh.cells, einv,
                                     np.zeros(mesh.n_cell, dtype=np.int64)))
    else:
        c = mesh.cells
        opp = [(1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)]
        tri = np.stack([np.sort(c[:, list(o)], axis=1) for o in opp], axis=1)  # [E,4,3]
        fkey = (tri[..., 0] * nv + tri[..., 1]) * nv + tri[..., 2]
        fkeys, finv = np.unique(fkey.ravel(), return_inverse=True)
        finv = finv.reshape(fkey.shape)
        fa, rem = np.divmod(fkeys, nv * nv)
        fb, fc = np.divmod(rem, nv)
        fvert = np.stack([fa, fb, fc], axis=1)
        fedge = np.stack([eid_of(fb, fc), eid_of(fa, fc), eid_of(fa, fb)], axis=1)
        fbm = ((mesh.bmask[fa] & mesh.bmask[fb] & mesh.bmask[fc]) != 0).astype(np.int64)
        parts.append(_geometry_block(np.arange(fkeys.shape[0]), fvert, fedge, fbm))
        parts.append(_geometry_block(np.arange(mesh.n_cell), c, finv,
                                     np.zeros(mesh.n_cell, dtype=np.int64)))
    with open(path, "w") as fh:
        fh.write("".join(parts))

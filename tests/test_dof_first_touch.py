"""The first-touch restatement of FEMSpace::buildDof that the GPU numbering
(afepack_gb300/csrc/assemble.cu, k_first_touch + k_number_dofs) implements,
checked on the CPU against the host numbering of mesh.py (itself checked
against AFEPack's own DOF maps in test_host.py).

A touch is slot s of element e, t = e*T + s (vertices, then edges).  The
first touch of a vertex is the lowest (cell, local vertex) on its incidence
list; that of an edge (a, b) is the lowest cell on a's list that also holds
b; a geometry's DOF number is the number of first touches before its own."""
import numpy as np
import pytest

from afepack_gb300.mesh import TET_EDGES, TRI_EDGES, FESpace, cube_mesh, square_mesh


def first_touch_numbering(cells, n_vertex, dim, degree):
    nv = dim + 1
    edges = (TRI_EDGES if dim == 2 else TET_EDGES) if degree == 2 else np.zeros((0, 2), int)
    T = nv + len(edges)
    n_cell = cells.shape[0]
    # vertex -> ascending (cell * nv + local) incidence
    flat = cells.ravel()
    order = np.argsort(flat, kind="stable")
    ptr = np.zeros(n_vertex + 1, dtype=np.int64)
    np.add.at(ptr, flat + 1, 1)
    ptr = np.cumsum(ptr)
    inc = order  # flat positions, ascending within each vertex (stable sort)
    first = np.empty(n_cell * T, dtype=np.int64)
    for e in range(n_cell):
        for s in range(T):
            t = e * T + s
            if s < nv:
                g = inc[ptr[cells[e, s]]]
                first[t] = (g // nv) * T + g % nv
                continue
            la, lb = edges[s - nv]
            a, b = cells[e, la], cells[e, lb]
            f = t
            for q in range(ptr[a], ptr[a + 1]):
                c = inc[q] // nv
                if c >= e:
                    break
                row = cells[c]
                if b not in row:
                    continue
                ja, jb = inc[q] % nv, int(np.nonzero(row == b)[0][0])
                for j, (x, y) in enumerate(edges):
                    if {x, y} == {ja, jb}:
                        f = c * T + nv + j
                break
            first[t] = f
    is_first = (first == np.arange(n_cell * T)).astype(np.int64)
    rank = np.concatenate([[0], np.cumsum(is_first)])
    return rank[first].reshape(n_cell, T)


@pytest.mark.parametrize("dim,degree,n", [(2, 1, 9), (2, 2, 7), (3, 1, 4), (3, 2, 3)])
def test_first_touch_matches_host_numbering(dim, degree, n):
    mesh = square_mesh(n, 0.2, 5) if dim == 2 else cube_mesh(n, 0.15, 5)
    host = FESpace(mesh, degree)
    got = first_touch_numbering(np.asarray(mesh.cells), mesh.n_vertex, dim, degree)
    assert np.array_equal(got, host.elem_dof)

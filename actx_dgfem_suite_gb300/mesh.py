"""Box simplex meshes: tetrahedra (3D) and triangles (2D).

Replaces ``meshmode.mesh.generation.generate_regular_rect_mesh`` as called by
the suite's builders (``actx_dgfem_suite/equations/wave.py:250-252``,
``euler.py:153-155``, ``maxwell.py:51-53``): an ``n x n x n`` grid of hexahedra,
each split into six positively oriented tetrahedra.  The vertex numbering
(C order over the (x, y, z) vertex grid), the element order (hexahedra in C
order, six tetrahedra each) and the per-hexahedron split follow meshmode's
``generate_box_mesh`` for 3D simplices; the split is translation-invariant and
conforming (every hexahedron face is cut along the same diagonal as its
neighbour's).  In 2D each square of the grid is split along its
(1, 0)-(0, 1) diagonal into two counter-clockwise triangles, (a, b, c) and
(d, c, b) with corners a = (0, 0), b = (1, 0), c = (0, 1), d = (1, 1), the
split of meshmode's ``generate_box_mesh`` for triangles.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

#: the six tetrahedra of a hexahedron, as corner labels (x, y, z bits)
HEX_TO_TETS = (
    ("000", "100", "010", "001"),
    ("101", "100", "001", "010"),
    ("101", "011", "010", "001"),
    ("100", "010", "101", "110"),
    ("011", "010", "110", "101"),
    ("011", "111", "101", "110"),
)


@dataclass(frozen=True)
class TetMesh:
    vertices: np.ndarray   # (nvertices, 3) float64
    elements: np.ndarray   # (nelements, 4) int64 vertex indices

    @property
    def nelements(self) -> int:
        return self.elements.shape[0]


def generate_box_tet_mesh(a, b, n) -> TetMesh:
    """Box ``[a, b]`` with ``n`` hexahedra per axis (``n`` int or 3-tuple),
    6 n^3 tetrahedra."""
    if np.isscalar(n):
        n = (int(n),) * 3
    n = tuple(int(k) for k in n)
    if min(n) < 1:
        raise ValueError("need at least one element per axis")
    a = np.broadcast_to(np.asarray(a, dtype=np.float64), (3,))
    b = np.broadcast_to(np.asarray(b, dtype=np.float64), (3,))
    axes = [np.linspace(a[d], b[d], n[d] + 1) for d in range(3)]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    vertices = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)

    nv = (n[0] + 1, n[1] + 1, n[2] + 1)
    I, J, K = np.meshgrid(np.arange(n[0]), np.arange(n[1]), np.arange(n[2]),
                          indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()

    def corner(label: str) -> np.ndarray:
        di, dj, dk = (int(ch) for ch in label)
        return ((I + di) * nv[1] + (J + dj)) * nv[2] + (K + dk)

    corners = {lab: corner(lab) for lab in
               ("000", "001", "010", "011", "100", "101", "110", "111")}
    tets = np.stack(
        [np.stack([corners[lab] for lab in tet], axis=1) for tet in HEX_TO_TETS],
        axis=1)  # (nhex, 6, 4)
    elements = tets.reshape(-1, 4).astype(np.int64)
    return TetMesh(vertices=vertices, elements=elements)


@dataclass(frozen=True)
class TriMesh:
    vertices: np.ndarray   # (nvertices, 2) float64
    elements: np.ndarray   # (nelements, 3) int64 vertex indices, counter-clockwise

    @property
    def nelements(self) -> int:
        return self.elements.shape[0]


def generate_box_tri_mesh(a, b, n) -> TriMesh:
    """Square ``[a, b]^2`` with ``n`` squares per axis (``n`` int or 2-tuple),
    2 n^2 triangles."""
    if np.isscalar(n):
        n = (int(n),) * 2
    n = tuple(int(k) for k in n)
    if min(n) < 1:
        raise ValueError("need at least one element per axis")
    a = np.broadcast_to(np.asarray(a, dtype=np.float64), (2,))
    b = np.broadcast_to(np.asarray(b, dtype=np.float64), (2,))
    axes = [np.linspace(a[d], b[d], n[d] + 1) for d in range(2)]
    X, Y = np.meshgrid(*axes, indexing="ij")
    vertices = np.stack([X.ravel(), Y.ravel()], axis=1)
    I, J = np.meshgrid(np.arange(n[0]), np.arange(n[1]), indexing="ij")
    I, J = I.ravel(), J.ravel()
    ny = n[1] + 1
    va, vb = I * ny + J, (I + 1) * ny + J
    vc, vd = I * ny + J + 1, (I + 1) * ny + J + 1
    tris = np.stack([np.stack([va, vb, vc], axis=1),
                     np.stack([vd, vc, vb], axis=1)], axis=1)   # (nsq, 2, 3)
    return TriMesh(vertices=vertices, elements=tris.reshape(-1, 3).astype(np.int64))

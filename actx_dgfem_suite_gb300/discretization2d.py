"""Affine geometry and edge connectivity of a conforming triangle mesh.

The 2D counterpart of :mod:`actx_dgfem_suite_gb300.discretization`: what
grudge's ``DiscretizationCollection`` supplies to the operators when the
suite's builders run with ``dim=2`` (``actx_dgfem_suite/equations/wave.py:248-270``,
``euler.py:153-166``, ``maxwell.py:50-55``):

* per element: the inverse metric ``dr/dx`` (2x2) and the Jacobian J;
* per edge: the outward unit normal and the surface Jacobian sJ (edge
  length / 2, the biunit segment having length 2);
* the face gather: for every edge node of every element the flat index
  ``e' * Np + i'`` of the matching node of the neighbour, bit 31 set on the
  boundary (the low bits then name the element's own node), as in 3D.

Device formats: metric (Nel, 2, 2); face geometry (Nel, 3, 4) holding
n_x, n_y, sJ/J and a zero pad per edge; gather (Nel, 3, Nfp) uint32.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from actx_dgfem_suite_gb300.discretization import BOUNDARY_FLAG
from actx_dgfem_suite_gb300.mesh import TriMesh, generate_box_tri_mesh
from actx_dgfem_suite_gb300.refelem import (
    TRI_FACE_OPPOSITE_VERTEX,
    TRI_FACE_VERTICES,
    TRI_NFACES,
    ReferenceTri,
    recursive_barycentric_nodes,
    reference_tri,
)


@dataclass
class DGDiscretization2D:
    order: int
    ref: ReferenceTri
    mesh: TriMesh
    jac: np.ndarray             # (Nel,) det(dx/dr)
    metric: np.ndarray          # (Nel, 2, 2) metric[e, r, x] = d r_r / d x_x
    normal: np.ndarray          # (Nel, 3, 2) outward unit normals
    face_jac: np.ndarray        # (Nel, 3) edge length / 2
    neighbor: np.ndarray        # (Nel, 3) neighbour element, -1 on the boundary
    neighbor_face: np.ndarray   # (Nel, 3) neighbour's local edge, -1 on the boundary
    ext_index: np.ndarray       # (Nel, 3, Nfp) int64 flat exterior node index
    perm_id: np.ndarray | None = None   # not used in 2D (no face-shared path)
    _cache: dict = field(default_factory=dict, repr=False)

    dim = 2

    @property
    def nelements(self) -> int:
        return self.jac.shape[0]

    @property
    def np_(self) -> int:
        return self.ref.np_

    @property
    def nfp(self) -> int:
        return self.ref.nfp

    @property
    def is_boundary(self) -> np.ndarray:
        return self.neighbor < 0

    def nodes(self) -> np.ndarray:
        """(2, Nel, Np) physical node coordinates (``dcoll.nodes()``)."""
        if "nodes" not in self._cache:
            bary = recursive_barycentric_nodes(2, self.order)   # (Np, 3)
            ev = self.mesh.vertices[self.mesh.elements]          # (Nel, 3, 2)
            self._cache["nodes"] = np.einsum("iv,evx->xei", bary, ev)
        return self._cache["nodes"]

    def metric_flat(self) -> np.ndarray:
        """(Nel, 4) float64, row-major ``dr/dx``."""
        return np.ascontiguousarray(self.metric.reshape(-1, 4))

    def face_geometry(self) -> np.ndarray:
        """(Nel, 3, 4) float64: n_x, n_y, sJ/J, 0 per edge."""
        out = np.zeros((self.nelements, TRI_NFACES, 4))
        out[:, :, :2] = self.normal
        out[:, :, 2] = self.face_jac / self.jac[:, None]
        return out

    def gather_index(self) -> np.ndarray:
        """(Nel, 3, Nfp) uint32 flat exterior node index, bit 31 set on
        boundary edges."""
        if self.nelements * self.np_ >= int(BOUNDARY_FLAG):
            raise ValueError("mesh too large for 31-bit gather indices")
        idx = self.ext_index.astype(np.uint32)
        idx[self.is_boundary] |= BOUNDARY_FLAG
        return idx


def make_discretization_2d(mesh: TriMesh, order: int) -> DGDiscretization2D:
    ref = reference_tri(order)
    verts = mesh.vertices
    el = mesh.elements
    nel = el.shape[0]
    ev = verts[el]                                        # (Nel, 3, 2)
    jmat = 0.5 * np.stack([ev[:, 1] - ev[:, 0], ev[:, 2] - ev[:, 0]], axis=2)  # (Nel, x, r)
    jac = jmat[:, 0, 0] * jmat[:, 1, 1] - jmat[:, 0, 1] * jmat[:, 1, 0]
    if np.any(jac <= 0):
        raise ValueError("mesh has clockwise elements")
    metric = np.linalg.inv(jmat)                          # (Nel, r, x)

    fv = np.array(TRI_FACE_VERTICES)                      # (3, 2)
    p0, p1 = ev[:, fv[:, 0]], ev[:, fv[:, 1]]             # (Nel, 3, 2)
    t = p1 - p0
    length = np.linalg.norm(t, axis=2)
    nrm = np.stack([t[..., 1], -t[..., 0]], axis=2) / length[..., None]
    opp = ev[:, np.array(TRI_FACE_OPPOSITE_VERTEX)]       # (Nel, 3, 2)
    sgn = np.sign(np.einsum("efx,efx->ef", nrm, p0 - opp))
    normal = sgn[..., None] * nrm
    face_jac = length / 2.0

    # {{{ edge matching

    gverts = el[:, fv].reshape(-1, 2)                     # (Nel*3, 2) global ids
    s = np.sort(gverts, axis=1)
    keys = s[:, 0] * (verts.shape[0] + 1) + s[:, 1]
    order_ = np.argsort(keys, kind="stable")
    ks = keys[order_]
    same = ks[1:] == ks[:-1]
    if np.any(same[1:] & same[:-1]):
        raise ValueError("non-manifold mesh: an edge is shared by > 2 elements")
    first = order_[:-1][same]
    second = order_[1:][same]
    neighbor = np.full(nel * TRI_NFACES, -1, dtype=np.int64)
    neighbor_face = np.full(nel * TRI_NFACES, -1, dtype=np.int64)
    reversed_ = np.zeros(nel * TRI_NFACES, dtype=bool)
    for a_, b_ in ((first, second), (second, first)):
        neighbor[a_] = b_ // TRI_NFACES
        neighbor_face[a_] = b_ % TRI_NFACES
        reversed_[a_] = gverts[a_, 0] != gverts[b_, 0]

    # }}}

    npn, nfp = ref.np_, ref.nfp
    fnodes = ref.face_nodes                                # (3, Nfp)
    e_of = np.repeat(np.arange(nel, dtype=np.int64), TRI_NFACES)
    f_of = np.tile(np.arange(TRI_NFACES, dtype=np.int64), nel)
    ext = e_of[:, None] * npn + fnodes[f_of]               # (Nel*3, Nfp)
    interior = neighbor >= 0
    nb_nodes = fnodes[neighbor_face[interior]]             # (nint, Nfp)
    rev = reversed_[interior]
    nb_nodes = np.where(rev[:, None], nb_nodes[:, ::-1], nb_nodes)
    ext[interior] = neighbor[interior][:, None] * npn + nb_nodes

    return DGDiscretization2D(
        order=order, ref=ref, mesh=mesh, jac=jac, metric=metric,
        normal=normal, face_jac=face_jac,
        neighbor=neighbor.reshape(nel, TRI_NFACES),
        neighbor_face=neighbor_face.reshape(nel, TRI_NFACES),
        ext_index=ext.reshape(nel, TRI_NFACES, nfp))


def make_box_discretization_2d(order: int, n, a=-0.5, b=0.5) -> DGDiscretization2D:
    """Discretisation of the square [a, b]^2 with ``n`` squares per axis."""
    return make_discretization_2d(generate_box_tri_mesh(a, b, n), order)

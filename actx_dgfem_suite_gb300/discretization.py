"""Affine geometry and face connectivity of a conforming tetrahedral mesh.

Replaces what grudge's ``DiscretizationCollection`` supplies to the RHS
operators on the suite's box meshes (``actx_dgfem_suite/equations/wave.py:261-270``):

* per element: the inverse metric ``dr/dx`` (3x3) and the volume Jacobian J
  (affine simplices: constant per element, so grudge's einsums carry them as
  ``re`` / ``xre`` / ``e`` operands, see
  ``actx_dgfem_suite/arraycontext/mass_inverse_fuser.py:20-76``);
* per face: the outward unit normal and the surface Jacobian sJ;
* the face gather: for every face node of every element the flat index
  ``e' * Np + i'`` of the matching node of the neighbouring element, i.e. the
  unsigned index array that ``fold_constants_in_einsum_indirections``
  (``actx_dgfem_suite/arraycontext/constants_folder.py:69-100``) folds the
  trace-pair gathers into.  Boundary faces (meshmode ``BTAG_ALL``) point at the
  element's own node and carry the flag bit ``BOUNDARY_FLAG``.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from itertools import permutations

import numpy as np

from actx_dgfem_suite_gb300.mesh import TetMesh, generate_box_tet_mesh
from actx_dgfem_suite_gb300.refelem import (
    FACE_OPPOSITE_VERTEX,
    FACE_VERTICES,
    NFACES,
    ReferenceTet,
    recursive_barycentric_nodes,
    reference_tet,
)

#: bit 31 of a gather index marks a boundary face node
BOUNDARY_FLAG = np.uint32(1 << 31)
_PERMS = list(permutations(range(3)))
_PERM_CODE_TO_ID = np.full(27, -1, dtype=np.int64)
for _pid, _p in enumerate(_PERMS):
    _PERM_CODE_TO_ID[_p[0] * 9 + _p[1] * 3 + _p[2]] = _pid


@dataclass
class DGDiscretization:
    order: int
    ref: ReferenceTet
    mesh: TetMesh
    jac: np.ndarray             # (Nel,) volume Jacobian det(dx/dr)
    metric: np.ndarray          # (Nel, 3, 3) metric[e, r, x] = d r_r / d x_x
    normal: np.ndarray          # (Nel, 4, 3) outward unit normals
    face_jac: np.ndarray        # (Nel, 4) surface Jacobian sJ (area / 2)
    neighbor: np.ndarray        # (Nel, 4) neighbour element, -1 on the boundary
    neighbor_face: np.ndarray   # (Nel, 4) neighbour's local face, -1 on the boundary
    ext_index: np.ndarray       # (Nel, 4, Nfp) int64 flat exterior node index
    perm_id: np.ndarray | None = None  # (Nel, 4) gluing permutation id, -1 on the boundary
    _cache: dict = field(default_factory=dict, repr=False)

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
        """(3, Nel, Np) physical node coordinates (``dcoll.nodes()``)."""
        if "nodes" not in self._cache:
            bary = recursive_barycentric_nodes(3, self.order)   # (Np, 4)
            ev = self.mesh.vertices[self.mesh.elements]          # (Nel, 4, 3)
            self._cache["nodes"] = np.einsum("iv,evx->xei", bary, ev)
        return self._cache["nodes"]

    # {{{ device formats

    def metric_flat(self) -> np.ndarray:
        """(Nel, 9) float64, row-major ``dr/dx``."""
        return np.ascontiguousarray(self.metric.reshape(-1, 9))

    def face_geometry(self) -> np.ndarray:
        """(Nel, 4, 4) float64: n_x, n_y, n_z, sJ/J per face."""
        out = np.empty((self.nelements, NFACES, 4))
        out[:, :, :3] = self.normal
        out[:, :, 3] = self.face_jac / self.jac[:, None]
        return out

    def face_partner(self) -> np.ndarray:
        """(Nel, 4, Nfp) int32 flat face-point index (e' * 4 + f') * Nfp + j'
        of the face point glued to each face point, -1 on the boundary.  The
        adjoint uses it to turn the transpose of the face gather into a
        gather (deterministic, no atomics)."""
        if self.perm_id is None:
            raise ValueError("discretisation was built without gluing permutations")
        nfp = self.nfp
        perm_maps = np.stack([self.ref.face_perm[p] for p in _PERMS])  # (6, Nfp)
        out = np.full((self.nelements, NFACES, nfp), -1, dtype=np.int64)
        inter = self.neighbor >= 0
        nb = self.neighbor[inter]
        nf = self.neighbor_face[inter]
        pm = perm_maps[self.perm_id[inter]]
        out[inter] = (nb * NFACES + nf)[:, None] * nfp + pm
        if out.max() >= (1 << 31):
            raise ValueError("mesh too large for 31-bit face-point indices")
        return out.astype(np.int32)

    def gather_index(self) -> np.ndarray:
        """(Nel, 4, Nfp) uint32 flat exterior node index, bit 31 set on
        boundary faces (the low bits then name the element's own node)."""
        if self.nelements * self.np_ >= int(BOUNDARY_FLAG):
            raise ValueError("mesh too large for 31-bit gather indices")
        idx = self.ext_index.astype(np.uint32)
        idx[self.is_boundary] |= BOUNDARY_FLAG
        return idx

    # }}}


def _face_keys(face_verts: np.ndarray, nvertices: int) -> np.ndarray:
    s = np.sort(face_verts, axis=1)
    if nvertices < (1 << 21):
        return (s[:, 0] << 42) | (s[:, 1] << 21) | s[:, 2]
    # general case: rank the sorted triples
    _, inv = np.unique(s, axis=0, return_inverse=True)
    return inv.astype(np.int64)


def make_discretization(mesh: TetMesh, order: int) -> DGDiscretization:
    ref = reference_tet(order)
    verts = mesh.vertices
    el = mesh.elements
    nel = el.shape[0]
    ev = verts[el]                                        # (Nel, 4, 3)

    # dx/dr: columns are half the spanning vectors of the biunit map
    jmat = 0.5 * np.stack([ev[:, 1] - ev[:, 0], ev[:, 2] - ev[:, 0],
                           ev[:, 3] - ev[:, 0]], axis=2)  # (Nel, x, r)
    jac = np.linalg.det(jmat)
    if np.any(jac <= 0):
        raise ValueError("mesh has non-positively oriented elements")
    metric = np.linalg.inv(jmat)                          # (Nel, r, x)

    # gradients of the barycentric coordinates: lambda_1 = (r+1)/2, ...
    grad_bary = np.empty((nel, 4, 3))
    grad_bary[:, 1:, :] = 0.5 * metric
    grad_bary[:, 0, :] = -grad_bary[:, 1:, :].sum(axis=1)
    opp = np.array(FACE_OPPOSITE_VERTEX)
    gn = -grad_bary[:, opp, :]                            # outward direction
    normal = gn / np.linalg.norm(gn, axis=2, keepdims=True)

    fv = np.array(FACE_VERTICES)                          # (4, 3)
    fpts = ev[:, fv, :]                                   # (Nel, 4, 3 verts, 3)
    area = 0.5 * np.linalg.norm(
        np.cross(fpts[:, :, 1] - fpts[:, :, 0], fpts[:, :, 2] - fpts[:, :, 0]),
        axis=2)
    face_jac = area / 2.0                                 # biunit triangle area 2

    # {{{ face matching

    face_verts = el[:, fv].reshape(-1, 3)                 # (Nel*4, 3) global ids
    keys = _face_keys(face_verts, verts.shape[0])
    order_ = np.argsort(keys, kind="stable")
    ks = keys[order_]
    same = ks[1:] == ks[:-1]
    if np.any(same[1:] & same[:-1]):
        raise ValueError("non-manifold mesh: a face is shared by > 2 elements")
    first = order_[:-1][same]
    second = order_[1:][same]

    neighbor = np.full(nel * NFACES, -1, dtype=np.int64)
    neighbor_face = np.full(nel * NFACES, -1, dtype=np.int64)
    perm_id = np.full(nel * NFACES, -1, dtype=np.int64)

    def _perm(f_own: np.ndarray, f_nb: np.ndarray) -> np.ndarray:
        g_own = face_verts[f_own]                         # (npair, 3)
        g_nb = face_verts[f_nb]
        eq = g_nb[:, :, None] == g_own[:, None, :]        # [x, y]: nb x == own y
        p = np.argmax(eq, axis=2)
        return _PERM_CODE_TO_ID[p[:, 0] * 9 + p[:, 1] * 3 + p[:, 2]]

    for a_, b_ in ((first, second), (second, first)):
        neighbor[a_] = b_ // NFACES
        neighbor_face[a_] = b_ % NFACES
        perm_id[a_] = _perm(a_, b_)

    # }}}

    # {{{ exterior node indices

    npn, nfp = ref.np_, ref.nfp
    fnodes = ref.face_nodes                                # (4, Nfp)
    perm_maps = np.stack([ref.face_perm[p] for p in _PERMS])  # (6, Nfp)
    e_of = np.repeat(np.arange(nel, dtype=np.int64), NFACES)
    f_of = np.tile(np.arange(NFACES, dtype=np.int64), nel)
    own = e_of[:, None] * npn + fnodes[f_of]               # (Nel*4, Nfp)
    ext = own.copy()
    interior = neighbor >= 0
    nb_e = neighbor[interior]
    nb_f = neighbor_face[interior]
    pm = perm_maps[perm_id[interior]]                      # (nint, Nfp)
    ext[interior] = nb_e[:, None] * npn + fnodes[nb_f[:, None], pm]

    # }}}

    return DGDiscretization(
        order=order, ref=ref, mesh=mesh, jac=jac, metric=metric,
        normal=normal, face_jac=face_jac,
        neighbor=neighbor.reshape(nel, NFACES),
        neighbor_face=neighbor_face.reshape(nel, NFACES),
        ext_index=ext.reshape(nel, NFACES, nfp),
        perm_id=perm_id.reshape(nel, NFACES))


def affine_image(disc: DGDiscretization, scale: float,
                 offset) -> DGDiscretization:
    """The discretisation of the mesh mapped by x -> scale * x + offset
    (scale > 0): connectivity and normals are shared, metric terms rescaled."""
    if not scale > 0:
        raise ValueError("scale must be positive")
    offset = np.broadcast_to(np.asarray(offset, dtype=np.float64), (3,))
    mesh = TetMesh(vertices=disc.mesh.vertices * scale + offset,
                   elements=disc.mesh.elements)
    return DGDiscretization(
        order=disc.order, ref=disc.ref, mesh=mesh, jac=disc.jac * scale**3,
        metric=disc.metric / scale, normal=disc.normal,
        face_jac=disc.face_jac * scale**2, neighbor=disc.neighbor,
        neighbor_face=disc.neighbor_face, ext_index=disc.ext_index,
        perm_id=disc.perm_id)


def union_discretization(discs: list[DGDiscretization]) -> tuple[DGDiscretization, np.ndarray]:
    """One discretisation holding independent meshes side by side.

    Elements, geometry and gather indices are concatenated; every member's
    exterior indices are shifted by its element offset, so no face connects
    two members.  Returns the union and the element offsets (len + 1)."""
    if not discs:
        raise ValueError("need at least one member")
    if any(getattr(d, "dim", 3) != 3 for d in discs):
        raise NotImplementedError("ensembles are built from tetrahedral meshes")
    order = discs[0].order
    if any(d.order != order for d in discs):
        raise ValueError("all members must have the same order")
    npn = discs[0].np_
    nels = np.array([d.nelements for d in discs], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(nels)])
    voffs = np.concatenate([[0], np.cumsum([d.mesh.vertices.shape[0] for d in discs])])
    mesh = TetMesh(vertices=np.concatenate([d.mesh.vertices for d in discs]),
                   elements=np.concatenate([d.mesh.elements + voffs[k]
                                            for k, d in enumerate(discs)]))

    def shifted_neighbor(k, d):
        nb = d.neighbor.copy()
        nb[nb >= 0] += offs[k]
        return nb

    union = DGDiscretization(
        order=order, ref=discs[0].ref, mesh=mesh,
        jac=np.concatenate([d.jac for d in discs]),
        metric=np.concatenate([d.metric for d in discs]),
        normal=np.concatenate([d.normal for d in discs]),
        face_jac=np.concatenate([d.face_jac for d in discs]),
        neighbor=np.concatenate([shifted_neighbor(k, d) for k, d in enumerate(discs)]),
        neighbor_face=np.concatenate([d.neighbor_face for d in discs]),
        ext_index=np.concatenate([d.ext_index + offs[k] * npn
                                  for k, d in enumerate(discs)]),
        perm_id=(None if any(d.perm_id is None for d in discs)
                 else np.concatenate([d.perm_id for d in discs])))
    return union, offs


_UNIT_BOX_CACHE: dict = {}


def make_box_discretization(order: int, n, a=-0.5, b=0.5) -> DGDiscretization:
    """Discretisation of the box [a, b]^3 with ``n`` hexahedra per axis.

    For cubes (scalar ``a``, ``b``, ``n``) the unit-cube discretisation of the
    most recent (order, n) is cached and mapped affinely, so building the same
    grid on several boxes costs one connectivity pass."""
    if np.isscalar(a) and np.isscalar(b) and np.isscalar(n):
        key = (order, int(n))
        base = _UNIT_BOX_CACHE.get(key)
        if base is None:
            _UNIT_BOX_CACHE.clear()
            base = make_discretization(generate_box_tet_mesh(0.0, 1.0, n), order)
            _UNIT_BOX_CACHE[key] = base
        return affine_image(base, float(b) - float(a), float(a))
    return make_discretization(generate_box_tet_mesh(a, b, n), order)


def clear_box_cache() -> None:
    _UNIT_BOX_CACHE.clear()

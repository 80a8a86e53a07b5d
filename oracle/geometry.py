"""Geometry and trace pairs by coordinate matching (oracle; test infrastructure).

Restates what grudge's ``DiscretizationCollection`` and
``op.interior_trace_pairs`` / ``op.bdry_trace_pair`` supply to the operators
(``actx_dgfem_suite/equations/wave.py:148-199``), computed independently of the
product's connectivity code:

* faces are glued by a dictionary on sorted vertex triples;
* face nodes are the volume nodes found at the face-node reference
  coordinates; exterior values come from the neighbour node at the same
  physical position (nearest-point matching, checked to round-off);
* normals from cross products of face edges, oriented away from the
  opposite vertex; sJ = face area / 2 and J = volume / (4/3).

For triangle meshes (:func:`build_oracle_disc_2d`) the faces are the edges,
glued by sorted vertex pairs, with normals rotated from the edge vectors and
sJ = edge length / 2.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from oracle.refelem import FACES as FACE_VERTICES
from oracle.refelem import TRI_EDGES
from oracle.refops import OracleRefOps, oracle_ref_ops, oracle_ref_ops_2d


@dataclass
class OracleDisc:
    order: int
    ops: OracleRefOps
    nel: int
    jac: np.ndarray         # (Nel,)
    jg: np.ndarray          # (Nel, d, d) J * dr_r/dx_x  (grudge: times_area_element)
    metric: np.ndarray      # (Nel, d, d) dr_r/dx_x
    normal: np.ndarray      # (Nel, F, d)   (3D: F = 4 faces; 2D: F = 3 edges)
    sj: np.ndarray          # (Nel, F)
    nodes: np.ndarray       # (d, Nel, Np) physical node coordinates
    int_idx: np.ndarray     # (Nel, F, Nfp) flat index of the interior trace node
    ext_idx: np.ndarray     # (Nel, F, Nfp) flat index of the exterior trace node
    bdry: np.ndarray        # (Nel, F) bool: face on the boundary (BTAG_ALL)

    @property
    def dim(self) -> int:
        return self.normal.shape[-1]


def build_oracle_disc(vertices: np.ndarray, elements: np.ndarray,
                      order: int) -> OracleDisc:
    ops = oracle_ref_ops(order)
    nel = elements.shape[0]
    ev = vertices[elements]                           # (Nel, 4, 3)
    jm = 0.5 * np.stack([ev[:, 1] - ev[:, 0], ev[:, 2] - ev[:, 0],
                         ev[:, 3] - ev[:, 0]], axis=2)  # dx/dr (x, r)
    jac = np.linalg.det(jm)
    metric = np.linalg.inv(jm)                        # (r, x)
    jg = jac[:, None, None] * metric
    ref = ops.nodes
    nodes = (ev[:, 0, :][:, None, :]
             + np.einsum("exr,ir->eix", jm, ref + 1.0)).transpose(2, 0, 1)

    normal = np.zeros((nel, 4, 3))
    sj = np.zeros((nel, 4))
    for f, fv in enumerate(FACE_VERTICES):
        p0, p1, p2 = ev[:, fv[0]], ev[:, fv[1]], ev[:, fv[2]]
        cr = np.cross(p1 - p0, p2 - p0)
        area = 0.5 * np.linalg.norm(cr, axis=1)
        opp = [v for v in range(4) if v not in fv][0]
        sgn = np.sign(np.einsum("ex,ex->e", cr, p0 - ev[:, opp]))
        normal[:, f] = sgn[:, None] * cr / (2 * area)[:, None]
        sj[:, f] = area / 2.0

    npn = ref.shape[0]
    nfp = ops.face_node_coords.shape[1]
    # face nodes: the volume nodes at the face-node reference coordinates
    fidx = np.zeros((4, nfp), dtype=np.int64)
    for f in range(4):
        d = np.linalg.norm(ref[None, :, :] - ops.face_node_coords[f][:, None, :],
                           axis=2)
        fidx[f] = np.argmin(d, axis=1)
        assert np.all(d[np.arange(nfp), fidx[f]] < 1e-12)

    int_idx = np.arange(nel)[:, None, None] * npn + fidx[None, :, :]
    ext_idx = int_idx.copy()
    bdry = np.ones((nel, 4), dtype=bool)

    faces: dict = {}
    for e in range(nel):
        for f, fv in enumerate(FACE_VERTICES):
            key = tuple(sorted(int(elements[e, v]) for v in fv))
            faces.setdefault(key, []).append((e, f))
    xf = nodes.reshape(3, -1)
    pairs = []
    for key, lst in faces.items():
        if len(lst) == 2:
            pairs.append(lst[0] + lst[1])
            pairs.append(lst[1] + lst[0])
        elif len(lst) > 2:
            raise ValueError("non-manifold mesh")
    if pairs:
        pairs = np.array(pairs)
        e1, f1, e2, f2 = pairs.T
        own = int_idx[e1, f1]                          # (npair, Nfp)
        nb = int_idx[e2, f2]
        dist = np.linalg.norm(xf[:, own][:, :, :, None] - xf[:, nb][:, :, None, :],
                              axis=0)                   # (npair, Nfp, Nfp)
        jmatch = np.argmin(dist, axis=2)
        dmin = np.take_along_axis(dist, jmatch[:, :, None], axis=2)
        assert np.all(dmin < 1e-10), "face nodes do not match"
        ext_idx[e1, f1] = np.take_along_axis(nb, jmatch, axis=1)
        bdry[e1, f1] = False
    return OracleDisc(order=order, ops=ops, nel=nel, jac=jac, jg=jg,
                      metric=metric, normal=normal, sj=sj, nodes=nodes,
                      int_idx=int_idx, ext_idx=ext_idx, bdry=bdry)


def _match_exterior(nodes, int_idx, pairs_list):
    """Exterior trace indices by nearest physical node of the glued face."""
    ext_idx = int_idx.copy()
    bdry = np.ones(int_idx.shape[:2], dtype=bool)
    if pairs_list:
        pairs = np.array(pairs_list)
        e1, f1, e2, f2 = pairs.T
        xf = nodes.reshape(nodes.shape[0], -1)
        own = int_idx[e1, f1]
        nb = int_idx[e2, f2]
        dist = np.linalg.norm(xf[:, own][:, :, :, None] - xf[:, nb][:, :, None, :],
                              axis=0)
        jmatch = np.argmin(dist, axis=2)
        dmin = np.take_along_axis(dist, jmatch[:, :, None], axis=2)
        assert np.all(dmin < 1e-10), "face nodes do not match"
        ext_idx[e1, f1] = np.take_along_axis(nb, jmatch, axis=1)
        bdry[e1, f1] = False
    return ext_idx, bdry


def build_oracle_disc_2d(vertices: np.ndarray, elements: np.ndarray,
                         order: int) -> OracleDisc:
    """The oracle discretisation of a triangle mesh (vertices (nv, 2),
    counter-clockwise elements (Nel, 3))."""
    ops = oracle_ref_ops_2d(order)
    nel = elements.shape[0]
    ev = vertices[elements]                                  # (Nel, 3, 2)
    jm = 0.5 * np.stack([ev[:, 1] - ev[:, 0], ev[:, 2] - ev[:, 0]], axis=2)
    jac = np.linalg.det(jm)
    metric = np.linalg.inv(jm)
    jg = jac[:, None, None] * metric
    ref = ops.nodes
    nodes = (ev[:, 0, :][:, None, :]
             + np.einsum("exr,ir->eix", jm, ref + 1.0)).transpose(2, 0, 1)
    normal = np.zeros((nel, 3, 2))
    sj = np.zeros((nel, 3))
    for f, (a, b) in enumerate(TRI_EDGES):
        opp = [v for v in range(3) if v not in (a, b)][0]
        t = ev[:, b] - ev[:, a]
        length = np.linalg.norm(t, axis=1)
        nrm = np.stack([t[:, 1], -t[:, 0]], axis=1) / length[:, None]
        sgn = np.sign(np.einsum("ex,ex->e", nrm, ev[:, a] - ev[:, opp]))
        normal[:, f] = sgn[:, None] * nrm
        sj[:, f] = length / 2.0
    npn = ref.shape[0]
    nfp = ops.face_node_coords.shape[1]
    fidx = np.zeros((3, nfp), dtype=np.int64)
    for f in range(3):
        d = np.linalg.norm(ref[None, :, :] - ops.face_node_coords[f][:, None, :], axis=2)
        fidx[f] = np.argmin(d, axis=1)
        assert np.all(d[np.arange(nfp), fidx[f]] < 1e-12)
    int_idx = np.arange(nel)[:, None, None] * npn + fidx[None, :, :]
    edges: dict = {}
    for e in range(nel):
        for f, (a, b) in enumerate(TRI_EDGES):
            key = tuple(sorted((int(elements[e, a]), int(elements[e, b]))))
            edges.setdefault(key, []).append((e, f))
    pairs = []
    for lst in edges.values():
        if len(lst) == 2:
            pairs.append(lst[0] + lst[1])
            pairs.append(lst[1] + lst[0])
        elif len(lst) > 2:
            raise ValueError("non-manifold mesh")
    ext_idx, bdry = _match_exterior(nodes, int_idx, pairs)
    return OracleDisc(order=order, ops=ops, nel=nel, jac=jac, jg=jg,
                      metric=metric, normal=normal, sj=sj, nodes=nodes,
                      int_idx=int_idx, ext_idx=ext_idx, bdry=bdry)

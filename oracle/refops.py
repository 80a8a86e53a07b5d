"""Reference-element matrices by quadrature (oracle; test infrastructure).

Assembles, on the biunit tetrahedron and with the nodal (Lagrange) basis on
the volume node set, the matrices grudge builds through modepy:

* mass ``M[i, j] = int phi_i phi_j``;
* stiffness transpose ``ST[r, i, j] = int d_r phi_i phi_j`` (grudge's
  ``_reference_stiffness_transpose_matrices``, used by ``weak_local_grad`` /
  ``weak_local_div``);
* strong derivative ``D[r] = M^-1 ST[r]^T`` (``local_d_dx``);
* face mass ``E[k, f, j] = int_{face f} phi_k l_j`` over the face's own
  biunit-triangle parametrisation, ``l_j`` the Lagrange basis on the face
  nodes (``reference_face_mass_matrix``).

Every integral uses a collapsed Gauss-Legendre rule exact for the
integrand's degree, so none relies on the face nodes being volume nodes.
Nodes, basis and quadrature come from :mod:`oracle.refelem`, which shares no
code with the product; the assembly runs in 32-digit arithmetic and rounds
each matrix to FP64 once.
"""

from __future__ import annotations

from dataclasses import dataclass
from functools import lru_cache

import numpy as np

from oracle.refelem import (
    FACES,
    MP,
    TET_VERTICES,
    TRI_EDGES,
    TRI_VERTICES,
    gauss_01_mp,
    gll_01_mp,
    legendre,
    modal_basis,
    modal_basis_grads,
    tet_nodes,
    tet_nodes_mp,
    tet_rule,
    tri_nodes,
    tri_nodes_mp,
    tri_rule,
)


@dataclass(frozen=True)
class OracleRefOps:
    order: int
    nodes: np.ndarray   # (Np, 3)
    mass: np.ndarray    # (Np, Np)
    stiff_t: np.ndarray # (3, Np, Np)
    diff: np.ndarray    # (3, Np, Np)
    face_mass: np.ndarray  # (Np, 4, Nfp)
    face_node_coords: np.ndarray  # (4, Nfp, 3) reference coords of face nodes


def _mat(rows) -> "MP.matrix":
    return MP.matrix(rows)


def _f64(m) -> np.ndarray:
    return np.array([[float(m[i, j]) for j in range(m.cols)] for i in range(m.rows)])


@lru_cache(maxsize=None)
def oracle_ref_ops(order: int) -> OracleRefOps:
    """The reference matrices, assembled by quadrature in extended precision
    (32 digits) and rounded to FP64 once at the end."""
    nodes_mp = tet_nodes_mp(order)
    np_ = len(nodes_mp)
    q, w = tet_rule(order + 2)                               # exact to degree 2N + 1
    vinv = _mat(modal_basis(order, nodes_mp)) ** -1          # modal -> nodal
    lag = _mat(modal_basis(order, q)) * vinv                 # (nq, Np)
    dlag = [_mat(g) * vinv for g in modal_basis_grads(order, q)]
    nq = len(w)
    wd = MP.diag(w)
    mass = lag.T * wd * lag
    stiff_t = [d.T * wd * lag for d in dlag]                 # ST[r][i][j] = int d_r phi_i phi_j
    minv = mass ** -1
    diff = [minv * st.T for st in stiff_t]

    fref = tri_nodes_mp(order)
    nfp = len(fref)
    v2inv = _mat(modal_basis(order, fref)) ** -1
    q2, w2 = tri_rule(order + 1)                             # exact to degree 2N
    lag2 = _mat(modal_basis(order, q2)) * v2inv              # (nq2, Nfp)
    w2d = MP.diag(w2)

    def bary2(x2):  # biunit-triangle coordinates -> barycentric
        l1, l2 = (x2[0] + 1) / 2, (x2[1] + 1) / 2
        return (1 - l1 - l2, l1, l2)

    emat = np.zeros((np_, 4, nfp))
    fcoords = np.zeros((4, nfp, 3))
    for f, fv in enumerate(FACES):
        fverts = [[int(v) for v in TET_VERTICES[k]] for k in fv]   # (3, 3)

        def on_face(x2):
            b = bary2(x2)
            return tuple(sum(b[k] * fverts[k][x] for k in range(3)) for x in range(3))

        vol_lag = _mat(modal_basis(order, [on_face(x) for x in q2])) * vinv   # (nq2, Np)
        emat[:, f, :] = _f64(vol_lag.T * w2d * lag2)
        fcoords[f] = np.array([[float(v) for v in on_face(x)] for x in fref])
    del nq
    return OracleRefOps(order=order, nodes=tet_nodes(order), mass=_f64(mass),
                        stiff_t=np.stack([_f64(st) for st in stiff_t]),
                        diff=np.stack([_f64(d) for d in diff]), face_mass=emat,
                        face_node_coords=fcoords)


@lru_cache(maxsize=None)
def oracle_ref_ops_2d(order: int) -> OracleRefOps:
    """The reference-triangle matrices (2D meshes), assembled like
    :func:`oracle_ref_ops`: volume integrals by the collapsed rule, edge
    integrals by Gauss-Legendre over each edge's own [-1, 1]
    parametrisation with the Lagrange basis on the edge's GLL points."""
    nodes_mp = tri_nodes_mp(order)
    np_ = len(nodes_mp)
    q, w = tri_rule(order + 1)                               # exact to degree 2N
    vinv = _mat(modal_basis(order, nodes_mp)) ** -1
    lag = _mat(modal_basis(order, q)) * vinv
    dlag = [_mat(g) * vinv for g in modal_basis_grads(order, q)]
    wd = MP.diag(w)
    mass = lag.T * wd * lag
    stiff_t = [d.T * wd * lag for d in dlag]
    minv = mass ** -1
    diff = [minv * st.T for st in stiff_t]

    # edge nodes: GLL points on [-1, 1]; Lagrange basis through them
    g = [2 * x - 1 for x in gll_01_mp(order)]
    nfp = len(g)
    v1inv = _mat([[legendre(k, x)[0] for k in range(order + 1)] for x in g]) ** -1
    u, wu = gauss_01_mp(order + 1)                           # exact to degree 2N + 1
    s1 = [2 * x - 1 for x in u]
    w1 = MP.diag([2 * x for x in wu])
    lag1 = _mat([[legendre(k, x)[0] for k in range(order + 1)] for x in s1]) * v1inv
    emat = np.zeros((np_, 3, nfp))
    fcoords = np.zeros((3, nfp, 2))
    for f, (a, b) in enumerate(TRI_EDGES):
        va, vb = [int(v) for v in TRI_VERTICES[a]], [int(v) for v in TRI_VERTICES[b]]

        def on_edge(t):   # t in [-1, 1] from vertex a to vertex b
            return tuple(((1 - t) * va[x] + (1 + t) * vb[x]) / 2 for x in range(2))

        vol_lag = _mat(modal_basis(order, [on_edge(t) for t in s1])) * vinv
        emat[:, f, :] = _f64(vol_lag.T * w1 * lag1)
        fcoords[f] = np.array([[float(v) for v in on_edge(t)] for t in g])
    return OracleRefOps(order=order, nodes=tri_nodes(order), mass=_f64(mass),
                        stiff_t=np.stack([_f64(st) for st in stiff_t]),
                        diff=np.stack([_f64(d) for d in diff]), face_mass=emat,
                        face_node_coords=fcoords)

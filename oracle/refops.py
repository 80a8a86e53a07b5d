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
code with the product.
"""

from __future__ import annotations

from dataclasses import dataclass
from functools import lru_cache

import numpy as np

from oracle.refelem import (
    FACES,
    TET_VERTICES,
    modal_basis_grads,
    modal_basis,
    tet_nodes,
    tet_rule,
    tri_nodes,
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


@lru_cache(maxsize=None)
def oracle_ref_ops(order: int) -> OracleRefOps:
    nodes = tet_nodes(order)
    q, w = tet_rule(order + 3)
    # orthonormalise the modal basis on the tetrahedron (Cholesky factor of
    # its Gram matrix under the quadrature), which keeps the Vandermonde
    # matrix well conditioned at order 4
    bq = modal_basis(order, q)
    tr = np.linalg.inv(np.linalg.cholesky(np.einsum("q,qm,qn->mn", w, bq, bq))).T
    vinv = np.linalg.inv(modal_basis(order, nodes) @ tr)
    lag = bq @ tr @ vinv                                    # (nq, Np)
    dlag = np.einsum("rqm,mn,nj->rqj", modal_basis_grads(order, q), tr, vinv)
    mass = np.einsum("q,qi,qj->ij", w, lag, lag)
    stiff_t = np.einsum("q,rqi,qj->rij", w, dlag, lag)
    diff = np.einsum("ik,rjk->rij", np.linalg.inv(mass), stiff_t)

    fref = tri_nodes(order)                                 # (Nfp, 2)
    v2inv = np.linalg.inv(modal_basis(order, fref))
    q2, w2 = tri_rule(order + 2)
    lag2 = modal_basis(order, q2) @ v2inv                     # (nq2, Nfp)

    def bary2(x2):  # biunit-triangle coordinates -> barycentric
        l1 = (x2[:, 0] + 1) / 2
        l2 = (x2[:, 1] + 1) / 2
        return np.stack([1 - l1 - l2, l1, l2], axis=1)

    npn, nfp = nodes.shape[0], fref.shape[0]
    emat = np.zeros((npn, 4, nfp))
    fcoords = np.zeros((4, nfp, 3))
    for f, fv in enumerate(FACES):
        fverts = TET_VERTICES[list(fv)]                     # (3, 3)
        xq = bary2(q2) @ fverts
        vol_lag = modal_basis(order, xq) @ tr @ vinv          # (nq2, Np)
        emat[:, f, :] = np.einsum("q,qk,qj->kj", w2, vol_lag, lag2)
        fcoords[f] = bary2(fref) @ fverts
    return OracleRefOps(order=order, nodes=nodes, mass=mass, stiff_t=stiff_t,
                        diff=diff, face_mass=emat, face_node_coords=fcoords)

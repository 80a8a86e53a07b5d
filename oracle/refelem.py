"""The oracle's own reference tetrahedron (test infrastructure).

Built without any code of the product, so that a wrong node family, node
order, basis or quadrature in the product cannot hide behind a shared
implementation:

* Gauss-Lobatto-Legendre points from NumPy's Legendre module (the roots of
  P_n'), not from a Newton iteration;
* volume and face nodes of the recursive family (Isaac, "Recursive,
  parameter-free, explicitly defined interpolation nodes for simplices",
  SIAM J. Sci. Comput. 42(6), 2020), which meshmode's
  ``default_simplex_group_factory`` uses when ``recursivenodes`` is
  installed.  For orders <= 3 every node is a vertex, a GLL point of an edge
  or a face centroid, and the oracle places them so directly (the same set as
  Hesthaven and Warburton's warp-and-blend nodes, Nodal DG Methods section
  6.1); the order-4 face-interior nodes come from the recursive rule, written
  here in closed form for the barycentric multi-index (2, 1, 1) of a triangle,
  and the order-4 volume node is the centroid;
* products of Legendre polynomials L_a(r) L_b(s) L_c(t) (a + b + c <= N) as
  the modal basis of the Vandermonde matrices: a nodal Lagrange basis does
  not depend on the modal basis that spans P_N;
* Gauss-Legendre rules mapped to the simplex by the collapsed (Duffy)
  transform.

Conventions restated as data (they are the modepy/meshmode conventions the
reference's discretisation follows): the biunit tetrahedron with vertices
(-1,-1,-1), (1,-1,-1), (-1,1,-1), (-1,-1,1); node (i, j, k) (multi-indices
with i + j + k <= N, first index fastest) has barycentric multi-index
(N-i-j-k, i, j, k); the faces are the vertex triples (0,2,1), (0,1,3),
(0,3,2), (1,2,3).
"""

from __future__ import annotations

from functools import lru_cache
from math import comb

import numpy as np
from numpy.polynomial import legendre as npleg

TET_VERTICES = np.array([[-1.0, -1.0, -1.0], [1.0, -1.0, -1.0],
                         [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]])
TRI_VERTICES = np.array([[-1.0, -1.0], [1.0, -1.0], [-1.0, 1.0]])
FACES = ((0, 2, 1), (0, 1, 3), (0, 3, 2), (1, 2, 3))


def gll_01(n: int) -> np.ndarray:
    """The n + 1 Gauss-Lobatto-Legendre points on [0, 1], ascending."""
    if n == 1:
        return np.array([0.0, 1.0])
    inner = np.sort(npleg.Legendre.basis(n).deriv().roots().real)
    x = np.concatenate([[-1.0], inner, [1.0]])
    x = 0.5 * (x - x[::-1])          # symmetric to round-off
    return 0.5 * (x + 1.0)


def enumerate_nodes(dim: int, order: int) -> list[tuple[int, ...]]:
    """Multi-indices with sum <= order, first index varying fastest."""
    out = []
    if dim == 2:
        for j in range(order + 1):
            for i in range(order + 1 - j):
                out.append((i, j))
    else:
        for k in range(order + 1):
            for j in range(order + 1 - k):
                for i in range(order + 1 - j - k):
                    out.append((i, j, k))
    return out


def _face_interior_211(order: int) -> np.ndarray:
    """Barycentric coordinates of the recursive node with multi-index
    (2, 1, 1) on a triangle (order 4): the facet projections weighted by
    x_4[n - alpha_i], i.e. (0, 1/2, 1/2) with weight x_4[2] and the two
    order-3 edge nodes ((1 + 5^-1/2)/2 on the vertex with the 2) with weight
    x_4[3] each."""
    assert order == 4
    x4, x3 = gll_01(4), gll_01(3)
    w0, w1 = x4[2], x4[3]
    a, c = x3[2], x3[1]
    b = (w0 * np.array([0.0, 0.5, 0.5]) + w1 * np.array([a, 0.0, c])
         + w1 * np.array([a, c, 0.0]))
    return b / (w0 + 2 * w1)


def barycentric_node(alpha: tuple[int, ...]) -> np.ndarray:
    """Barycentric coordinates of the node with barycentric multi-index
    ``alpha`` (length 3 or 4, sum N <= 4)."""
    alpha = tuple(int(a) for a in alpha)
    n = sum(alpha)
    d = len(alpha)
    nz = [k for k in range(d) if alpha[k] > 0]
    b = np.zeros(d)
    if len(nz) == 1:                       # vertex
        b[nz[0]] = 1.0
    elif len(nz) == 2:                     # edge: the GLL point
        g = gll_01(n)
        b[nz[0]] = g[alpha[nz[0]]]
        b[nz[1]] = g[alpha[nz[1]]]
    elif all(alpha[k] == alpha[nz[0]] for k in nz):   # centroid of a face or the volume
        b[nz] = 1.0 / len(nz)
    elif len(nz) == 3 and n == 4:          # order-4 face interior, (2,1,1) up to order
        big = [k for k in nz if alpha[k] == 2][0]
        rest = [k for k in nz if k != big]
        loc = _face_interior_211(4)
        b[big], b[rest[0]], b[rest[1]] = loc
    else:
        raise NotImplementedError(f"node {alpha} (orders 1..4 only)")
    return b


@lru_cache(maxsize=None)
def tet_nodes(order: int) -> np.ndarray:
    """(Np, 3) biunit-tetrahedron coordinates of the volume nodes."""
    pts = [barycentric_node((order - sum(m),) + m) for m in enumerate_nodes(3, order)]
    out = np.array(pts) @ TET_VERTICES
    out.setflags(write=False)
    return out


@lru_cache(maxsize=None)
def tri_nodes(order: int) -> np.ndarray:
    """(Nfp, 2) biunit-triangle coordinates of the face nodes."""
    pts = [barycentric_node((order - sum(m),) + m) for m in enumerate_nodes(2, order)]
    out = np.array(pts) @ TRI_VERTICES
    out.setflags(write=False)
    return out


# {{{ a modal basis of P_N: products of Legendre polynomials


def _exponents(dim: int, order: int) -> list[tuple[int, ...]]:
    return enumerate_nodes(dim, order)


def _leg(k: int, x: np.ndarray, deriv: int = 0) -> np.ndarray:
    c = np.zeros(k + 1)
    c[k] = 1.0
    if deriv:
        c = npleg.legder(c, deriv)
    return npleg.legval(x, c)


def modal_basis(order: int, x: np.ndarray) -> np.ndarray:
    """(npts, nbasis) values of L_a(r) L_b(s) (L_c(t)), a + b (+ c) <= N:
    the products of Legendre polynomials of total degree <= N span P_N
    (better conditioned on the biunit simplex than plain modal_basis)."""
    dim = x.shape[1]
    ex = _exponents(dim, order)
    assert len(ex) == comb(order + dim, dim)
    return np.stack([np.prod([_leg(e[k], x[:, k]) for k in range(dim)], axis=0)
                     for e in ex], axis=1)


def modal_basis_grads(order: int, x: np.ndarray) -> np.ndarray:
    """(3, npts, nbasis) derivatives of the tetrahedron basis functions."""
    ex = _exponents(3, order)
    out = np.zeros((3, x.shape[0], len(ex)))
    for m, e in enumerate(ex):
        for r in range(3):
            val = np.ones(x.shape[0])
            for k in range(3):
                val = val * _leg(e[k], x[:, k], 1 if k == r else 0)
            out[r, :, m] = val
    return out


# }}}


# {{{ collapsed Gauss-Legendre quadrature


def _gl01(m: int):
    x, w = npleg.leggauss(m)
    return 0.5 * (x + 1.0), 0.5 * w


def tet_rule(m: int):
    """Points (biunit tetrahedron) and weights; exact for polynomials of
    degree <= 2 m - 3."""
    u, wu = _gl01(m)
    pts, wts = [], []
    for a, wa in zip(u, wu):
        for b, wb in zip(u, wu):
            for c, wc in zip(u, wu):
                x = a
                y = (1 - a) * b
                z = (1 - a) * (1 - b) * c
                pts.append((x, y, z))
                wts.append(wa * wb * wc * (1 - a) ** 2 * (1 - b))
    p = np.array(pts)
    # unit tetrahedron -> biunit: X = -1 + 2 x, Jacobian 8
    return -1.0 + 2.0 * p, 8.0 * np.array(wts)


def tri_rule(m: int):
    """Points (biunit triangle) and weights; exact for degree <= 2 m - 2."""
    u, wu = _gl01(m)
    pts, wts = [], []
    for a, wa in zip(u, wu):
        for b, wb in zip(u, wu):
            pts.append((a, (1 - a) * b))
            wts.append(wa * wb * (1 - a))
    return -1.0 + 2.0 * np.array(pts), 4.0 * np.array(wts)


# }}}

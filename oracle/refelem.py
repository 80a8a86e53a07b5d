"""The oracle's own reference tetrahedron (test infrastructure).

Built without any code of the product, so that a wrong node family, node
order, basis or quadrature in the product cannot hide behind a shared
implementation, and evaluated in 32-digit arithmetic (mpmath) so that the
oracle's matrices are exact to FP64 rounding:

* Gauss-Lobatto-Legendre points: the roots of P_n' by Newton's method (from
  NumPy's double-precision roots), in extended precision;
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
(0,3,2), (1,2,3).  For 2D meshes the same constructions give the reference
triangle: vertices (-1,-1), (1,-1), (-1,1), node (i, j) with barycentric
multi-index (N-i-j, i, j), edges (0,1), (2,0), (1,2), and GLL points on the
edges.
"""

from __future__ import annotations

from functools import lru_cache
from math import comb

import mpmath
import numpy as np
from numpy.polynomial import legendre as npleg

#: working precision of the reference-element construction (decimal digits)
DPS = 32
MP = mpmath.MPContext()
MP.dps = DPS

TET_VERTICES = np.array([[-1.0, -1.0, -1.0], [1.0, -1.0, -1.0],
                         [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]])
TRI_VERTICES = np.array([[-1.0, -1.0], [1.0, -1.0], [-1.0, 1.0]])
FACES = ((0, 2, 1), (0, 1, 3), (0, 3, 2), (1, 2, 3))
#: the edges of the triangle (2D meshes), meshmode's order
TRI_EDGES = ((0, 1), (2, 0), (1, 2))


# {{{ Legendre polynomials, Gauss and Gauss-Lobatto points (extended precision)


def legendre(n: int, x):
    """(P_n(x), P_n'(x)) by the three-term recurrence (and P_k' = P_{k-2}' +
    (2k - 1) P_{k-1})."""
    x = MP.mpf(x)
    p0, p1 = MP.mpf(1), x
    d0, d1 = MP.mpf(0), MP.mpf(1)
    if n == 0:
        return p0, d0
    for k in range(2, n + 1):
        p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
        d0, d1 = d1, d0 + (2 * k - 1) * p0
    return p1, d1


def _dlegendre(n: int, x):
    """(P_n'(x), P_n''(x)) for |x| < 1, from the Legendre equation
    (1 - x^2) P'' = 2 x P' - n (n + 1) P."""
    p, d = legendre(n, x)
    return d, (2 * x * d - n * (n + 1) * p) / (1 - x * x)


def _newton(f, x0, iters: int = 60):
    x = MP.mpf(x0)
    for _ in range(iters):
        fx, dfx = f(x)
        step = fx / dfx
        x -= step
        if abs(step) < MP.mpf(10) ** (-DPS + 2):
            break
    return x


@lru_cache(maxsize=None)
def gll_01_mp(n: int) -> tuple:
    """The n + 1 Gauss-Lobatto-Legendre points on [0, 1], ascending."""
    if n == 1:
        return (MP.mpf(0), MP.mpf(1))
    guess = np.sort(npleg.Legendre.basis(n).deriv().roots().real)
    inner = [_newton(lambda x: _dlegendre(n, x), g) for g in guess]
    pts = [MP.mpf(-1)] + inner + [MP.mpf(1)]
    pts = [(p - q) / 2 for p, q in zip(pts, pts[::-1])]   # exactly symmetric
    return tuple((p + 1) / 2 for p in pts)


def gll_01(n: int) -> np.ndarray:
    return np.array([float(x) for x in gll_01_mp(n)])


@lru_cache(maxsize=None)
def gauss_01_mp(m: int) -> tuple:
    """m-point Gauss-Legendre points and weights on [0, 1]."""
    guess, _ = npleg.leggauss(m)
    xs = [_newton(lambda x: legendre(m, x), g) for g in guess]
    ws = [2 / ((1 - x * x) * legendre(m, x)[1] ** 2) for x in xs]
    return tuple((x + 1) / 2 for x in xs), tuple(w / 2 for w in ws)


# }}}


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


def _face_interior_211(order: int) -> list:
    """Barycentric coordinates of the recursive node with multi-index
    (2, 1, 1) on a triangle (order 4): the facet projections weighted by
    x_4[n - alpha_i], i.e. (0, 1/2, 1/2) with weight x_4[2] and the two
    order-3 edge nodes ((1 + 5^-1/2)/2 on the vertex with the 2) with weight
    x_4[3] each."""
    assert order == 4
    x4, x3 = gll_01_mp(4), gll_01_mp(3)
    w0, w1 = x4[2], x4[3]
    a, c = x3[2], x3[1]
    half = MP.mpf(1) / 2
    b = [2 * w1 * a, w0 * half + w1 * c, w0 * half + w1 * c]
    tot = w0 + 2 * w1
    return [v / tot for v in b]


def barycentric_node_mp(alpha: tuple[int, ...]) -> list:
    """Barycentric coordinates (extended precision) of the node with
    barycentric multi-index ``alpha`` (length 3 or 4, sum N <= 4)."""
    alpha = tuple(int(a) for a in alpha)
    n = sum(alpha)
    d = len(alpha)
    nz = [k for k in range(d) if alpha[k] > 0]
    b = [MP.mpf(0)] * d
    if len(nz) == 1:                       # vertex
        b[nz[0]] = MP.mpf(1)
    elif len(nz) == 2:                     # edge: the GLL point
        g = gll_01_mp(n)
        b[nz[0]] = g[alpha[nz[0]]]
        b[nz[1]] = g[alpha[nz[1]]]
    elif all(alpha[k] == alpha[nz[0]] for k in nz):   # centroid of a face or the volume
        for k in nz:
            b[k] = MP.mpf(1) / len(nz)
    elif len(nz) == 3 and n == 4:          # order-4 face interior, (2,1,1) up to order
        big = [k for k in nz if alpha[k] == 2][0]
        rest = [k for k in nz if k != big]
        loc = _face_interior_211(4)
        b[big], b[rest[0]], b[rest[1]] = loc
    else:
        raise NotImplementedError(f"node {alpha} (orders 1..4 only)")
    return b


def barycentric_node(alpha: tuple[int, ...]) -> np.ndarray:
    return np.array([float(v) for v in barycentric_node_mp(alpha)])


def _to_ref(bary: list, verts: np.ndarray) -> list:
    dim = verts.shape[1]
    return [sum(bary[v] * int(verts[v, x]) for v in range(len(bary))) for x in range(dim)]


@lru_cache(maxsize=None)
def tet_nodes_mp(order: int) -> tuple:
    """Biunit-tetrahedron coordinates of the volume nodes (extended precision)."""
    return tuple(tuple(_to_ref(barycentric_node_mp((order - sum(m),) + m), TET_VERTICES))
                 for m in enumerate_nodes(3, order))


@lru_cache(maxsize=None)
def tri_nodes_mp(order: int) -> tuple:
    """Biunit-triangle coordinates of the face nodes (extended precision)."""
    return tuple(tuple(_to_ref(barycentric_node_mp((order - sum(m),) + m), TRI_VERTICES))
                 for m in enumerate_nodes(2, order))


def _as_float(pts) -> np.ndarray:
    out = np.array([[float(v) for v in p] for p in pts])
    out.setflags(write=False)
    return out


@lru_cache(maxsize=None)
def tet_nodes(order: int) -> np.ndarray:
    """(Np, 3) biunit-tetrahedron coordinates of the volume nodes."""
    return _as_float(tet_nodes_mp(order))


@lru_cache(maxsize=None)
def tri_nodes(order: int) -> np.ndarray:
    """(Nfp, 2) biunit-triangle coordinates of the face nodes."""
    return _as_float(tri_nodes_mp(order))


# {{{ a modal basis of P_N: products of Legendre polynomials


def _exponents(dim: int, order: int) -> list[tuple[int, ...]]:
    ex = enumerate_nodes(dim, order)
    assert len(ex) == comb(order + dim, dim)
    return ex


def modal_basis(order: int, x) -> list:
    """Rows (one per point) of L_a(r) L_b(s) (L_c(t)), a + b (+ c) <= N, in
    extended precision: the products of Legendre polynomials of total degree
    <= N span P_N."""
    rows = []
    for p in x:
        dim = len(p)
        vals = [[legendre(k, p[d])[0] for k in range(order + 1)] for d in range(dim)]
        rows.append([MP.fprod(vals[d][e[d]] for d in range(dim))
                     for e in _exponents(dim, order)])
    return rows


def modal_basis_grads(order: int, x) -> list:
    """[r][point][basis]: derivatives of the basis functions (tetrahedron or,
    for 2-coordinate points, triangle)."""
    dim = len(x[0])
    out = [[] for _ in range(dim)]
    for p in x:
        v = [[legendre(k, p[d]) for k in range(order + 1)] for d in range(dim)]
        for r in range(dim):
            out[r].append([MP.fprod(v[d][e[d]][1 if d == r else 0] for d in range(dim))
                           for e in _exponents(dim, order)])
    return out


# }}}


# {{{ collapsed Gauss-Legendre quadrature


def tet_rule(m: int):
    """Points (biunit tetrahedron) and weights, extended precision; exact for
    polynomials of degree <= 2 m - 3."""
    u, wu = gauss_01_mp(m)
    pts, wts = [], []
    for a, wa in zip(u, wu):
        for b, wb in zip(u, wu):
            for c, wc in zip(u, wu):
                x, y, z = a, (1 - a) * b, (1 - a) * (1 - b) * c
                # unit tetrahedron -> biunit: X = -1 + 2 x, Jacobian 8
                pts.append((2 * x - 1, 2 * y - 1, 2 * z - 1))
                wts.append(8 * wa * wb * wc * (1 - a) ** 2 * (1 - b))
    return pts, wts


def tri_rule(m: int):
    """Points (biunit triangle) and weights, extended precision; exact for
    degree <= 2 m - 2."""
    u, wu = gauss_01_mp(m)
    pts, wts = [], []
    for a, wa in zip(u, wu):
        for b, wb in zip(u, wu):
            pts.append((2 * a - 1, 2 * (1 - a) * b - 1))
            wts.append(4 * wa * wb * (1 - a))
    return pts, wts


# }}}

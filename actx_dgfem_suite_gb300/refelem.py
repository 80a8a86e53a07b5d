"""Reference tetrahedron for nodal DG: node set, orthonormal basis, operators.

This module replaces the parts of ``meshmode``/``modepy``/``grudge`` that the
suite's RHS builders reach through ``DiscretizationCollection`` (call sites
``actx_dgfem_suite/equations/wave.py:256-270``, ``euler.py:156-166``,
``maxwell.py:55``):

* volume nodes: the recursive LGL node family that meshmode's
  ``default_simplex_group_factory`` selects when ``recursivenodes`` is
  installed.  For N <= 3 it coincides with the warp-and-blend family (all
  nodes are vertices, GLL edge points and face centroids); it differs only in
  the three face-interior nodes per face at N = 4.
* the orthonormal Proriol-Koornwinder-Dubiner-Owens (PKDO) basis on the
  biunit tetrahedron and triangle,
* the fused operators that ``actx_dgfem_suite/arraycontext/mass_inverse_fuser.py:20-76``
  builds from grudge's matrices: ``ik,rkj->rij`` (inverse mass times
  stiffness-transpose, i.e. the weak derivative) and ``ik,kfj->ifj``
  (inverse mass times face mass, i.e. LIFT), plus the strong derivative
  matrices used by Maxwell's ``local_d_dx``.

Conventions (modepy): biunit tetrahedron with vertices
v0=(-1,-1,-1), v1=(1,-1,-1), v2=(-1,1,-1), v3=(-1,-1,1); nodes ordered by the
multi-index enumeration of ``generate_nonnegative_integer_tuples_summing_to_at_most``
(first index fastest); a node with multi-index (i, j, k) has barycentric
multi-index (N-i-j-k, i, j, k).  Faces follow meshmode's tetrahedron face
vertex tuples ((0,2,1), (0,1,3), (0,3,2), (1,2,3)).
"""

from __future__ import annotations

import itertools
import math
from dataclasses import dataclass
from functools import lru_cache

import numpy as np

DIM = 3
NFACES = 4
#: local vertex indices of each face, meshmode's order for tetrahedra
FACE_VERTICES = ((0, 2, 1), (0, 1, 3), (0, 3, 2), (1, 2, 3))
#: the local vertex opposite each face
FACE_OPPOSITE_VERTEX = (3, 2, 1, 0)

BIUNIT_TET_VERTICES = np.array(
    [[-1.0, -1.0, -1.0], [1.0, -1.0, -1.0], [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]]
)
BIUNIT_TRI_VERTICES = np.array([[-1.0, -1.0], [1.0, -1.0], [-1.0, 1.0]])
#: biunit tetrahedron volume and biunit triangle area
BIUNIT_TET_VOLUME = 4.0 / 3.0
BIUNIT_TRI_AREA = 2.0


def nnodes(dim: int, order: int) -> int:
    return math.comb(order + dim, dim)


def multi_indices(dim: int, order: int) -> list[tuple[int, ...]]:
    """All non-negative integer ``dim``-tuples with sum <= ``order``, first
    entry varying fastest (pytools' ``gnitstam`` order used by modepy)."""
    if dim == 0:
        return [()]
    out = []
    for last in range(order + 1):
        for rest in multi_indices(dim - 1, order - last):
            out.append(rest + (last,))
    return out


# {{{ 1D Gauss-Lobatto-Legendre points


@lru_cache(maxsize=None)
def gll_points_01(n: int) -> tuple[float, ...]:
    """The n+1 Gauss-Lobatto-Legendre points mapped to [0, 1], sorted.

    Interior points are the roots of P_n'(x); they are found by Newton's
    method from Chebyshev-Gauss-Lobatto initial guesses and symmetrised."""
    if n == 0:
        return (0.5,)
    x = -np.cos(np.pi * np.arange(n + 1) / n)
    for _ in range(100):
        # Legendre P_n and P_{n-1} via the three-term recurrence
        p_prev = np.ones_like(x)
        p = x.copy()
        for k in range(2, n + 1):
            p_prev, p = p, ((2 * k - 1) * x * p - (k - 1) * p_prev) / k
        # Newton on (1-x^2) P_n'(x) = n (P_{n-1} - x P_n); interior only
        dx = np.zeros_like(x)
        interior = slice(1, n)
        xi = x[interior]
        f = p_prev[interior] - xi * p[interior]
        # derivative of f: d/dx (P_{n-1} - x P_n) = -(n+1) P_n (Legendre identity)
        df = -(n + 1) * p[interior]
        dx[interior] = f / df
        x = x - dx
        if np.max(np.abs(dx)) < 1e-16:
            break
    x[0], x[-1] = -1.0, 1.0
    x = 0.5 * (x - x[::-1])  # enforce exact antisymmetry
    return tuple(0.5 * (x + 1.0))


# }}}


# {{{ recursive nodes (Isaac 2020, "Recursive, parameter-free, explicitly
# defined interpolation nodes for simplices", SIAM J. Sci. Comput. 42(6))


def _recursive_barycentric(alpha: tuple[int, ...]) -> np.ndarray:
    """Barycentric coordinates of the node with barycentric multi-index
    ``alpha`` (length d+1, sum n) in the recursive construction on the GLL
    family: the node is the weighted mean of its projections onto the facets,
    facet i being weighted by the 1D GLL point x_n[n - alpha_i]."""
    d = len(alpha) - 1
    n = sum(alpha)
    g = gll_points_01(n) if n > 0 else (1.0,)
    if d == 1:
        return np.array([g[alpha[0]], g[alpha[1]]])
    b = np.zeros(d + 1)
    wsum = 0.0
    for i in range(d + 1):
        n_noti = n - alpha[i]
        w = g[n_noti]
        if w == 0.0:
            continue
        sub = alpha[:i] + alpha[i + 1 :]
        br = _recursive_barycentric(sub)
        b[:i] += w * br[:i]
        b[i + 1 :] += w * br[i:]
        wsum += w
    return b / wsum


@lru_cache(maxsize=None)
def recursive_barycentric_nodes(dim: int, order: int) -> np.ndarray:
    """(Np, dim+1) barycentric coordinates, in ``multi_indices`` order."""
    rows = []
    for mi in multi_indices(dim, order):
        alpha = (order - sum(mi),) + tuple(mi)
        if order == 0:
            rows.append(np.full(dim + 1, 1.0 / (dim + 1)))
        else:
            rows.append(_recursive_barycentric(alpha))
    out = np.array(rows)
    out.setflags(write=False)
    return out


def barycentric_to_biunit(bary: np.ndarray) -> np.ndarray:
    dim = bary.shape[-1] - 1
    verts = BIUNIT_TET_VERTICES if dim == 3 else BIUNIT_TRI_VERTICES
    return bary @ verts


def volume_nodes(order: int) -> np.ndarray:
    """(Np, 3) reference coordinates of the volume nodes."""
    return barycentric_to_biunit(recursive_barycentric_nodes(3, order))


def face_reference_nodes(order: int) -> np.ndarray:
    """(Nfp, 2) biunit-triangle coordinates of the face nodes."""
    return barycentric_to_biunit(recursive_barycentric_nodes(2, order))


# }}}


# {{{ dual numbers (exact first derivatives of polynomial expressions)


class Dual:
    """Value plus gradient w.r.t. (r, s, t); enough arithmetic for the
    Jacobi recurrences and the collapsed-coordinate maps."""

    __slots__ = ("val", "grad")

    def __init__(self, val, grad):
        self.val = np.asarray(val, dtype=np.float64)
        self.grad = np.asarray(grad, dtype=np.float64)

    @staticmethod
    def _lift(x, like):
        if isinstance(x, Dual):
            return x
        return Dual(np.broadcast_to(x, like.val.shape),
                    np.zeros_like(like.grad))

    def __add__(self, o):
        o = Dual._lift(o, self)
        return Dual(self.val + o.val, self.grad + o.grad)

    __radd__ = __add__

    def __neg__(self):
        return Dual(-self.val, -self.grad)

    def __sub__(self, o):
        return self + (-Dual._lift(o, self))

    def __rsub__(self, o):
        return Dual._lift(o, self) - self

    def __mul__(self, o):
        if not isinstance(o, Dual):
            return Dual(self.val * o, self.grad * o)
        return Dual(self.val * o.val, self.grad * o.val + self.val * o.grad)

    __rmul__ = __mul__

    def __truediv__(self, o):
        if not isinstance(o, Dual):
            return Dual(self.val / o, self.grad / o)
        return Dual(self.val / o.val,
                    (self.grad * o.val - self.val * o.grad) / o.val**2)

    def __rtruediv__(self, o):
        return Dual._lift(o, self) / self

    def __pow__(self, k: int):
        out = Dual(np.ones_like(self.val), np.zeros_like(self.grad))
        for _ in range(k):
            out = out * self
        return out


# }}}


# {{{ orthonormal Jacobi polynomials and the PKDO basis


def jacobi_orthonormal(x, alpha: float, beta: float, n: int) -> list:
    """[p_0(x), ..., p_n(x)], orthonormal on [-1, 1] with weight
    (1-x)^alpha (1+x)^beta, from the standard three-term recurrence of the
    orthonormal Jacobi family.  ``x`` may be an array or a :class:`Dual`."""
    ab = alpha + beta
    gamma0 = (2.0 ** (ab + 1) / (ab + 1)
              * math.gamma(alpha + 1) * math.gamma(beta + 1) / math.gamma(ab + 1))
    p0 = x * 0.0 + 1.0 / math.sqrt(gamma0)
    out = [p0]
    if n == 0:
        return out
    gamma1 = (alpha + 1) * (beta + 1) / (ab + 3) * gamma0
    p1 = (x * ((ab + 2) / 2) + (alpha - beta) / 2) / math.sqrt(gamma1)
    out.append(p1)
    a_old = 2.0 / (2 + ab) * math.sqrt((alpha + 1) * (beta + 1) / (ab + 3))
    for i in range(1, n):
        h1 = 2 * i + ab
        a_new = 2.0 / (h1 + 2) * math.sqrt(
            (i + 1) * (i + 1 + ab) * (i + 1 + alpha) * (i + 1 + beta)
            / (h1 + 1) / (h1 + 3))
        b_new = -(alpha**2 - beta**2) / h1 / (h1 + 2)
        out.append(((x - b_new) * out[i] - out[i - 1] * a_old) / a_new)
        a_old = a_new
    return out


def _safe_ratio(num, den, fallback):
    """num/den where |den| > 1e-14, else ``fallback`` (the collapsed
    coordinate is arbitrary there: every basis function that depends on it
    carries a vanishing factor)."""
    ok = np.abs(den) > 1e-14
    out = np.full(np.shape(num), fallback, dtype=np.float64)
    np.divide(num, den, out=out, where=ok)
    return np.where(ok, out, fallback)


def _collapse_tet(r, s, t):
    """Collapsed coordinates (a, b, c) of biunit-tet points (arrays)."""
    a = _safe_ratio(2.0 * (1.0 + r), -s - t, 0.0) - 1.0
    a = np.where(np.abs(s + t) > 1e-14, a, -1.0)
    b = _safe_ratio(2.0 * (1.0 + s), 1.0 - t, 0.0) - 1.0
    b = np.where(np.abs(t - 1.0) > 1e-14, b, -1.0)
    return a, b, t


def pkdo_tet(order: int, x: np.ndarray) -> np.ndarray:
    """(npoints, Np) values of the orthonormal PKDO basis at biunit-tet
    points ``x`` (npoints, 3); basis index order = ``multi_indices(3, N)``."""
    r, s, t = x[:, 0], x[:, 1], x[:, 2]
    a, b, c = _collapse_tet(r, s, t)
    cols = []
    for (i, j, k) in multi_indices(3, order):
        pa = jacobi_orthonormal(a, 0.0, 0.0, i)[i]
        pb = jacobi_orthonormal(b, 2 * i + 1.0, 0.0, j)[j]
        pc = jacobi_orthonormal(c, 2 * (i + j) + 2.0, 0.0, k)[k]
        cols.append(2.0 * math.sqrt(2.0) * pa * pb * (1 - b) ** i * pc
                    * (1 - c) ** (i + j))
    return np.stack(cols, axis=1)


def pkdo_tet_grad_interior(order: int, x: np.ndarray) -> np.ndarray:
    """(3, npoints, Np) gradient of the PKDO basis at points strictly inside
    the tetrahedron (where the collapsed map is smooth), by dual numbers."""
    npt = x.shape[0]
    eye = np.eye(3)
    r = Dual(x[:, 0], np.outer(eye[0], np.ones(npt)))
    s = Dual(x[:, 1], np.outer(eye[1], np.ones(npt)))
    t = Dual(x[:, 2], np.outer(eye[2], np.ones(npt)))
    a = 2.0 * (1.0 + r) / (-s - t) - 1.0
    b = 2.0 * (1.0 + s) / (1.0 - t) - 1.0
    c = t
    cols = []
    for (i, j, k) in multi_indices(3, order):
        pa = jacobi_orthonormal(a, 0.0, 0.0, i)[i]
        pb = jacobi_orthonormal(b, 2 * i + 1.0, 0.0, j)[j]
        pc = jacobi_orthonormal(c, 2 * (i + j) + 2.0, 0.0, k)[k]
        psi = 2.0 * math.sqrt(2.0) * pa * pb * (1 - b) ** i * pc * (1 - c) ** (i + j)
        cols.append(psi.grad)
    return np.stack(cols, axis=2)


def pkdo_tri(order: int, x: np.ndarray) -> np.ndarray:
    """(npoints, Nfp) orthonormal PKDO basis on the biunit triangle."""
    r, s = x[:, 0], x[:, 1]
    a = _safe_ratio(2.0 * (1.0 + r), 1.0 - s, 0.0) - 1.0
    a = np.where(np.abs(s - 1.0) > 1e-14, a, -1.0)
    b = s
    cols = []
    for (i, j) in multi_indices(2, order):
        pa = jacobi_orthonormal(a, 0.0, 0.0, i)[i]
        pb = jacobi_orthonormal(b, 2 * i + 1.0, 0.0, j)[j]
        cols.append(math.sqrt(2.0) * pa * pb * (1 - b) ** i)
    return np.stack(cols, axis=1)


# }}}


# {{{ quadrature (Stroud conical product rules)


def _gauss_jacobi(q: int, alpha: float):
    from scipy.special import roots_jacobi
    x, w = roots_jacobi(q, alpha, 0.0)
    return x, w


def tet_quadrature(q: int) -> tuple[np.ndarray, np.ndarray]:
    """Conical-product rule with q^3 interior points on the biunit tet,
    exact for polynomials of total degree <= 2q-1."""
    xa, wa = _gauss_jacobi(q, 0.0)
    xb, wb = _gauss_jacobi(q, 1.0)
    xc, wc = _gauss_jacobi(q, 2.0)
    A, B, C = np.meshgrid(xa, xb, xc, indexing="ij")
    W = (wa[:, None, None] * wb[None, :, None] * wc[None, None, :]) / 8.0
    t = C
    s = (1 + B) * (1 - C) / 2 - 1
    r = (1 + A) * (1 - B) * (1 - C) / 4 - 1
    pts = np.stack([r.ravel(), s.ravel(), t.ravel()], axis=1)
    return pts, W.ravel()


def tri_quadrature(q: int) -> tuple[np.ndarray, np.ndarray]:
    """Conical-product rule with q^2 interior points on the biunit triangle,
    exact for total degree <= 2q-1."""
    xa, wa = _gauss_jacobi(q, 0.0)
    xb, wb = _gauss_jacobi(q, 1.0)
    A, B = np.meshgrid(xa, xb, indexing="ij")
    W = (wa[:, None] * wb[None, :]) / 2.0
    s = B
    r = (1 + A) * (1 - B) / 2 - 1
    return np.stack([r.ravel(), s.ravel()], axis=1), W.ravel()


# }}}


# {{{ the reference element


@dataclass(frozen=True)
class ReferenceTet:
    """All per-order constants of the nodal DG discretisation.

    Array shapes use Np volume nodes and Nfp nodes per face."""

    order: int
    nodes: np.ndarray            # (Np, 3) reference coordinates
    vdm: np.ndarray              # (Np, Np) V[node, mode]
    mass: np.ndarray             # (Np, Np) reference mass matrix
    diff: np.ndarray             # (3, Np, Np) strong D_r = V_r V^-1
    weak_diff: np.ndarray        # (3, Np, Np) M^-1 S_r^T   (mass_inverse_fuser ``ik,rkj->rij``)
    face_nodes: np.ndarray       # (4, Nfp) volume-node index of each face node
    face_mass: np.ndarray        # (Nfp, Nfp) biunit-triangle mass on face nodes
    lift: np.ndarray             # (Np, 4, Nfp) M^-1 E   (mass_inverse_fuser ``ik,kfj->ifj``)
    face_perm: dict              # vertex permutation -> (Nfp,) face-node map

    @property
    def np_(self) -> int:
        return self.nodes.shape[0]

    @property
    def nfp(self) -> int:
        return self.face_nodes.shape[1]


def _face_node_lists(order: int) -> np.ndarray:
    """(4, Nfp): for face f with local vertices (a, b, c), the volume nodes
    with zero barycentric weight at the opposite vertex, ordered by the 2D
    multi-index (alpha_b, alpha_c) in ``multi_indices(2, N)`` order."""
    vol_mis = multi_indices(3, order)
    bary_mi = {(order - sum(mi),) + tuple(mi): idx for idx, mi in enumerate(vol_mis)}
    out = []
    for f in range(NFACES):
        a, b, c = FACE_VERTICES[f]
        opp = FACE_OPPOSITE_VERTEX[f]
        row = []
        for (i2, j2) in multi_indices(2, order):
            alpha = [0, 0, 0, 0]
            alpha[a] = order - i2 - j2
            alpha[b] = i2
            alpha[c] = j2
            alpha[opp] = 0
            row.append(bary_mi[tuple(alpha)])
        out.append(row)
    return np.array(out, dtype=np.int64)


def _face_permutation_maps(order: int) -> dict:
    """For each permutation p of the three face vertices, the map j -> j'
    between face-node indices of two glued faces: if neighbour face vertex x
    is our face vertex p[x], our node with face barycentric multi-index mu
    is the neighbour's node with multi-index (mu[p[0]], mu[p[1]], mu[p[2]])."""
    mis2 = multi_indices(2, order)
    index_of = {mi: k for k, mi in enumerate(mis2)}
    out = {}
    for p in itertools.permutations(range(3)):
        m = []
        for (i2, j2) in mis2:
            mu = (order - i2 - j2, i2, j2)
            mu_n = (mu[p[0]], mu[p[1]], mu[p[2]])
            m.append(index_of[(mu_n[1], mu_n[2])])
        out[p] = np.array(m, dtype=np.int64)
    return out


@lru_cache(maxsize=None)
def reference_tet(order: int) -> ReferenceTet:
    if order < 1:
        raise ValueError("order must be >= 1")
    nodes = volume_nodes(order)
    npn = nodes.shape[0]
    vdm = pkdo_tet(order, nodes)
    vinv = np.linalg.inv(vdm)
    mass = vinv.T @ vinv

    # modal derivative matrices C_r[m, n] = int psi_m d_r psi_n, exact with a
    # rule of degree 2N-1 at interior points (orthonormal basis).
    qpts, qw = tet_quadrature(order + 1)
    psi_q = pkdo_tet(order, qpts)
    dpsi_q = pkdo_tet_grad_interior(order, qpts)
    cmod = np.einsum("q,qm,rqn->rmn", qw, psi_q, dpsi_q)
    diff = np.einsum("pm,rmn,nk->rpk", vdm, cmod, vinv)
    weak_diff = np.einsum("pm,rnm,nk->rpk", vdm, cmod, vinv)

    fnodes = _face_node_lists(order)
    fref = face_reference_nodes(order)
    v2 = pkdo_tri(order, fref)
    v2inv = np.linalg.inv(v2)
    fmass = v2inv.T @ v2inv
    nfp = fref.shape[0]
    emat = np.zeros((npn, NFACES, nfp))
    for f in range(NFACES):
        emat[fnodes[f], f, :] = fmass
    lift = np.einsum("ik,kfj->ifj", vdm @ vdm.T, emat)

    arrs = dict(nodes=nodes, vdm=vdm, mass=mass, diff=diff,
                weak_diff=weak_diff, face_nodes=fnodes, face_mass=fmass,
                lift=lift)
    for v in arrs.values():
        v.setflags(write=False)
    return ReferenceTet(order=order, face_perm=_face_permutation_maps(order),
                        **arrs)


# }}}


# {{{ the reference triangle (2D meshes)

#: local vertex indices of each edge of a triangle, meshmode's order (edge k
#: leaves out vertex 2 - k, like the tetrahedron's face k leaves out 3 - k)
TRI_FACE_VERTICES = ((0, 1), (2, 0), (1, 2))
TRI_FACE_OPPOSITE_VERTEX = (2, 1, 0)
TRI_NFACES = 3


def pkdo_tri_grad_interior(order: int, x: np.ndarray) -> np.ndarray:
    """(2, npoints, Np) gradient of :func:`pkdo_tri` at points strictly
    inside the triangle, by dual numbers."""
    npt = x.shape[0]
    eye = np.eye(2)
    r = Dual(x[:, 0], np.outer(eye[0], np.ones(npt)))
    s = Dual(x[:, 1], np.outer(eye[1], np.ones(npt)))
    a = 2.0 * (1.0 + r) / (1.0 - s) - 1.0
    b = s
    cols = []
    for (i, j) in multi_indices(2, order):
        pa = jacobi_orthonormal(a, 0.0, 0.0, i)[i]
        pb = jacobi_orthonormal(b, 2 * i + 1.0, 0.0, j)[j]
        cols.append((math.sqrt(2.0) * pa * pb * (1 - b) ** i).grad)
    return np.stack(cols, axis=2)


def legendre_orthonormal_1d(order: int, x: np.ndarray) -> np.ndarray:
    """(npoints, N+1) orthonormal Legendre polynomials on [-1, 1]."""
    return np.stack(jacobi_orthonormal(x, 0.0, 0.0, order), axis=1)


@dataclass(frozen=True)
class ReferenceTri:
    """Per-order constants of the nodal DG discretisation on triangles.

    Array shapes use Np = (N+1)(N+2)/2 volume nodes and Nfp = N+1 nodes per
    edge; the fields match :class:`ReferenceTet` with 2 reference axes and
    3 faces."""

    order: int
    nodes: np.ndarray            # (Np, 2) biunit-triangle coordinates
    vdm: np.ndarray              # (Np, Np)
    mass: np.ndarray             # (Np, Np)
    diff: np.ndarray             # (2, Np, Np) strong D_r
    weak_diff: np.ndarray        # (2, Np, Np) M^-1 S_r^T
    face_nodes: np.ndarray       # (3, Nfp) volume-node index of each edge node
    face_mass: np.ndarray        # (Nfp, Nfp) biunit-segment mass on the edge nodes
    lift: np.ndarray             # (Np, 3, Nfp) M^-1 E
    face_perm: dict              # vertex permutation of an edge -> (Nfp,) node map

    @property
    def np_(self) -> int:
        return self.nodes.shape[0]

    @property
    def nfp(self) -> int:
        return self.face_nodes.shape[1]


def _tri_face_node_lists(order: int) -> np.ndarray:
    """(3, Nfp): for edge k with local vertices (a, b), the volume nodes with
    barycentric multi-index (N - i at a, i at b), i = 0..N (from a to b)."""
    bary_mi = {(order - sum(mi),) + tuple(mi): idx
               for idx, mi in enumerate(multi_indices(2, order))}
    out = []
    for (a, b) in TRI_FACE_VERTICES:
        row = []
        for i in range(order + 1):
            alpha = [0, 0, 0]
            alpha[a] = order - i
            alpha[b] = i
            row.append(bary_mi[tuple(alpha)])
        out.append(row)
    return np.array(out, dtype=np.int64)


@lru_cache(maxsize=None)
def reference_tri(order: int) -> ReferenceTri:
    if order < 1:
        raise ValueError("order must be >= 1")
    nodes = barycentric_to_biunit(recursive_barycentric_nodes(2, order))
    npn = nodes.shape[0]
    vdm = pkdo_tri(order, nodes)
    vinv = np.linalg.inv(vdm)
    mass = vinv.T @ vinv
    qpts, qw = tri_quadrature(order + 1)
    psi_q = pkdo_tri(order, qpts)
    dpsi_q = pkdo_tri_grad_interior(order, qpts)
    cmod = np.einsum("q,qm,rqn->rmn", qw, psi_q, dpsi_q)
    diff = np.einsum("pm,rmn,nk->rpk", vdm, cmod, vinv)
    weak_diff = np.einsum("pm,rnm,nk->rpk", vdm, cmod, vinv)

    fnodes = _tri_face_node_lists(order)
    g = 2.0 * np.array(gll_points_01(order)) - 1.0       # edge nodes on [-1, 1]
    v1 = legendre_orthonormal_1d(order, g)
    v1inv = np.linalg.inv(v1)
    fmass = v1inv.T @ v1inv
    nfp = order + 1
    emat = np.zeros((npn, TRI_NFACES, nfp))
    for f in range(TRI_NFACES):
        emat[fnodes[f], f, :] = fmass
    lift = np.einsum("ik,kfj->ifj", vdm @ vdm.T, emat)
    # edge gluing: the neighbour runs its edge in the opposite direction
    # (conforming meshes) or in the same one
    perm = {(0, 1): np.arange(nfp, dtype=np.int64),
            (1, 0): np.arange(nfp, dtype=np.int64)[::-1].copy()}
    arrs = dict(nodes=nodes, vdm=vdm, mass=mass, diff=diff, weak_diff=weak_diff,
                face_nodes=fnodes, face_mass=fmass, lift=lift)
    for v in arrs.values():
        v.setflags(write=False)
    return ReferenceTri(order=order, face_perm=perm, **arrs)


# }}}

"""The oracle's own reference element (``oracle/refelem.py``) against
published values and against the product's node layout.

Published values: the Gauss-Lobatto-Legendre points of orders 2-4 on [-1, 1]
(0; +-1/sqrt(5); 0 and +-sqrt(3/7)), the equispaced vertices and edge
midpoints of order 2, the face centroids of order 3 and the volume centroid
of order 4; the order-4 face-interior node of the recursive family from its
defining formula (facet projections weighted by the GLL points of order 4).
The product's node set and order are compared with the oracle's built
independently."""

from __future__ import annotations

import math

import numpy as np
import pytest

from oracle import refelem as O


def test_gll_points_match_published_values():
    np.testing.assert_allclose(2 * O.gll_01(2) - 1, [-1, 0, 1], atol=1e-15)
    s5 = 1 / math.sqrt(5)
    np.testing.assert_allclose(2 * O.gll_01(3) - 1, [-1, -s5, s5, 1], atol=1e-15)
    s37 = math.sqrt(3 / 7)
    np.testing.assert_allclose(2 * O.gll_01(4) - 1, [-1, -s37, 0, s37, 1], atol=1e-15)


def test_low_order_nodes_are_vertices_midpoints_and_centroids():
    # order 2: vertices and edge midpoints of the biunit tetrahedron
    x2 = O.tet_nodes(2)
    pts = {tuple(np.round(p, 12)) for p in x2}
    v = O.TET_VERTICES
    want = {tuple(np.round(p, 12)) for p in v}
    want |= {tuple(np.round((v[a] + v[b]) / 2, 12)) for a in range(4) for b in range(a + 1, 4)}
    assert pts == want
    # order 3: the four face centroids are nodes
    x3 = O.tet_nodes(3)
    for fv in O.FACES:
        c = v[list(fv)].mean(axis=0)
        assert np.min(np.linalg.norm(x3 - c, axis=1)) < 1e-14
    # order 4: the centroid is the one interior node
    x4 = O.tet_nodes(4)
    assert np.min(np.linalg.norm(x4 - v.mean(axis=0), axis=1)) < 1e-14
    assert len(x4) == 35 and len(O.tri_nodes(4)) == 15


def test_order4_face_interior_node_from_its_definition():
    x4, x3 = O.gll_01(4), O.gll_01(3)
    a = (1 + 1 / math.sqrt(5)) / 2
    num = x4[2] * np.array([0, 0.5, 0.5]) + x4[3] * (np.array([a, 0, 1 - a])
                                                     + np.array([a, 1 - a, 0]))
    want = num / (x4[2] + 2 * x4[3])
    np.testing.assert_allclose(O.barycentric_node((2, 1, 1)), want, atol=1e-15)
    np.testing.assert_allclose(x3[2], a, atol=1e-15)
    # symmetric, inside the face, on neither an edge nor the centroid
    b = O.barycentric_node((2, 1, 1))
    assert abs(b[1] - b[2]) < 1e-15 and abs(b.sum() - 1) < 1e-15
    assert b[0] > 1 / 3 and b.min() > 0


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_face_nodes_of_the_volume_are_the_triangle_nodes(order):
    """Each face's volume nodes are the triangle nodes mapped onto it."""
    x = O.tet_nodes(order)
    for fv in O.FACES:
        l1 = (O.tri_nodes(order)[:, 0] + 1) / 2
        l2 = (O.tri_nodes(order)[:, 1] + 1) / 2
        mapped = np.stack([1 - l1 - l2, l1, l2], axis=1) @ O.TET_VERTICES[list(fv)]
        d = np.linalg.norm(mapped[:, None, :] - x[None, :, :], axis=2)
        assert np.all(d.min(axis=1) < 1e-14)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_product_nodes_match_the_oracle(order):
    from actx_dgfem_suite_gb300.refelem import reference_tet
    np.testing.assert_allclose(reference_tet(order).nodes, O.tet_nodes(order),
                               rtol=0, atol=1e-14)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_quadrature_exactness(order):
    """The collapsed rule the oracle assembles with integrates monomials of
    degree <= 2N + 1 exactly (closed form on the unit simplex:
    a! b! c! / (a + b + c + 3)!)."""
    q, w = O.tet_rule(order + 2)
    q = np.array([[float(v) for v in p] for p in q])
    w = np.array([float(v) for v in w])
    u = (q + 1) / 2                      # unit tetrahedron coordinates
    for a, b, c in [(0, 0, 0), (2, 1, 0), (order, order, 1), (2 * order + 1, 0, 0)]:
        exact = math.factorial(a) * math.factorial(b) * math.factorial(c) \
            / math.factorial(a + b + c + 3) * 8
        got = np.sum(w * u[:, 0] ** a * u[:, 1] ** b * u[:, 2] ** c)
        assert abs(got - exact) <= 1e-14 * max(1.0, exact)

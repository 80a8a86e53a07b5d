"""Reference tetrahedron: node set, basis, operators (CPU)."""

import numpy as np
import pytest

from actx_dgfem_suite_gb300 import refelem as R


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_basis_orthonormal(order):
    q, w = R.tet_quadrature(order + 2)
    P = R.pkdo_tet(order, q)
    assert np.abs(P.T @ (w[:, None] * P) - np.eye(P.shape[1])).max() < 1e-13
    q2, w2 = R.tri_quadrature(order + 2)
    P2 = R.pkdo_tri(order, q2)
    assert np.abs(P2.T @ (w2[:, None] * P2) - np.eye(P2.shape[1])).max() < 1e-13


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_node_counts_and_symmetry(order):
    ref = R.reference_tet(order)
    assert ref.np_ == (order + 1) * (order + 2) * (order + 3) // 6
    assert ref.nfp == (order + 1) * (order + 2) // 2
    bary = R.recursive_barycentric_nodes(3, order)
    assert np.allclose(bary.sum(axis=1), 1.0, atol=1e-15)
    # the node set is invariant under every vertex permutation
    import itertools
    key = {tuple(np.round(b, 12)) for b in bary}
    for p in itertools.permutations(range(4)):
        assert {tuple(np.round(b[list(p)], 12)) for b in bary} == key


def test_p1_to_p3_nodes_are_gll_on_edges():
    # P3: edge nodes at the 1D GLL points (1 -+ 1/sqrt 5)/2
    g = R.gll_points_01(3)
    assert np.allclose(g, [0, (1 - 1 / np.sqrt(5)) / 2, (1 + 1 / np.sqrt(5)) / 2, 1],
                       atol=1e-15)
    g4 = R.gll_points_01(4)
    assert np.allclose(g4, [0, (1 - np.sqrt(3 / 7)) / 2, 0.5, (1 + np.sqrt(3 / 7)) / 2, 1],
                       atol=1e-15)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_derivative_exact_on_polynomials(order):
    ref = R.reference_tet(order)
    x = ref.nodes
    for (a, b, c) in R.multi_indices(3, order):
        f = x[:, 0] ** a * x[:, 1] ** b * x[:, 2] ** c
        grads = [a * x[:, 0] ** max(a - 1, 0) * x[:, 1] ** b * x[:, 2] ** c,
                 b * x[:, 0] ** a * x[:, 1] ** max(b - 1, 0) * x[:, 2] ** c,
                 c * x[:, 0] ** a * x[:, 1] ** b * x[:, 2] ** max(c - 1, 0)]
        for r in range(3):
            assert np.abs(ref.diff[r] @ f - grads[r]).max() < 1e-12


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_face_nodes_are_2d_recursive_nodes(order):
    ref = R.reference_tet(order)
    bary2 = R.recursive_barycentric_nodes(2, order)
    for f, fv in enumerate(R.FACE_VERTICES):
        mapped = bary2 @ R.BIUNIT_TET_VERTICES[list(fv)]
        assert np.abs(mapped - ref.nodes[ref.face_nodes[f]]).max() < 1e-14


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_operators_match_quadrature_assembly(order):
    """Nodal-shortcut operators == oracle's quadrature-assembled matrices."""
    from oracle.refops import oracle_ref_ops
    ref = R.reference_tet(order)
    o = oracle_ref_ops(order)
    minv = np.linalg.inv(o.mass)
    wd = np.einsum("ik,rkj->rij", minv, o.stiff_t)
    lift = np.einsum("ik,kfj->ifj", minv, o.face_mass)
    assert np.abs(o.mass - ref.mass).max() < 1e-14
    assert np.abs(wd - ref.weak_diff).max() / np.abs(wd).max() < 1e-13
    assert np.abs(o.diff - ref.diff).max() / np.abs(o.diff).max() < 1e-13
    assert np.abs(lift - ref.lift).max() / np.abs(lift).max() < 1e-13


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_weak_strong_identity(order):
    """M W_r = D_r^T M (weak derivative is the mass-weighted transpose)."""
    ref = R.reference_tet(order)
    for r in range(3):
        lhs = ref.mass @ ref.weak_diff[r]
        rhs = ref.diff[r].T @ ref.mass
        assert np.abs(lhs - rhs).max() < 1e-12


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_face_permutation_maps(order):
    """Gluing by a vertex permutation maps face nodes onto the same points."""
    ref = R.reference_tet(order)
    bary2 = R.recursive_barycentric_nodes(2, order)
    for p, m in ref.face_perm.items():
        # our node j at weights bary2[j] over (v0,v1,v2); neighbour vertex x = our p[x]
        nb = bary2[m]                               # neighbour's weights
        ours_on_nb = bary2[:, list(p)]              # our weights read in nb's order
        assert np.abs(nb - ours_on_nb).max() < 1e-14

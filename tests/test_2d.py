"""Triangle meshes (the suite's dim = 2 runs), without a GPU: the product's
reference triangle and 2D discretisation against the oracle's independent
construction, the oracle's 2D operators against known answers, and the
builders' 2D problem setup."""

from __future__ import annotations

import numpy as np
import pytest

from actx_dgfem_suite_gb300.discretization2d import (
    make_box_discretization_2d,
    make_discretization_2d,
)
from actx_dgfem_suite_gb300.refelem import TRI_FACE_VERTICES, reference_tri
from tests._helpers import jittered_square_mesh


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_reference_triangle_matches_oracle(order):
    from oracle.refops import oracle_ref_ops_2d
    r = reference_tri(order)
    o = oracle_ref_ops_2d(order)
    assert np.abs(r.nodes - o.nodes).max() < 1e-14        # same nodes, same order
    assert np.abs(r.mass - o.mass).max() < 1e-14
    assert np.abs(r.diff - o.diff).max() < 1e-13
    # weak derivative = M^-1 S_r^T, LIFT = M^-1 E
    weak = np.einsum("ik,rkj->rij", np.linalg.inv(o.mass), o.stiff_t)
    assert np.abs(r.weak_diff - weak).max() < 1e-12
    lift = np.linalg.solve(o.mass, o.face_mass.reshape(o.mass.shape[0], -1))
    assert np.abs(r.lift - lift.reshape(r.lift.shape)).max() < 1e-12


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_reference_triangle_edges(order):
    r = reference_tri(order)
    assert r.np_ == (order + 1) * (order + 2) // 2 and r.nfp == order + 1
    from oracle.refelem import gll_01
    g = 2 * gll_01(order) - 1
    verts = np.array([[-1.0, -1.0], [1.0, -1.0], [-1.0, 1.0]])
    for f, (a, b) in enumerate(TRI_FACE_VERTICES):
        # edge nodes run from vertex a to vertex b at the GLL points
        want = ((1 - g)[:, None] * verts[a] + (1 + g)[:, None] * verts[b]) / 2
        assert np.abs(r.nodes[r.face_nodes[f]] - want).max() < 1e-14
    # integration by parts: S_r + S_r^T = sum_f n_r,f sJ_f E_f (reference element)
    m = r.mass
    s = np.einsum("ij,rjk->rik", m, r.diff)
    e = np.einsum("ij,jfk->ifk", m, r.lift)
    nrm = np.array([[0.0, -1.0], [-1.0, 0.0], [1.0, 1.0]]) / np.array([1, 1, np.sqrt(2)])[:, None]
    sj = np.array([1.0, 1.0, np.sqrt(2)])
    for rr in range(2):
        bnd = np.zeros_like(m)
        for f in range(3):
            bnd[:, r.face_nodes[f]] += nrm[f, rr] * sj[f] * e[:, f, :]
        assert np.abs(s[rr] + s[rr].T - bnd).max() < 1e-12


@pytest.mark.parametrize("order", [1, 3])
def test_discretization_2d_geometry_and_gather(order):
    d = make_discretization_2d(jittered_square_mesh(5), order)
    x = d.nodes().reshape(2, -1)
    own = np.arange(d.nelements)[:, None, None] * d.np_ + d.ref.face_nodes[None]
    assert np.abs(x[:, d.ext_index] - x[:, own]).max() < 1e-14
    assert d.is_boundary.sum() == 4 * 5
    assert np.allclose(np.linalg.norm(d.normal, axis=2), 1.0)
    ev = d.mesh.vertices[d.mesh.elements]
    cent = ev.mean(axis=1)
    for f, (a, b) in enumerate(TRI_FACE_VERTICES):
        mid = 0.5 * (ev[:, a] + ev[:, b])
        assert np.all(np.einsum("ex,ex->e", d.normal[:, f], mid - cent) > 0)
    assert abs(d.jac.sum() * 2.0 - 1.0) < 1e-12              # area of [0,1]^2
    g = d.gather_index()
    assert g.dtype == np.uint32 and g.shape == (d.nelements, 3, d.nfp)
    assert np.all((g[d.is_boundary] >> 31) == 1)
    fg = d.face_geometry()
    assert fg.shape == (d.nelements, 3, 4) and np.all(fg[..., 3] == 0)


def test_product_nodes_match_oracle_nodes():
    from oracle.geometry import build_oracle_disc_2d
    from tests._helpers import check_node_layout
    for order in (1, 2, 3, 4):
        d = make_box_discretization_2d(order, 3)
        od = build_oracle_disc_2d(d.mesh.vertices, d.mesh.elements, order)
        check_node_layout(d, od)
        assert np.array_equal(od.bdry, d.is_boundary)


# {{{ oracle known answers in 2D


def _od(order, n=4):
    from oracle.geometry import build_oracle_disc_2d
    m = jittered_square_mesh(n, seed=order)
    return build_oracle_disc_2d(m.vertices, m.elements, order)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_oracle_2d_wave_polynomial_exactness(order):
    from oracle.rhs import wave_rhs
    d = _od(order)
    x, y = d.nodes
    u = x ** order + y
    v = np.stack([y ** order, x * y ** (order - 1)])
    ru, rv = wave_rhs(d, u, v)
    inner = ~d.bdry.any(axis=1)          # no boundary edge: continuous data, no jumps
    # weak form: rhs_v = c grad u, rhs_u = c div v on elements away from the boundary
    assert np.abs(rv[0] - order * x ** (order - 1))[inner].max() < 1e-11
    assert np.abs(rv[1] - 1.0)[inner].max() < 1e-11
    div = (order - 1) * x * y ** (order - 2) if order > 1 else 0 * x
    assert np.abs(ru - div)[inner].max() < 1e-11


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_oracle_2d_euler_free_stream_and_conservation(order):
    from oracle.rhs import euler_rhs
    d = _od(order)
    x, _ = d.nodes
    q = np.stack([np.ones_like(x), 2.5 + 0 * x, 0 * x, 0 * x])
    assert np.abs(euler_rhs(d, q)).max() < 1e-12
    # walls: mass and energy are conserved, sum_e J 1^T M rhs = 0
    rng = np.random.default_rng(order)
    q = np.stack([1 + 0.1 * rng.random(x.shape), 2.5 + 0.1 * rng.random(x.shape),
                  0.05 * rng.standard_normal(x.shape), 0.05 * rng.standard_normal(x.shape)])
    r = euler_rhs(d, q)
    w = d.ops.mass.sum(axis=0)
    for k in (0, 1):
        total = float(np.einsum("i,ei,e->", w, r[k], d.jac))
        assert abs(total) < 1e-12 * float(np.abs(r[k]).max() + 1.0)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_oracle_2d_maxwell_energy(order):
    from oracle.rhs import maxwell_rhs
    d = _od(order)
    rng = np.random.default_rng(order)
    w = rng.standard_normal((3,) + d.nodes.shape[1:])
    mw = np.einsum("ij,kej->kei", d.ops.mass, w) * d.jac[None, :, None]
    central = float((mw * maxwell_rhs(d, w, 0.0)).sum())
    upwind = float((mw * maxwell_rhs(d, w, 1.0)).sum())
    assert abs(central) < 1e-11 * float(np.abs(mw).sum())       # energy conserved
    assert upwind < -1e-3                                       # and dissipated


# }}}


@pytest.mark.parametrize("eq,nf", [("wave", 3), ("euler", 4), ("maxwell", 3)])
def test_builders_2d_problem_setup(eq, nf):
    from actx_dgfem_suite_gb300.rhs_builder import get_problem
    from actx_dgfem_suite_gb300.utils import get_nel_1d_for_regular_rect_mesh
    for order in (1, 2, 3, 4):
        p = get_problem("tiny_" + eq, 2, order)
        n = get_nel_1d_for_regular_rect_mesh(2, order, 1_000)
        assert p.dim == 2 and p.disc.nelements == 2 * n * n
        assert p.fields.shape == (nf, 2 * n * n, (order + 1) * (order + 2) // 2)
    p = get_problem("tiny_" + eq, 2, 2, definition="reference")
    x, y = p.disc.nodes()
    if eq == "wave":        # bump at (0.2, 0.35), wave.py:216-236
        want = np.exp(-((x - 0.2) ** 2 + (y - 0.35) ** 2) / 0.05 ** 2)
        assert np.array_equal(p.fields[0], want) and not p.fields[1:].any()
    elif eq == "euler":
        assert np.all(p.fields[0] == 1.0) and not p.fields[2:].any()
    else:
        assert np.allclose(p.fields[0], np.sin(2 * np.pi * x) * np.sin(3 * np.pi * y))
        assert not p.fields[1:].any()


def test_ensembles_refuse_triangle_meshes():
    from actx_dgfem_suite_gb300.discretization import union_discretization
    d = make_box_discretization_2d(2, 3)
    with pytest.raises(NotImplementedError):
        union_discretization([d, d])


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_oracle_2d_maxwell_tm_curls_are_exact(order):
    """Continuous polynomial TM fields of degree <= N: away from the boundary
    (no jumps, so no flux) the RHS is E_z' = dH_y/dx - dH_x/dy,
    H_x' = -dE_z/dy, H_y' = dE_z/dx (epsilon = mu = 1)."""
    from oracle.rhs import maxwell_rhs
    d = _od(order)
    x, y = d.nodes
    ez = x ** order + 2 * y
    hx = y ** order - x
    hy = x * y ** (order - 1) + 3 * x
    r = maxwell_rhs(d, np.stack([ez, hx, hy]), 0.5)
    inner = ~d.bdry.any(axis=1)
    dhy_dx = y ** (order - 1) + 3
    dhx_dy = order * y ** (order - 1)
    assert np.abs(r[0] - (dhy_dx - dhx_dy))[inner].max() < 1e-10
    assert np.abs(r[1] - (-2.0))[inner].max() < 1e-10
    assert np.abs(r[2] - order * x ** (order - 1))[inner].max() < 1e-10

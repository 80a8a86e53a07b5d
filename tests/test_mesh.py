"""Box mesh, geometry and face connectivity (CPU)."""

import numpy as np
import pytest

from actx_dgfem_suite_gb300.discretization import (BOUNDARY_FLAG,
                                                   make_box_discretization,
                                                   make_discretization)
from actx_dgfem_suite_gb300.mesh import generate_box_tet_mesh
from actx_dgfem_suite_gb300.refelem import FACE_VERTICES
from actx_dgfem_suite_gb300.utils import (get_ndof_for_regular_rect_mesh,
                                          get_nel_1d_for_regular_rect_mesh)


@pytest.mark.parametrize("n", [1, 2, 3])
def test_box_mesh_counts_and_volume(n):
    m = generate_box_tet_mesh(-0.5, 0.5, n)
    assert m.nelements == 6 * n**3
    assert m.vertices.shape[0] == (n + 1) ** 3
    d = make_box_discretization(2, n)
    assert np.isclose((d.jac * 4 / 3).sum(), 1.0, rtol=1e-14)
    assert np.all(d.jac > 0)
    assert d.is_boundary.sum() == 6 * 2 * n * n


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_connectivity_matches_coordinates(order):
    d = make_box_discretization(order, 3)
    x = d.nodes().reshape(3, -1)
    own = np.arange(d.nelements)[:, None, None] * d.np_ + d.ref.face_nodes[None]
    assert np.abs(x[:, d.ext_index] - x[:, own]).max() < 1e-14
    nb, nf = d.neighbor, d.neighbor_face
    inter = nb >= 0
    e = np.nonzero(inter)
    assert np.all(nb[nb[e], nf[e]] == e[0])
    assert np.all(nf[nb[e], nf[e]] == e[1])
    # opposite normals across interior faces
    assert np.abs(d.normal[inter] + d.normal[nb[inter], nf[inter]]).max() < 1e-14


def test_connectivity_matches_oracle():
    from oracle.geometry import build_oracle_disc
    from tests._helpers import jittered_box_mesh
    m = jittered_box_mesh(3)
    for order in (1, 3, 4):
        d = make_discretization(m, order)
        od = build_oracle_disc(m.vertices, m.elements, order)
        assert np.array_equal(od.ext_idx, d.ext_index)
        assert np.array_equal(od.bdry, d.is_boundary)
        assert np.abs(od.normal - d.normal).max() < 1e-14
        assert np.abs(od.sj - d.face_jac).max() < 1e-14


def test_outward_normals_and_gather_format():
    d = make_box_discretization(2, 2)
    ev = d.mesh.vertices[d.mesh.elements]
    fc = ev[:, np.array(FACE_VERTICES)].mean(axis=2)
    ec = ev.mean(axis=1)
    assert (((fc - ec[:, None]) * d.normal).sum(-1) > 0).all()
    g = d.gather_index()
    assert g.dtype == np.uint32
    bd = (g & BOUNDARY_FLAG) != 0
    assert np.array_equal(bd.all(axis=2), d.is_boundary)
    low = (g & ~BOUNDARY_FLAG).astype(np.int64)
    assert low.max() < d.nelements * d.np_
    fg = d.face_geometry()
    assert np.allclose(np.linalg.norm(fg[:, :, :3], axis=2), 1.0)


def test_nel_1d_matches_reference_sizes():
    # large_ (2e7 DOFs) sizes are the benchmark grids 95/70/56/46
    assert [get_nel_1d_for_regular_rect_mesh(3, p, 20_000_000) for p in (1, 2, 3, 4)] \
        == [95, 70, 56, 46]
    assert [get_nel_1d_for_regular_rect_mesh(3, p, 1_000) for p in (1, 2, 3, 4)] \
        == [4, 3, 3, 2]
    assert get_ndof_for_regular_rect_mesh(3, 3, 56) == 6 * 56**3 * 20
    with pytest.raises(NotImplementedError):
        get_nel_1d_for_regular_rect_mesh(3, 7, 1000)


def test_nonmanifold_mesh_rejected():
    from actx_dgfem_suite_gb300.mesh import TetMesh
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, -1], [1, 1, 1.0]])
    el = np.array([[0, 1, 2, 3], [0, 2, 1, 4], [0, 1, 2, 5]])
    # element orientation: make all positive first
    m = TetMesh(v, el)
    with pytest.raises(ValueError):
        make_discretization(m, 1)


def test_union_discretization_offsets():
    from actx_dgfem_suite_gb300.discretization import union_discretization
    a = make_box_discretization(2, 2)
    b = make_box_discretization(2, 3, 0.0, 2.0)
    u, offs = union_discretization([a, b])
    assert list(offs) == [a.nelements, a.nelements + b.nelements][:0] + [0, a.nelements, a.nelements + b.nelements]
    assert u.nelements == a.nelements + b.nelements
    # member b's exterior indices point into member b only
    eb = u.ext_index[a.nelements:]
    assert eb.min() >= a.nelements * u.np_
    assert np.array_equal(u.ext_index[:a.nelements], a.ext_index)
    x = u.nodes().reshape(3, -1)
    own = np.arange(u.nelements)[:, None, None] * u.np_ + u.ref.face_nodes[None]
    assert np.abs(x[:, u.ext_index] - x[:, own]).max() < 1e-14


@pytest.mark.parametrize("order", [1, 2, 4])
def test_face_partner_is_an_involution(order):
    from tests._helpers import jittered_box_mesh
    d = make_discretization(jittered_box_mesh(3), order)
    p = d.face_partner().reshape(-1).astype(np.int64)
    inter = p >= 0
    idx = np.arange(p.size)
    assert np.array_equal(p[p[inter]], idx[inter])
    # partner face points sit at the same physical node as the exterior index
    nfpt = 4 * d.nfp
    fn = d.ref.face_nodes.reshape(-1)
    node_of_fp = (idx // nfpt) * d.np_ + fn[idx % nfpt]
    assert np.array_equal(node_of_fp[p[inter]], d.ext_index.reshape(-1)[inter])
    assert np.array_equal(~inter.reshape(d.nelements, 4, -1).all(axis=2), d.is_boundary)

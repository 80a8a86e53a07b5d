"""Host-side pieces of the adjoint path (CPU): receivers, checkpoint sizing."""

import numpy as np
import torch

from actx_dgfem_suite_gb300.adjoint import (Receivers, locate_points,
                                            random_interior_points)
from actx_dgfem_suite_gb300.discretization import make_box_discretization


def test_receivers_interpolate_polynomials_exactly():
    d = make_box_discretization(3, 3, -1.0, 1.0)
    pts = random_interior_points(20, (-1, -1, -1), (1, 1, 1), 0.05, seed=2)
    rec = Receivers(d, pts, "cpu")
    x, y, z = d.nodes()
    f = 1 + x**3 - 2 * x * y * z + z**2
    q = torch.zeros((4,) + f.shape, dtype=torch.float64)
    q[0] = torch.from_numpy(f)
    got = rec.sample(q).numpy()
    px, py, pz = pts.T
    assert np.abs(got - (1 + px**3 - 2 * px * py * pz + pz**2)).max() < 1e-12


def test_inject_is_the_transpose_of_sample():
    d = make_box_discretization(2, 2, -1.0, 1.0)
    pts = random_interior_points(30, (-1, -1, -1), (1, 1, 1), 0.05, seed=3)
    pts[5] = pts[4] + 1e-3          # two receivers in one element
    rec = Receivers(d, pts, "cpu")
    g = torch.from_numpy(np.random.default_rng(0).standard_normal(30))
    q = torch.from_numpy(np.random.default_rng(1).standard_normal((4, d.nelements, d.np_)))
    lam = torch.zeros_like(q)
    rec.inject(lam, g)
    assert abs(float((rec.sample(q) * g).sum()) - float((q * lam).sum())) < 1e-12


def test_locate_points_barycentric():
    d = make_box_discretization(1, 2, 0.0, 1.0)
    pts = np.array([[0.1, 0.2, 0.3], [0.9, 0.8, 0.7]])
    el, ref = locate_points(d, pts)
    verts = d.mesh.vertices[d.mesh.elements[el]]
    lam1 = (ref + 1) / 2
    lam0 = 1 - lam1.sum(axis=1)
    back = lam0[:, None] * verts[:, 0] + np.einsum("pk,pkx->px", lam1, verts[:, 1:])
    assert np.abs(back - pts).max() < 1e-14

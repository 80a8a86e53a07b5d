"""Known-answer tests that pin the CPU oracle (the reference ships none).

1. wave: polynomial exactness on elements away from the boundary;
2. Euler: free-stream preservation (rest state everywhere, uniform flow in
   the interior);
3. Euler: discrete conservation of mass and energy with wall boundaries;
4. wave / Maxwell: semi-discrete energy stability (upwind dissipates,
   central conserves);
5. Maxwell: convergence of the cavity-mode RHS to the analytic -curl E;
6. linearity of the wave and Maxwell operators.
"""

import numpy as np
import pytest

from actx_dgfem_suite_gb300.discretization import make_box_discretization
from actx_dgfem_suite_gb300.equations.maxwell import rectangular_cavity_mode
from oracle.geometry import build_oracle_disc
from oracle.rhs import euler_rhs, maxwell_rhs, wave_rhs
from tests._helpers import jittered_box_mesh


def _od(order, n=3, a=-0.5, b=0.5, mesh=None):
    if mesh is None:
        d = make_box_discretization(order, n, a, b)
        mesh = d.mesh
    return build_oracle_disc(mesh.vertices, mesh.elements, order)


def _mass_inner(od, a, b):
    """sum_e J_e a_e^T M b_e"""
    return float(np.einsum("e,ei,ij,ej->", od.jac, a, od.ops.mass, b))


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_wave_polynomial_exactness(order):
    od = _od(order, mesh=jittered_box_mesh(3))
    x, y, z = od.nodes
    N = order
    u = x**N + 0.3 * y * z ** (N - 1) + 1
    v = np.stack([y**N, x * z ** (N - 1), 2 * z**N])
    ru, rv = wave_rhs(od, u, v)
    inner = ~od.bdry.any(axis=1)
    assert inner.sum() > 0
    div_v = 2 * N * z ** (N - 1)
    grad_u = [N * x ** (N - 1), 0.3 * z ** (N - 1),
              0.3 * y * (N - 1) * z ** max(N - 2, 0)]
    scale = max(np.abs(div_v).max(), 1.0)
    assert np.abs(ru[inner] - div_v[inner]).max() < 1e-11 * scale * 10
    for k in range(3):
        assert np.abs(rv[k][inner] - grad_u[k][inner]).max() < 1e-10


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_euler_free_stream(order):
    od = _od(order, mesh=jittered_box_mesh(3))
    shape = od.nodes.shape[1:]
    q = np.zeros((5,) + shape)
    q[0] = 1.0
    q[1] = 2.5
    assert np.abs(euler_rhs(od, q)).max() < 1e-10  # O(100) terms cancel
    # uniform flow: exact away from the walls
    u = np.array([0.3, -0.2, 0.1])
    q[2:5] = u[:, None, None]
    q[1] = 2.5 + 0.5 * (u**2).sum()
    r = euler_rhs(od, q)
    inner = ~od.bdry.any(axis=1)
    assert np.abs(r[:, inner]).max() < 1e-10


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_euler_conservation_with_walls(order):
    from tests._helpers import smooth_fields
    d = make_box_discretization(order, 3)
    od = build_oracle_disc(d.mesh.vertices, d.mesh.elements, order)
    q = smooth_fields(d, 5, "euler", seed=order)
    r = euler_rhs(od, q)
    ones = np.ones_like(q[0])
    mass_rate = _mass_inner(od, ones, r[0])
    energy_rate = _mass_inner(od, ones, r[1])
    scale = _mass_inner(od, np.abs(r[0]), ones) + _mass_inner(od, np.abs(r[1]), ones)
    assert abs(mass_rate) < 1e-13 * scale
    assert abs(energy_rate) < 1e-13 * scale


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_wave_energy_stability(order):
    from tests._helpers import smooth_fields
    d = make_box_discretization(order, 3)
    od = build_oracle_disc(d.mesh.vertices, d.mesh.elements, order)
    q = smooth_fields(d, 4, "wave", seed=order)
    ru, rv = wave_rhs(od, q[0], q[1:4])
    rate = _mass_inner(od, q[0], ru) + sum(_mass_inner(od, q[1 + k], rv[k]) for k in range(3))
    energy = _mass_inner(od, q[0], q[0]) + sum(_mass_inner(od, q[1 + k], q[1 + k]) for k in range(3))
    assert rate < 1e-12 * energy
    assert rate < -1e-6 * energy  # upwind dissipates on a non-smooth-in-h state


@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("alpha", [0.0, 0.5, 1.0])
def test_maxwell_energy(order, alpha):
    from tests._helpers import smooth_fields
    d = make_box_discretization(order, 3, 0.0, 1.0)
    od = build_oracle_disc(d.mesh.vertices, d.mesh.elements, order)
    w = smooth_fields(d, 6, "maxwell", seed=order)
    r = maxwell_rhs(od, w, alpha)
    rate = sum(_mass_inner(od, w[k], r[k]) for k in range(6))
    energy = sum(_mass_inner(od, w[k], w[k]) for k in range(6))
    scale = sum(_mass_inner(od, np.abs(w[k]), np.abs(r[k])) for k in range(6))
    if alpha == 0.0:
        assert abs(rate) < 1e-12 * scale   # central flux + PEC: conservative
    else:
        assert rate < 1e-12 * energy
        assert rate < 0.0


@pytest.mark.parametrize("order", [1, 2, 3])
def test_maxwell_cavity_mode_convergence(order):
    """rhs_H of the (1,2,2) cavity mode -> -curl E, rhs_E -> 0 (H = 0)."""
    errs = []
    for n in (2, 4):
        d = make_box_discretization(order, n, 0.0, 1.0)
        od = build_oracle_disc(d.mesh.vertices, d.mesh.elements, order)
        x, y, z = od.nodes
        w = np.real(rectangular_cavity_mode(od.nodes, 0.0))
        r = maxwell_rhs(od, w, 0.5)
        kx, ky, kz = np.pi, 2 * np.pi, 2 * np.pi
        g2 = kx**2 + ky**2
        sx, cx, sy, cy = np.sin(kx * x), np.cos(kx * x), np.sin(ky * y), np.cos(ky * y)
        sz, cz = np.sin(kz * z), np.cos(kz * z)
        ex_y = -kx * kz * cx * ky * cy * sz / g2
        ex_z = -kx * kz * cx * sy * kz * cz / g2
        ey_x = -ky * kz * kx * cx * cy * sz / g2
        ey_z = -ky * kz * sx * cy * kz * cz / g2
        ez_x = kx * cx * sy * cz
        ez_y = sx * ky * cy * cz
        curl_e = np.stack([ez_y - ey_z, ex_z - ez_x, ey_x - ex_y])
        exact = np.concatenate([np.zeros_like(curl_e), -curl_e])
        err = np.sqrt(sum(_mass_inner(od, r[k] - exact[k], r[k] - exact[k])
                          for k in range(6)))
        errs.append(err)
    rate = np.log2(errs[0] / errs[1])
    assert rate > order - 0.6, (errs, rate)


@pytest.mark.parametrize("order", [2, 4])
def test_linearity(order):
    from tests._helpers import smooth_fields
    d = make_box_discretization(order, 2, 0.0, 1.0)
    od = build_oracle_disc(d.mesh.vertices, d.mesh.elements, order)
    a = smooth_fields(d, 6, "maxwell", seed=1)
    b = smooth_fields(d, 6, "maxwell", seed=2)
    lhs = maxwell_rhs(od, 2.0 * a - 3.0 * b)
    rhs = 2.0 * maxwell_rhs(od, a) - 3.0 * maxwell_rhs(od, b)
    assert np.abs(lhs - rhs).max() < 1e-11 * np.abs(rhs).max()
    ua, va = a[0], a[1:4]
    ub, vb = b[0], b[1:4]
    l1, l2 = wave_rhs(od, ua + 0.5 * ub, va + 0.5 * vb)
    r1a, r2a = wave_rhs(od, ua, va)
    r1b, r2b = wave_rhs(od, ub, vb)
    assert np.abs(l1 - (r1a + 0.5 * r1b)).max() < 1e-11 * np.abs(l1).max()
    assert np.abs(l2 - (r2a + 0.5 * r2b)).max() < 1e-11 * np.abs(l2).max()

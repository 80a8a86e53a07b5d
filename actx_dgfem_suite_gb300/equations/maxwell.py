"""Maxwell's equations, mirroring ``actx_dgfem_suite/equations/maxwell.py``.

Operator: grudge's ``MaxwellOperator`` in 3D with constant epsilon, mu, the
alpha-weighted upwind flux (alpha = ``flux_type``) and PEC on all boundaries
(``maxwell.py:55-70``).  The state is (E_x, E_y, E_z, H_x, H_y, H_z).

Problem definitions:

* ``"reference"`` (``maxwell.py:43-74``): box [0, 1]^3, epsilon = mu = 1,
  alpha = 0.5, state = real part of the rectangular-cavity mode (1, 2, 2) at
  t = 0, called with t = 0.5.
* ``"baseline"``: box [0, 1]^3, epsilon = mu = 1, alpha = 1 (upwind), state =
  a seeded mix of eight plane waves with random directions, polarisations and
  phases.

With ``dim=2`` (triangles on [0, 1]^2) the operator is the TM restriction,
grudge's field subset for ``dimensions=2``: state (E_z, H_x, H_y).  The
reference definition uses the cavity mode (2, 3) (``maxwell.py:62-66``),
whose real part at t = 0 is E_z = sin(2 pi x) sin(3 pi y), H = 0; the
benchmark one a seeded mix of in-plane TM plane waves.
"""

from __future__ import annotations

import numpy as np

from actx_dgfem_suite_gb300.discretization import make_box_discretization
from actx_dgfem_suite_gb300.discretization2d import make_box_discretization_2d
from actx_dgfem_suite_gb300.equations.common import Problem, make_rhs_and_args
from actx_dgfem_suite_gb300.utils import get_nel_1d_for_regular_rect_mesh
from actx_dgfem_suite_gb300.xp import array_module, zeros

#: flux parameter alpha of each problem definition, box [0, 1]^3 for both
ALPHA = {"reference": 0.5, "baseline": 1.0}
BOXES = {"reference": (0.0, 1.0), "baseline": (0.0, 1.0)}


def rectangular_cavity_mode(nodes: np.ndarray, t: float = 0.0,
                            mode=(1, 2, 2)) -> np.ndarray:
    """Complex (6, ...) TM cavity mode of the unit cube (grudge's
    ``get_rectangular_cavity_mode`` in 3D, E_0 = 1)."""
    kx, ky, kz = (m * np.pi for m in mode)
    omega = np.sqrt(kx**2 + ky**2 + kz**2)
    x, y, z = nodes
    sx, cx = np.sin(kx * x), np.cos(kx * x)
    sy, cy = np.sin(ky * y), np.cos(ky * y)
    sz, cz = np.sin(kz * z), np.cos(kz * z)
    tdep = np.exp(-1j * omega * t)
    g2 = kx**2 + ky**2
    return np.stack([
        -kx * kz * cx * sy * sz * tdep / g2,
        -ky * kz * sx * cy * sz * tdep / g2,
        sx * sy * cz * tdep,
        -1j * omega * ky * sx * cy * cz * tdep / g2,
        1j * omega * kx * cx * sy * cz / g2 + 0 * x,
        0 * x + 0j,
    ])


def cavity_mode_real_t0(nodes, mode=(1, 2, 2)):
    """Real part of :func:`rectangular_cavity_mode` at t = 0: (E, 0), for
    NumPy arrays or torch tensors."""
    xp = array_module(nodes)
    kx, ky, kz = (m * np.pi for m in mode)
    x, y, z = nodes[0], nodes[1], nodes[2]
    sx, cx = xp.sin(kx * x), xp.cos(kx * x)
    sy, cy = xp.sin(ky * y), xp.cos(ky * y)
    sz, cz = xp.sin(kz * z), xp.cos(kz * z)
    g2 = kx**2 + ky**2
    out = zeros(x, (6,) + tuple(x.shape))
    out[0] = -kx * kz * cx * sy * sz / g2
    out[1] = -ky * kz * sx * cy * sz / g2
    out[2] = sx * sy * cz
    return out


def plane_wave_mix(nodes, seed: int = 0, nwaves: int = 8):
    """Sum of vacuum plane waves E = a e cos(k.x + phi), H = a (k^ x e)
    cos(k.x + phi), |k| in 2 pi [1, 3], from a fixed seed (parameters drawn
    on the host; ``nodes`` may be a NumPy array or a torch tensor)."""
    xp = array_module(nodes)
    rng = np.random.default_rng(seed)
    out = zeros(nodes, (6,) + tuple(nodes.shape[1:]))
    for _ in range(nwaves):
        khat = rng.normal(size=3)
        khat /= np.linalg.norm(khat)
        e = np.cross(khat, rng.normal(size=3))
        e /= np.linalg.norm(e)
        h = np.cross(khat, e)
        kmag = 2 * np.pi * rng.uniform(1.0, 3.0)
        amp = rng.uniform(0.5, 1.0)
        phase = rng.uniform(0.0, 2 * np.pi)
        arg = kmag * (khat[0] * nodes[0] + khat[1] * nodes[1]
                      + khat[2] * nodes[2]) + phase
        c = amp * xp.cos(arg)
        for i in range(3):
            out[i] += e[i] * c
            out[3 + i] += h[i] * c
    return out


def cavity_mode_tm_real_t0(nodes, mode=(2, 3)):
    """Real part at t = 0 of the 2D TM cavity mode of the unit square:
    (E_z, H_x, H_y) = (sin(kx x) sin(ky y), 0, 0)."""
    xp = array_module(nodes)
    kx, ky = (m * np.pi for m in mode)
    x, y = nodes[0], nodes[1]
    out = zeros(x, (3,) + tuple(x.shape))
    out[0] = xp.sin(kx * x) * xp.sin(ky * y)
    return out


def plane_wave_mix_tm(nodes, seed: int = 0, nwaves: int = 8):
    """Sum of in-plane TM vacuum plane waves E_z = a cos(k.x + phi),
    (H_x, H_y) = (k^_y, -k^_x) E_z, |k| in 2 pi [1, 3], from a fixed seed."""
    xp = array_module(nodes)
    rng = np.random.default_rng(seed)
    out = zeros(nodes, (3,) + tuple(nodes.shape[1:]))
    for _ in range(nwaves):
        theta = rng.uniform(0.0, 2 * np.pi)
        kx, ky = np.cos(theta), np.sin(theta)
        kmag = 2 * np.pi * rng.uniform(1.0, 3.0)
        amp = rng.uniform(0.5, 1.0)
        phase = rng.uniform(0.0, 2 * np.pi)
        ez = amp * xp.cos(kmag * (kx * nodes[0] + ky * nodes[1]) + phase)
        out[0] += ez
        out[1] += ky * ez
        out[2] += -kx * ez
    return out


def maxwell_problem(order: int, nel_1d: int, definition: str = "reference",
                    epsilon: float = 1.0, mu: float = 1.0, seed: int = 0,
                    dim: int = 3) -> Problem:
    if definition not in ALPHA:
        raise ValueError(f"unknown problem definition {definition!r}")
    disc = (make_box_discretization(order, nel_1d, 0.0, 1.0) if dim == 3
            else make_box_discretization_2d(order, nel_1d, 0.0, 1.0))
    fields = initial_state(disc.nodes(), definition, seed)
    return Problem("maxwell", disc, fields,
                   (ALPHA[definition], float(epsilon), float(mu)), 0.5, definition)


def initial_state(nodes, definition: str, seed: int = 0):
    if len(nodes) == 2:   # triangle meshes: TM fields
        if definition == "reference":
            return cavity_mode_tm_real_t0(nodes)
        if definition == "baseline":
            return plane_wave_mix_tm(nodes, seed=seed)
    elif definition == "reference":
        return cavity_mode_real_t0(nodes)
    elif definition == "baseline":
        return plane_wave_mix(nodes, seed=seed)
    raise ValueError(f"unknown problem definition {definition!r}")


def get_maxwell_rhs(*, actx, dim: int, order: int, ndofs: int,
                    definition: str = "reference", nel_1d: int | None = None):
    """``(rhs, (t, w))`` as ``maxwell.py:43-74`` (``dim`` 3: tetrahedra, 2:
    triangles with the TM fields)."""
    if dim not in (2, 3):
        raise NotImplementedError("dim must be 2 or 3")
    if nel_1d is None:
        nel_1d = get_nel_1d_for_regular_rect_mesh(dim, order, int(ndofs))
    return make_rhs_and_args(maxwell_problem(order, nel_1d, definition, dim=dim), actx)

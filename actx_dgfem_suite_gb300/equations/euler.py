"""Compressible Euler equations, mirroring ``actx_dgfem_suite/equations/euler.py``.

Operator: grudge's ``EulerOperator`` with gamma = 1.4, Lax-Friedrichs flux and
``InviscidWallBC`` on all boundaries, no over-integration
(``euler.py:168-179``).  The state order is mass, energy, momentum.

Problem definitions:

* ``"reference"`` (``euler.py:119-137, 140-186``): box [-0.5, 0.5]^3,
  rho = 1, momentum = 0, energy = 1/(gamma-1) + exp(-|x|^2 / (2 * 0.1^2)),
  called with t = 0.5.
* ``"baseline"``: box [-0.5, 0.5]^3, rho = 1 + 0.1 exp(-|x|^2 / 0.2^2),
  u = (0.1, 0, 0), p = 1.
"""

from __future__ import annotations

import numpy as np

from actx_dgfem_suite_gb300.discretization import make_box_discretization
from actx_dgfem_suite_gb300.equations.common import Problem, make_rhs_and_args
from actx_dgfem_suite_gb300.utils import get_nel_1d_for_regular_rect_mesh

GAMMA = 1.4


def acoustic_pulse_condition(nodes: np.ndarray, gamma: float = GAMMA) -> np.ndarray:
    """``euler.py:119-137`` (gaussian_profile with rhoamp = 0 plus make_pulse
    with width 0.1 at the origin); returns (5, Nel, Np)."""
    r2 = (nodes**2).sum(axis=0)
    mass = 0.0 * np.exp(1 - r2) + 1.0
    energy = 1.0 / (gamma - 1.0) + 0.0 / (2.0 * mass)
    pulse = np.exp(-0.5 * r2 / 0.1**2)
    out = np.zeros((5,) + r2.shape)
    out[0] = mass
    out[1] = energy + pulse
    return out


def density_pulse_condition(nodes: np.ndarray, gamma: float = GAMMA) -> np.ndarray:
    r2 = (nodes**2).sum(axis=0)
    rho = 1.0 + 0.1 * np.exp(-r2 / 0.2**2)
    u = np.array([0.1, 0.0, 0.0])
    p = 1.0
    out = np.zeros((5,) + r2.shape)
    out[0] = rho
    out[1] = p / (gamma - 1.0) + 0.5 * rho * (u**2).sum()
    for i in range(3):
        out[2 + i] = rho * u[i]
    return out


def euler_problem(order: int, nel_1d: int, definition: str = "reference",
                  gamma: float = GAMMA) -> Problem:
    disc = make_box_discretization(order, nel_1d, -0.5, 0.5)
    nodes = disc.nodes()
    if definition == "reference":
        fields = acoustic_pulse_condition(nodes, gamma)
    elif definition == "baseline":
        fields = density_pulse_condition(nodes, gamma)
    else:
        raise ValueError(f"unknown problem definition {definition!r}")
    return Problem("euler", disc, fields, (float(gamma),), 0.5, definition)


def get_euler_rhs(*, actx, dim: int, order: int, ndofs: int,
                  definition: str = "reference", nel_1d: int | None = None):
    """``(rhs, (t, ConservedEulerField))`` as ``euler.py:140-186``."""
    if dim != 3:
        raise NotImplementedError("only 3D tetrahedral meshes are implemented")
    if nel_1d is None:
        nel_1d = get_nel_1d_for_regular_rect_mesh(dim, order, int(ndofs))
    return make_rhs_and_args(euler_problem(order, nel_1d, definition), actx)

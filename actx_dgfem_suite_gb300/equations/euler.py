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

With ``dim=2`` the same definitions on the square [-0.5, 0.5]^2 with a
two-component momentum (state mass, energy, momentum_x, momentum_y).
"""

from __future__ import annotations

import numpy as np

from actx_dgfem_suite_gb300.discretization import make_box_discretization
from actx_dgfem_suite_gb300.discretization2d import make_box_discretization_2d
from actx_dgfem_suite_gb300.equations.common import Problem, make_rhs_and_args
from actx_dgfem_suite_gb300.utils import get_nel_1d_for_regular_rect_mesh
from actx_dgfem_suite_gb300.xp import array_module, r2, zeros

GAMMA = 1.4
#: box corners of each problem definition
BOXES = {"reference": (-0.5, 0.5), "baseline": (-0.5, 0.5)}


def acoustic_pulse_condition(nodes, gamma: float = GAMMA):
    """``euler.py:119-137`` (gaussian_profile with rhoamp = 0 plus make_pulse
    with width 0.1 at the origin); returns (2 + dim, Nel, Np).  ``nodes``:
    (dim, ...) NumPy array or torch tensor."""
    xp = array_module(nodes)
    rr = r2(nodes)
    mass = 0.0 * xp.exp(1 - rr) + 1.0
    energy = 1.0 / (gamma - 1.0) + 0.0 / (2.0 * mass)
    pulse = xp.exp(-0.5 * rr / 0.1**2)
    out = zeros(rr, (2 + len(nodes),) + tuple(rr.shape))
    out[0] = mass
    out[1] = energy + pulse
    return out


def density_pulse_condition(nodes, gamma: float = GAMMA):
    xp = array_module(nodes)
    rr = r2(nodes)
    rho = 1.0 + 0.1 * xp.exp(-rr / 0.2**2)
    dim = len(nodes)
    u = (0.1, 0.0, 0.0)[:dim]
    p = 1.0
    out = zeros(rr, (2 + dim,) + tuple(rr.shape))
    out[0] = rho
    out[1] = p / (gamma - 1.0) + 0.5 * rho * sum(c * c for c in u)
    for i in range(dim):
        out[2 + i] = rho * u[i]
    return out


def initial_state(nodes, definition: str, gamma: float = GAMMA):
    if definition == "reference":
        return acoustic_pulse_condition(nodes, gamma)
    if definition == "baseline":
        return density_pulse_condition(nodes, gamma)
    raise ValueError(f"unknown problem definition {definition!r}")


def euler_problem(order: int, nel_1d: int, definition: str = "reference",
                  gamma: float = GAMMA, dim: int = 3) -> Problem:
    if definition not in BOXES:
        raise ValueError(f"unknown problem definition {definition!r}")
    disc = (make_box_discretization(order, nel_1d, *BOXES[definition]) if dim == 3
            else make_box_discretization_2d(order, nel_1d, *BOXES[definition]))
    fields = initial_state(disc.nodes(), definition, gamma)
    return Problem("euler", disc, fields, (float(gamma),), 0.5, definition)


def get_euler_rhs(*, actx, dim: int, order: int, ndofs: int,
                  definition: str = "reference", nel_1d: int | None = None):
    """``(rhs, (t, ConservedEulerField))`` as ``euler.py:140-186`` (``dim`` 3:
    tetrahedra, 2: triangles)."""
    if dim not in (2, 3):
        raise NotImplementedError("dim must be 2 or 3")
    if nel_1d is None:
        nel_1d = get_nel_1d_for_regular_rect_mesh(dim, order, int(ndofs))
    return make_rhs_and_args(euler_problem(order, nel_1d, definition, dim=dim), actx)

"""First-order acoustic wave equation, mirroring
``actx_dgfem_suite/equations/wave.py``.

Operator (``wave.py:121-200``): weak-form DG for u_t = c div v, v_t = c grad u
with central-plus-upwind flux (``wave.py:80-114``) and the Dirichlet mirror
u_ext = -u, v_ext = v on all boundaries (``wave.py:152-156``).

Problem definitions:

* ``"reference"`` (``wave.py:239-285``): box [-0.5, 0.5]^3, c = 1,
  u = bump = exp(-|x - (0.2, 0.35, 0.1)|^2 / 0.05^2) (``wave.py:216-236`` at
  t = 0), v = 0.
* ``"baseline"``: box [-1, 1]^3, c = 1, u = exp(-|x|^2 / 0.1^2), v = 0 (the
  tiny_wave benchmark configuration; used for every performance run).

With ``dim=2`` the same definitions on the square of the box's side, with
the bump centred at (0.2, 0.35) (``wave.py:220``: the centre's first ``dim``
entries) and v = (v_x, v_y).
"""

from __future__ import annotations

import math

import numpy as np

from actx_dgfem_suite_gb300.discretization import make_box_discretization
from actx_dgfem_suite_gb300.discretization2d import make_box_discretization_2d
from actx_dgfem_suite_gb300.equations.common import Problem, make_rhs_and_args
from actx_dgfem_suite_gb300.utils import get_nel_1d_for_regular_rect_mesh
from actx_dgfem_suite_gb300.xp import array_module, r2, zeros

DEFINITIONS = ("reference", "baseline")
#: box corners of each problem definition
BOXES = {"reference": (-0.5, 0.5), "baseline": (-1.0, 1.0)}


def bump(nodes, t: float = 0.0):
    """``wave.py:216-236``: cos(3 t) exp(-|x - c|^2 / w^2).  ``nodes``: (dim, ...)
    NumPy array or torch tensor."""
    center = (0.2, 0.35, 0.1)
    width = 0.05
    omega = 3.0
    return math.cos(omega * t) * array_module(nodes).exp(-r2(nodes, center) / width**2)


def gaussian_pulse(nodes, width: float = 0.1):
    """exp(-|x|^2 / width^2), the benchmark pressure pulse."""
    return array_module(nodes).exp(-r2(nodes) / width**2)


def initial_state(nodes, definition: str):
    """(1 + dim, Nel, Np) wave state of a problem definition at the given nodes."""
    if definition == "reference":
        u = bump(nodes)
    elif definition == "baseline":
        u = gaussian_pulse(nodes)
    else:
        raise ValueError(f"unknown problem definition {definition!r}")
    fields = zeros(u, (1 + len(nodes),) + tuple(u.shape))
    fields[0] = u
    return fields


def wave_problem(order: int, nel_1d: int, definition: str = "reference",
                 c: float = 1.0, dim: int = 3) -> Problem:
    a, b = BOXES[definition]
    disc = (make_box_discretization(order, nel_1d, a, b) if dim == 3
            else make_box_discretization_2d(order, nel_1d, a, b))
    fields = initial_state(disc.nodes(), definition)
    return Problem("wave", disc, fields, (float(c),), None, definition)


def get_wave_rhs(*, actx, dim: int, order: int, ndofs: int,
                 definition: str = "reference", nel_1d: int | None = None):
    """``(rhs, (WaveState,))`` as ``actx_dgfem_suite/equations/wave.py:239-285``
    (``dim`` 3: tetrahedra, 2: triangles)."""
    if dim not in (2, 3):
        raise NotImplementedError("dim must be 2 or 3")
    if nel_1d is None:
        nel_1d = get_nel_1d_for_regular_rect_mesh(dim, order, int(ndofs))
    return make_rhs_and_args(wave_problem(order, nel_1d, definition, dim=dim), actx)

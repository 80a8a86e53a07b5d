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
"""

from __future__ import annotations

import numpy as np

from actx_dgfem_suite_gb300.discretization import make_box_discretization
from actx_dgfem_suite_gb300.equations.common import Problem, make_rhs_and_args
from actx_dgfem_suite_gb300.utils import get_nel_1d_for_regular_rect_mesh

DEFINITIONS = ("reference", "baseline")


def bump(nodes: np.ndarray, t: float = 0.0) -> np.ndarray:
    """``wave.py:216-236``: cos(3 t) exp(-|x - c|^2 / w^2)."""
    center = np.array([0.2, 0.35, 0.1])
    width = 0.05
    omega = 3.0
    d2 = sum((nodes[i] - center[i]) ** 2 for i in range(3))
    return np.cos(omega * t) * np.exp(-d2 / width**2)


def wave_problem(order: int, nel_1d: int, definition: str = "reference",
                 c: float = 1.0) -> Problem:
    if definition == "reference":
        disc = make_box_discretization(order, nel_1d, -0.5, 0.5)
        nodes = disc.nodes()
        u = bump(nodes)
    elif definition == "baseline":
        disc = make_box_discretization(order, nel_1d, -1.0, 1.0)
        nodes = disc.nodes()
        u = np.exp(-(nodes**2).sum(axis=0) / 0.1**2)
    else:
        raise ValueError(f"unknown problem definition {definition!r}")
    fields = np.zeros((4,) + u.shape)
    fields[0] = u
    return Problem("wave", disc, fields, (float(c),), None, definition)


def get_wave_rhs(*, actx, dim: int, order: int, ndofs: int,
                 definition: str = "reference", nel_1d: int | None = None):
    """``(rhs, (WaveState,))`` as ``actx_dgfem_suite/equations/wave.py:239-285``."""
    if dim != 3:
        raise NotImplementedError("only 3D tetrahedral meshes are implemented")
    if nel_1d is None:
        nel_1d = get_nel_1d_for_regular_rect_mesh(dim, order, int(ndofs))
    return make_rhs_and_args(wave_problem(order, nel_1d, definition), actx)

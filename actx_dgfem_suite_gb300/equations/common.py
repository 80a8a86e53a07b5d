"""Operator objects returned by the RHS builders.

A :class:`DGOperator` is the ``rhs`` callable of ``(rhs, args) = get_rhs(...)``
(``actx_dgfem_suite/rhs_builder.py:14-45``): calling it evaluates the RHS on the
array context it was built with, and ``actx.compile(rhs)`` binds it to a
device plan once.  :class:`Problem` is the host-side setup (mesh, geometry,
initial state) the builders produce before anything touches the GPU.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from actx_dgfem_suite_gb300.containers import (
    ConservedEulerField,
    DOFArray,
    WaveState,
    _obj_array,
)
from actx_dgfem_suite_gb300.discretization import DGDiscretization


@dataclass
class Problem:
    equation: str             # "wave" | "euler" | "maxwell"
    disc: DGDiscretization    # or discretization2d.DGDiscretization2D (triangles)
    fields: np.ndarray        # (nfields, Nel, Np) initial state, FP64
    params: tuple             # wave (c,), euler (gamma,), maxwell (alpha, eps, mu)
    t: float | None           # time argument of euler / maxwell operators
    definition: str           # "reference" | "baseline"

    @property
    def nfields(self) -> int:
        return self.fields.shape[0]

    @property
    def dim(self) -> int:
        return getattr(self.disc, "dim", 3)


def state_template(equation: str, dim: int = 3):
    """An empty container of the equation's state type (for rebuilding); on
    triangle meshes (``dim=2``) vectors have two components and Maxwell
    carries the TM fields (E_z, H_x, H_y)."""
    ph = DOFArray(None, [None])
    if equation == "wave":
        return WaveState(u=ph, v=_obj_array([ph] * dim))
    if equation == "euler":
        return ConservedEulerField(mass=ph, energy=ph,
                                   momentum=_obj_array([ph] * dim))
    if equation == "maxwell":
        return _obj_array([ph] * (6 if dim == 3 else 3))
    raise ValueError(equation)


class DGOperator:
    """The RHS callable of one equation on one discretisation."""

    def __init__(self, problem: Problem, actx):
        self.problem = problem
        self.equation = problem.equation
        self.disc = problem.disc
        self.params = problem.params
        self.state_argnum = 0 if self.equation == "wave" else 1
        #: arithmetic of the compiled plan: "fp64" or "fp32-mixed"
        self.precision = "fp64"
        self._actx = actx
        self._plans: dict[int, object] = {}
        self._compiled = None

    @property
    def dg_operator(self) -> DGOperator:
        return self

    def plan_for(self, actx):
        from actx_dgfem_suite_gb300.plan import DevicePlan
        key = (id(actx), self.precision)
        if key not in self._plans:
            self._plans[key] = DevicePlan(actx.device_mesh(self.disc),
                                          self.equation, self.params,
                                          self.precision)
        return self._plans[key]

    def __call__(self, *args):
        if self._compiled is None:
            self._compiled = self._actx.compile(self)
        return self._compiled(*args)

    def __repr__(self) -> str:
        return (f"DGOperator({self.equation}, P{self.disc.order}, "
                f"Nel={self.disc.nelements}, params={self.params})")


def make_rhs_and_args(problem: Problem, actx):
    """``(rhs, args)`` in the reference's calling convention: wave
    ``(WaveState,)``; euler ``(np.float64(t), ConservedEulerField)``; maxwell
    ``(np.float64(t), object ndarray of 6 DOFArrays)`` (3 on triangle
    meshes)."""
    from actx_dgfem_suite_gb300.array_context import stacked_state
    op = DGOperator(problem, actx)
    state = stacked_state(actx, state_template(problem.equation, problem.dim),
                          problem.fields)
    if problem.equation == "wave":
        return op, (state,)
    return op, (np.float64(problem.t), state)

"""Array containers of the suite's RHS signatures.

* :class:`DOFArray` -- stand-in for ``meshmode.dof_array.DOFArray`` with one
  element group: ``dofary[0]`` is the ``(Nel, Np)`` array.
* :class:`WaveState` -- ``actx_dgfem_suite/equations/wave.py:63-77``
  (``u``: DOFArray, ``v``: object array of ``dim`` DOFArrays).
* :class:`ConservedEulerField` -- grudge's Euler state (mass, energy,
  momentum), the argument of ``actx_dgfem_suite/equations/euler.py:176-179``.
* Maxwell's state is a plain object ndarray of 6 DOFArrays (E, H), as grudge's
  ``Vector`` (``actx_dgfem_suite/equations/maxwell.py:69-74``).

All support elementwise arithmetic with scalars and containers of the same
structure (``with_container_arithmetic`` in the reference).  Leaves are torch
tensors on a device or numpy arrays after ``to_numpy``.
"""

from __future__ import annotations

import operator
from dataclasses import dataclass
from typing import Any, Callable

import numpy as np


class _Arith:
    """Elementwise arithmetic through ``_map2``."""

    def _map2(self, other, op):  # pragma: no cover - abstract
        raise NotImplementedError

    def __add__(self, o):
        return self._map2(o, operator.add)

    def __radd__(self, o):
        return self._map2(o, lambda a, b: b + a)

    def __sub__(self, o):
        return self._map2(o, operator.sub)

    def __rsub__(self, o):
        return self._map2(o, lambda a, b: b - a)

    def __mul__(self, o):
        return self._map2(o, operator.mul)

    def __rmul__(self, o):
        return self._map2(o, lambda a, b: b * a)

    def __truediv__(self, o):
        return self._map2(o, operator.truediv)

    def __rtruediv__(self, o):
        return self._map2(o, lambda a, b: b / a)

    def __neg__(self):
        return self._map2(-1.0, operator.mul)

    def __pow__(self, o):
        return self._map2(o, operator.pow)


class DOFArray(_Arith):
    __array_ufunc__ = None

    def __init__(self, actx, data, *, stack=None):
        self.array_context = actx
        self._data = tuple(data)
        # (stacked tensor, field index) when this array is a view of a
        # (nfields, Nel, Np) buffer; lets a compiled RHS skip staging copies.
        self._stack = stack

    def __len__(self):
        return len(self._data)

    def __getitem__(self, i):
        return self._data[i]

    def __iter__(self):
        return iter(self._data)

    @property
    def shape(self):
        return self._data[0].shape

    def _map2(self, other, op):
        if isinstance(other, DOFArray):
            return DOFArray(self.array_context,
                            [op(a, b) for a, b in zip(self._data, other._data)])
        if isinstance(other, (_Arith, np.ndarray)) and not np.isscalar(other):
            return NotImplemented
        return DOFArray(self.array_context, [op(a, other) for a in self._data])

    def map(self, f: Callable[[Any], Any], actx="same") -> DOFArray:
        return DOFArray(self.array_context if actx == "same" else actx,
                        [f(a) for a in self._data])

    def __repr__(self):
        return f"DOFArray(ngroups={len(self._data)}, shape={self.shape})"


def _obj_array(items) -> np.ndarray:
    out = np.empty(len(items), dtype=object)
    for k, it in enumerate(items):
        out[k] = it
    return out


def _map_obj(a: np.ndarray, b, op) -> np.ndarray:
    if isinstance(b, np.ndarray) and b.dtype == object:
        return _obj_array([op(x, y) for x, y in zip(a, b)])
    return _obj_array([op(x, b) for x in a])


@dataclass(frozen=True)
class WaveState(_Arith):
    u: DOFArray
    v: np.ndarray  # object array of DOFArrays

    __array_ufunc__ = None

    def __post_init__(self):
        assert isinstance(self.v, np.ndarray) and self.v.dtype.char == "O"

    def _map2(self, o, op):
        if isinstance(o, WaveState):
            return WaveState(u=op(self.u, o.u), v=_map_obj(self.v, o.v, op))
        return WaveState(u=op(self.u, o), v=_map_obj(self.v, o, op))


@dataclass(frozen=True)
class ConservedEulerField(_Arith):
    mass: DOFArray
    energy: DOFArray
    momentum: np.ndarray  # object array of DOFArrays

    __array_ufunc__ = None

    def _map2(self, o, op):
        if isinstance(o, ConservedEulerField):
            return ConservedEulerField(mass=op(self.mass, o.mass),
                                       energy=op(self.energy, o.energy),
                                       momentum=_map_obj(self.momentum, o.momentum, op))
        return ConservedEulerField(mass=op(self.mass, o), energy=op(self.energy, o),
                                   momentum=_map_obj(self.momentum, o, op))


# {{{ flatten / rebuild in the C ABI's field order


def leaves(state) -> list[DOFArray]:
    """DOFArrays of a state in field order (wave: u, v; euler: mass,
    energy, momentum; maxwell: E, H)."""
    if isinstance(state, WaveState):
        return [state.u, *state.v]
    if isinstance(state, ConservedEulerField):
        return [state.mass, state.energy, *state.momentum]
    if isinstance(state, np.ndarray) and state.dtype == object:
        return list(state)
    raise TypeError(f"unsupported state container {type(state).__name__}")


def rebuild(template, new_leaves: list[DOFArray]):
    """A container shaped like ``template`` holding ``new_leaves``."""
    if isinstance(template, WaveState):
        return WaveState(u=new_leaves[0], v=_obj_array(new_leaves[1:]))
    if isinstance(template, ConservedEulerField):
        return ConservedEulerField(mass=new_leaves[0], energy=new_leaves[1],
                                   momentum=_obj_array(new_leaves[2:]))
    if isinstance(template, np.ndarray) and template.dtype == object:
        return _obj_array(new_leaves)
    raise TypeError(f"unsupported state container {type(template).__name__}")


def map_leaves(state, f: Callable[[DOFArray], DOFArray]):
    if isinstance(state, DOFArray):
        return f(state)
    if isinstance(state, (WaveState, ConservedEulerField)) or (
            isinstance(state, np.ndarray) and state.dtype == object):
        return rebuild(state, [map_leaves(x, f) for x in leaves(state)])
    return state


def from_stacked(actx, template, stacked) -> Any:
    """Container of DOFArray views into ``stacked`` (nfields, Nel, Np)."""
    return rebuild(template, [DOFArray(actx, [stacked[k]], stack=(stacked, k))
                              for k in range(stacked.shape[0])])


# }}}

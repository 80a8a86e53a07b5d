"""Containers and builders' host-side setup (CPU)."""

import numpy as np
import pytest

from actx_dgfem_suite_gb300.containers import (ConservedEulerField, DOFArray,
                                               WaveState, _obj_array, leaves,
                                               rebuild)
from actx_dgfem_suite_gb300.rhs_builder import get_problem, split_equation_name


def _d(x):
    return DOFArray(None, [np.asarray(x, dtype=float)])


def test_wavestate_arithmetic_and_leaves():
    w = WaveState(u=_d([1.0, 2.0]), v=_obj_array([_d([1.0]), _d([2.0]), _d([3.0])]))
    w2 = 2 * w + w - 1.0
    assert np.allclose(w2.u[0], [2.0, 5.0])
    assert np.allclose(w2.v[2][0], [8.0])
    lv = leaves(w2)
    assert len(lv) == 4
    back = rebuild(w, lv)
    assert isinstance(back, WaveState)


def test_euler_field_order():
    q = ConservedEulerField(mass=_d([1.0]), energy=_d([2.0]),
                            momentum=_obj_array([_d([3.0]), _d([4.0]), _d([5.0])]))
    assert [float(d[0][0]) for d in leaves(q)] == [1, 2, 3, 4, 5]
    assert np.allclose((q / 2).momentum[1][0], [2.0])


def test_split_names():
    assert split_equation_name("tiny_wave") == ("wave", 1_000)
    assert split_equation_name("large_euler") == ("euler", 20_000_000)
    assert split_equation_name("maxwell") == ("maxwell", 4_000_000)


@pytest.mark.parametrize("eq,nf", [("wave", 4), ("euler", 5), ("maxwell", 6)])
@pytest.mark.parametrize("definition", ["reference", "baseline"])
def test_problem_setup(eq, nf, definition):
    p = get_problem("tiny_" + eq, 3, 2, definition=definition)
    assert p.fields.shape == (nf, p.disc.nelements, 10)
    assert np.isfinite(p.fields).all()
    if eq == "euler":
        assert (p.fields[0] > 0).all()


def test_reference_initial_conditions():
    p = get_problem("tiny_euler", 3, 1)
    assert np.all(p.fields[0] == 1.0)                  # rho = 1
    assert np.all(p.fields[2:] == 0.0)                 # at rest
    assert np.isclose(p.fields[1].min(), 2.5, atol=1e-3)
    m = get_problem("tiny_maxwell", 3, 3)
    assert np.all(m.fields[3:] == 0.0)                 # real part of H is 0
    assert m.params == (0.5, 1.0, 1.0)
    w = get_problem("tiny_wave", 3, 2)
    assert np.all(w.fields[1:] == 0.0) and w.params == (1.0,)


def test_unsupported_dims_and_equations():
    assert get_problem("tiny_wave", 2, 1).dim == 2      # triangles
    with pytest.raises(NotImplementedError):
        get_problem("tiny_wave", 1, 1)
    with pytest.raises(NotImplementedError):
        get_problem("tiny_burgers", 3, 1)

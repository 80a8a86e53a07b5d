"""The package, the oracle and the product against the reference's own
equation code (``tests/golden/reference_equations.npz``, written by
``tests/golden/make_reference_equations.py``, which runs
``actx_dgfem_suite/equations/{wave,euler}.py`` on stand-in modules over the
oracle's grudge primitives):

* the initial states of the reference's wave and Euler definitions;
* ``wave_operator`` (``wave.py:121-200``) of a random state on a jittered
  mesh at orders 1-4: the oracle's restatement on the CPU, and the product
  through the C ABI on a GPU."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from tests._helpers import FP64_RTOL

GOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "reference_equations.npz")


def test_initial_states_match_the_reference_code():
    """Equal to the last bit where written (x86-64); NumPy's exp may differ
    by an ulp between platforms."""
    from actx_dgfem_suite_gb300.equations import euler, wave
    nodes = GOLDEN["ic_nodes"]
    np.testing.assert_allclose(wave.bump(nodes), GOLDEN["ic_wave_u"], rtol=1e-15, atol=1e-300)
    np.testing.assert_allclose(euler.acoustic_pulse_condition(nodes), GOLDEN["ic_euler"],
                               rtol=1e-15, atol=1e-300)


def test_initial_state_nodes_are_the_package_nodes():
    """The recorded nodes are where the package puts its nodes on that mesh."""
    from actx_dgfem_suite_gb300.discretization import make_discretization
    from actx_dgfem_suite_gb300.mesh import TetMesh
    disc = make_discretization(TetMesh(GOLDEN["ic_vertices"], GOLDEN["ic_elements"]), 3)
    assert np.abs(disc.nodes() - GOLDEN["ic_nodes"]).max() <= 1e-14


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_oracle_wave_operator_matches_the_reference_code(order):
    from oracle.geometry import build_oracle_disc
    from oracle.rhs import wave_rhs
    d = build_oracle_disc(GOLDEN["wave_vertices"], GOLDEN["wave_elements"], order)
    st = GOLDEN[f"wave_P{order}_state"]
    ru, rv = wave_rhs(d, st[0], st[1:])
    got = np.concatenate([ru[None], rv])
    ref = GOLDEN[f"wave_P{order}_rhs"]
    assert np.linalg.norm(got - ref) <= 1e-14 * np.linalg.norm(ref)


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("precision", ["fp64", "fp64-tc"])
def test_product_wave_operator_matches_the_reference_code(order, precision):
    import torch

    from actx_dgfem_suite_gb300.mesh import TetMesh
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    from tests._helpers import make_problem
    st = GOLDEN[f"wave_P{order}_state"]
    prob = make_problem("wave", TetMesh(GOLDEN["wave_vertices"], GOLDEN["wave_elements"]),
                        order, fields=st)
    plan = DevicePlan(DeviceMesh(prob.disc, "cuda:0"), "wave", (1.0,), precision)
    got = plan.rhs(torch.from_numpy(st).cuda()).cpu().numpy()
    plan.finish()
    ref = GOLDEN[f"wave_P{order}_rhs"]
    assert np.linalg.norm(got - ref) <= FP64_RTOL * np.linalg.norm(ref)


# {{{ triangle meshes (tests/golden/reference_equations_2d.npz, from the
# same run of the reference's wave.py with dim = 2)

GOLDEN_2D = np.load(Path(__file__).resolve().parent / "golden" / "reference_equations_2d.npz")


def test_2d_initial_state_matches_the_reference_code():
    from actx_dgfem_suite_gb300.discretization2d import make_discretization_2d
    from actx_dgfem_suite_gb300.equations import wave
    from actx_dgfem_suite_gb300.mesh import TriMesh
    from actx_dgfem_suite_gb300.equations import euler
    nodes = GOLDEN_2D["ic_nodes"]
    np.testing.assert_allclose(wave.bump(nodes), GOLDEN_2D["ic_wave_u"], rtol=1e-15,
                               atol=1e-300)
    np.testing.assert_allclose(euler.acoustic_pulse_condition(nodes), GOLDEN_2D["ic_euler"],
                               rtol=1e-15, atol=1e-300)
    disc = make_discretization_2d(TriMesh(GOLDEN_2D["ic_vertices"],
                                          GOLDEN_2D["ic_elements"]), 3)
    assert np.abs(disc.nodes() - nodes).max() <= 1e-14


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_oracle_2d_wave_operator_matches_the_reference_code(order):
    from oracle.geometry import build_oracle_disc_2d
    from oracle.rhs import wave_rhs
    d = build_oracle_disc_2d(GOLDEN_2D["wave_vertices"], GOLDEN_2D["wave_elements"], order)
    st = GOLDEN_2D[f"wave_P{order}_state"]
    ru, rv = wave_rhs(d, st[0], st[1:])
    got = np.concatenate([ru[None], rv])
    ref = GOLDEN_2D[f"wave_P{order}_rhs"]
    assert np.linalg.norm(got - ref) <= 1e-14 * np.linalg.norm(ref)


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_product_2d_wave_operator_matches_the_reference_code(order):
    import torch

    from actx_dgfem_suite_gb300.mesh import TriMesh
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    from tests._helpers import make_problem_2d
    st = GOLDEN_2D[f"wave_P{order}_state"]
    prob = make_problem_2d("wave", TriMesh(GOLDEN_2D["wave_vertices"],
                                           GOLDEN_2D["wave_elements"]), order, fields=st)
    plan = DevicePlan(DeviceMesh(prob.disc, "cuda:0"), "wave", (1.0,), "fp64")
    got = plan.rhs(torch.from_numpy(st).cuda()).cpu().numpy()
    plan.finish()
    ref = GOLDEN_2D[f"wave_P{order}_rhs"]
    assert np.linalg.norm(got - ref) <= FP64_RTOL * np.linalg.norm(ref)

# }}}

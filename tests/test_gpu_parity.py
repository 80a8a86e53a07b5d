"""FP64 parity of the CUDA RHS kernels against the CPU oracle, through the
C ABI (DevicePlan -> dg_rhs).  Bound: relative L2 <= 1e-12."""

from __future__ import annotations

import numpy as np
import pytest

from tests._helpers import (FP64_RTOL, jittered_box_mesh, make_problem, oracle_rhs,
                           parity_error, single_tet_mesh)
from actx_dgfem_suite_gb300.mesh import generate_box_tet_mesh
from actx_dgfem_suite_gb300.rhs_builder import get_problem

pytestmark = pytest.mark.gpu

EQUATIONS = ("wave", "euler", "maxwell")
ORDERS = (1, 2, 3, 4)


def _gpu_rhs(problem):
    import torch

    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    dm = DeviceMesh(problem.disc, "cuda:0")
    plan = DevicePlan(dm, problem.equation, problem.params)
    q = torch.from_numpy(problem.fields).to("cuda:0")
    out = plan.rhs(q)
    plan.finish()
    return out.cpu().numpy(), plan


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("definition", ("reference", "baseline"))
def test_parity_box(equation, order, definition):
    prob = get_problem(equation, 3, order, definition=definition, nel_1d=3)
    got, _ = _gpu_rhs(prob)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", ORDERS)
def test_parity_jittered_mesh(equation, order):
    prob = make_problem(equation, jittered_box_mesh(4), order, seed=order)
    got, _ = _gpu_rhs(prob)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", ORDERS)
def test_parity_single_element(equation, order):
    prob = make_problem(equation, single_tet_mesh(), order)
    got, _ = _gpu_rhs(prob)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
def test_parity_single_hex(equation):
    prob = make_problem(equation, generate_box_tet_mesh(0.0, 1.0, 1), 3)
    got, _ = _gpu_rhs(prob)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
def test_parity_anisotropic_box(equation):
    """n = (5, 2, 3) hexahedra per axis: a tile tail and uneven neighbours."""
    prob = make_problem(equation, generate_box_tet_mesh((0, 0, 0), (2.0, 0.5, 1.0),
                                                        (5, 2, 3)), 2, seed=3)
    got, _ = _gpu_rhs(prob)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


def test_deterministic_bitwise():
    prob = make_problem("euler", jittered_box_mesh(4), 3)
    a, plan = _gpu_rhs(prob)
    b, _ = _gpu_rhs(prob)
    assert np.array_equal(a, b)

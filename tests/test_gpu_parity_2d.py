"""Triangle meshes on the GPU: FP64 parity of dg_rhs2d_kernel (through
dg_plan_create_2d and the C ABI) with the CPU oracle's independent 2D
restatement.  Bound: relative L2 <= 1e-12, as in 3D."""

from __future__ import annotations

import numpy as np
import pytest

from actx_dgfem_suite_gb300.rhs_builder import get_problem
from tests._helpers import (
    FP64_RTOL,
    jittered_square_mesh,
    make_problem_2d,
    oracle_rhs,
    parity_error,
)

pytestmark = pytest.mark.gpu

EQUATIONS = ("wave", "euler", "maxwell")
ORDERS = (1, 2, 3, 4)


def _plan(problem):
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    dm = DeviceMesh(problem.disc, "cuda:0")
    plan = DevicePlan(dm, problem.equation, problem.params, "fp64")
    assert plan.dim == 2 and plan.shape == problem.fields.shape
    return plan


def _gpu_rhs(problem):
    import torch
    plan = _plan(problem)
    info = plan.info()
    assert not info["face_shared"] and not info["tensor_cores"]
    assert info["launches_per_rhs"] == 1
    q = torch.from_numpy(problem.fields).to("cuda:0")
    out = plan.rhs(q)
    plan.finish()
    return out.cpu().numpy()


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", ORDERS)
def test_parity_2d_jittered(equation, order):
    prob = make_problem_2d(equation, jittered_square_mesh(6, seed=order), order,
                           seed=order)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(_gpu_rhs(prob), ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("definition", ("reference", "baseline"))
def test_parity_2d_box(equation, order, definition):
    prob = get_problem(equation, 2, order, definition=definition, nel_1d=5)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(_gpu_rhs(prob), ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
def test_tiny_2d_through_the_array_context(equation):
    """The suite's calling convention with dim = 2: get_rhs("tiny_*", actx, 2,
    N), actx.compile(rhs)(*args), actx.to_numpy (run/__main__.py:73-96)."""
    from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext
    from actx_dgfem_suite_gb300.containers import leaves
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs
    actx = GB300DGArrayContext("cuda:0")
    for order in (1, 2, 3, 4):
        rhs, args = get_rhs("tiny_" + equation, actx, 2, order)
        out = actx.to_numpy(actx.compile(rhs)(*args))
        got = np.stack([np.asarray(d[0]) for d in leaves(out)])
        prob = rhs.dg_operator.problem
        ref, scale = oracle_rhs(prob, parts=True)
        assert got.shape == prob.fields.shape
        assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
def test_rk_stage_2d_with_element_scale(equation):
    import torch
    prob = make_problem_2d(equation, jittered_square_mesh(5), 3, seed=3)
    plan = _plan(prob)
    q = torch.from_numpy(prob.fields).to("cuda:0")
    nel = prob.disc.nelements
    scale = torch.linspace(0.8, 1.2, nel, dtype=torch.float64, device="cuda:0")
    res0 = torch.rand(q.shape, dtype=q.dtype, device=q.device,
                      generator=torch.Generator(device=q.device).manual_seed(5))
    plan.set_element_scale(scale)
    res = res0.clone()
    qo = torch.empty_like(q)
    unscaled = torch.empty_like(q)
    a, b, dt = 0.3, 0.5, 1e-3
    plan.rk_stage(q, qo, res, a, b, dt, rhs_unscaled=unscaled)
    plan.finish()
    lq = torch.from_numpy(oracle_rhs(prob)).to("cuda:0")
    ref_res = a * res0 + dt * scale[None, :, None] * lq
    n = float(torch.linalg.norm(lq))
    assert float(torch.linalg.norm(unscaled - lq)) <= FP64_RTOL * n
    assert float(torch.linalg.norm(res - ref_res)) <= FP64_RTOL * float(torch.linalg.norm(ref_res))
    assert float(torch.linalg.norm(qo - (q + b * ref_res))) <= 1e-14 * float(torch.linalg.norm(q))


def test_2d_plans_have_one_variant():
    import torch

    from actx_dgfem_suite_gb300._lib import DGError
    prob = make_problem_2d("wave", jittered_square_mesh(3), 2)
    plan = _plan(prob)
    plan.set_variant(0)
    with pytest.raises(DGError):
        plan.set_variant(1)
    with pytest.raises(DGError):
        plan.autotune(torch.from_numpy(prob.fields).to("cuda:0"), reps=1)
    from actx_dgfem_suite_gb300.plan import DevicePlan
    with pytest.raises(ValueError):
        DevicePlan(plan.mesh, "wave", prob.params, "fp32-mixed")

"""Fused RK stages and the mixed-precision path on the GPU."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from tests._helpers import (FP64_RTOL, jittered_box_mesh, make_problem,
                            oracle_rhs, rel_l2)

pytestmark = pytest.mark.gpu

#: relative L2 bound for the mixed-precision RHS against FP64
MIXED_RTOL = 1e-5


def _plan(prob, precision="fp64"):
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    return DevicePlan(DeviceMesh(prob.disc, "cuda:0"), prob.equation, prob.params,
                      precision)


def _oracle_rhs_fn(prob):
    from oracle.geometry import build_oracle_disc
    d = prob.disc
    od = build_oracle_disc(d.mesh.vertices, d.mesh.elements, d.order)
    import copy

    def f(q):
        p2 = copy.copy(prob)
        p2.fields = q
        return oracle_rhs(p2, od)
    return f


@pytest.mark.parametrize("equation", ["wave", "euler", "maxwell"])
def test_rk_stage_matches_oracle_lsrk45(equation):
    from actx_dgfem_suite_gb300.timestepping import LSRK45, estimate_rk4_timestep
    from oracle.timestep import lsrk45_step
    prob = make_problem(equation, jittered_box_mesh(3), 3, seed=5)
    plan = _plan(prob)
    dt = 0.3 * estimate_rk4_timestep(prob.disc, 2.0)
    q = torch.from_numpy(prob.fields.copy()).to("cuda:0")
    LSRK45(plan, dt).run(q, 3)
    plan.finish()
    ref = prob.fields
    f = _oracle_rhs_fn(prob)
    for _ in range(3):
        ref = lsrk45_step(f, ref, dt)
    got = q.cpu().numpy()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= FP64_RTOL


def test_rk_stage_first_stage_ignores_residual_contents():
    prob = make_problem("wave", jittered_box_mesh(2), 2)
    plan = _plan(prob)
    q = torch.from_numpy(prob.fields).to("cuda:0")
    out1 = torch.empty_like(q)
    out2 = torch.empty_like(q)
    res1 = torch.full_like(q, float("nan"))
    res2 = torch.zeros_like(q)
    plan.rk_stage(q, out1, res1, 0.0, 0.5, 1e-3)
    plan.rk_stage(q, out2, res2, 0.0, 0.5, 1e-3)
    plan.finish()
    assert torch.equal(out1, out2) and torch.equal(res1, res2)
    rhs = plan.rhs(q)
    plan.finish()
    assert torch.allclose(res2, 1e-3 * rhs, rtol=1e-14, atol=0)


def test_graph_replay_matches_eager():
    from actx_dgfem_suite_gb300.timestepping import LSRK45
    prob = make_problem("maxwell", jittered_box_mesh(3), 2, seed=2)
    plan = _plan(prob)
    q1 = torch.from_numpy(prob.fields.copy()).to("cuda:0")
    q2 = q1.clone()
    LSRK45(plan, 1e-3).run(q1, 4)
    LSRK45(plan, 1e-3, use_graph=True).run(q2, 4)
    plan.finish()
    assert torch.equal(q1, q2)


@pytest.mark.parametrize("equation", ["wave", "euler", "maxwell"])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_mixed_precision_rhs_error(equation, order):
    prob = make_problem(equation, jittered_box_mesh(3), order, seed=order)
    q = torch.from_numpy(prob.fields).to("cuda:0")
    r64 = _plan(prob, "fp64").rhs(q).cpu().numpy()
    r32 = _plan(prob, "fp32-mixed").rhs(q).cpu().numpy()
    ref, scale = oracle_rhs(prob, parts=True)
    err = np.linalg.norm(r32 - r64) / max(np.linalg.norm(r64), 1e-300)
    assert err <= MIXED_RTOL, err
    assert err > 1e-10  # really computed in FP32
    assert np.linalg.norm(r64 - ref) / max(np.linalg.norm(ref), scale) <= FP64_RTOL


def test_mixed_precision_euler_rk_trajectory():
    """Euler P3: FP32-arithmetic RK stays within 1e-5 of the FP64 run."""
    from actx_dgfem_suite_gb300.rhs_builder import get_problem
    from actx_dgfem_suite_gb300.timestepping import LSRK45, estimate_rk4_timestep
    prob = get_problem("euler", 3, 3, definition="baseline", nel_1d=6)
    dt = 0.5 * estimate_rk4_timestep(prob.disc, 2.0)
    q64 = torch.from_numpy(prob.fields.copy()).to("cuda:0")
    q32 = q64.clone()
    i64 = LSRK45(_plan(prob, "fp64"), dt)
    i32 = LSRK45(_plan(prob, "fp32-mixed"), dt)
    errs = []
    for _ in range(20):
        i64.step(q64)
        i32.step(q32)
        errs.append(float(torch.linalg.norm(q32 - q64) / torch.linalg.norm(q64)))
    assert max(errs) <= MIXED_RTOL, errs

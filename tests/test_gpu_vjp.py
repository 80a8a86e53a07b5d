"""Transposed Jacobian of the RHS (dg_rhs_vjp) against finite differences of
the forward RHS: <x, (L(q + e v) - L(q - e v)) / 2e> = <L'(q)^T x, v>."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from tests._helpers import jittered_box_mesh, make_problem

pytestmark = pytest.mark.gpu


def _plan(equation, order, seed=0):
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    prob = make_problem(equation, jittered_box_mesh(3), order, seed=seed)
    plan = DevicePlan(DeviceMesh(prob.disc, "cuda:0", with_partner=True), equation,
                      prob.params)
    return prob, plan


def _euler_state(shape, rng):
    q = np.empty(shape)
    q[0] = 1.0 + 0.2 * rng.random(shape[1:])                 # rho
    q[2:] = 0.3 * rng.standard_normal((3,) + shape[1:])      # momentum
    ke = 0.5 * (q[2:] ** 2).sum(axis=0) / q[0]
    q[1] = 2.5 + 0.3 * rng.random(shape[1:]) + ke            # energy, p ~ 1
    return q


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_euler_vjp_matches_finite_differences(order):
    prob, plan = _plan("euler", order, seed=order)
    rng = np.random.default_rng(order)
    q = torch.from_numpy(_euler_state(prob.fields.shape, rng)).cuda()
    x = torch.from_numpy(rng.standard_normal(prob.fields.shape)).cuda()
    v = torch.from_numpy(rng.standard_normal(prob.fields.shape)).cuda()
    y = plan.vjp(q, x)
    eps = 1e-6
    dl = (plan.rhs(q + eps * v) - plan.rhs(q - eps * v)) / (2 * eps)
    plan.finish()
    lhs, rhs = float((x * dl).sum()), float((y * v).sum())
    assert abs(lhs - rhs) <= 1e-6 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_euler_vjp_per_component_and_scale():
    """Directional checks along single fields, and with a per-element scale."""
    prob, plan = _plan("euler", 2, seed=9)
    rng = np.random.default_rng(3)
    q = torch.from_numpy(_euler_state(prob.fields.shape, rng)).cuda()
    scale = torch.from_numpy(rng.uniform(0.5, 1.5, prob.disc.nelements)).cuda()
    plan.set_element_scale(scale)
    x = torch.from_numpy(rng.standard_normal(prob.fields.shape)).cuda()
    y = plan.vjp(q, x)
    eps = 1e-6
    for k in range(5):
        v = torch.zeros_like(q)
        v[k] = torch.from_numpy(rng.standard_normal(prob.fields.shape[1:])).cuda()
        dl = (plan.rhs(q + eps * v) - plan.rhs(q - eps * v)) / (2 * eps)
        lhs, rhs = float((x * dl).sum()), float((y * v).sum())
        assert abs(lhs - rhs) <= 1e-6 * max(abs(lhs), abs(rhs)), (k, lhs, rhs)
    plan.finish()


def test_wave_vjp_is_the_adjoint():
    prob, plan = _plan("wave", 3)
    rng = np.random.default_rng(0)
    q = torch.from_numpy(rng.standard_normal(prob.fields.shape)).cuda()
    x = torch.from_numpy(rng.standard_normal(prob.fields.shape)).cuda()
    a = plan.vjp(q, x)
    b = plan.adjoint(x)
    plan.finish()
    assert float(torch.linalg.norm(a - b)) <= 1e-14 * float(torch.linalg.norm(b))


def test_rhs_function_autograd():
    from actx_dgfem_suite_gb300.adjoint import RHSFunction
    prob, plan = _plan("euler", 3, seed=2)
    rng = np.random.default_rng(5)
    q = torch.from_numpy(_euler_state(prob.fields.shape, rng)).cuda().requires_grad_(True)
    w = torch.from_numpy(rng.standard_normal(prob.fields.shape)).cuda()
    loss = (RHSFunction.apply(q, plan) * w).sum()
    loss.backward()
    ref = plan.vjp(q.detach(), w)
    plan.finish()
    assert torch.equal(q.grad, ref)


def test_vjp_unsupported_without_partners():
    from actx_dgfem_suite_gb300._lib import DGError
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    prob = make_problem("euler", jittered_box_mesh(2), 2)
    plan = DevicePlan(DeviceMesh(prob.disc, "cuda:0", with_partner=False), "euler",
                      prob.params)
    q = torch.from_numpy(prob.fields).cuda()
    with pytest.raises(DGError):
        plan.vjp(q, q.clone())


def test_euler_misfit_gradient_matches_finite_differences():
    """Gradient of a density-receiver misfit through 8 LSRK45 steps of the
    Euler operator with respect to the initial state."""
    from actx_dgfem_suite_gb300.adjoint import (EulerAdjointSolver, EulerMisfitFunction,
                                                Receivers, random_interior_points)
    from actx_dgfem_suite_gb300.equations.euler import euler_problem
    from actx_dgfem_suite_gb300.timestepping import estimate_rk4_timestep
    prob = euler_problem(2, 3, "baseline")
    d = prob.disc
    pts = random_interior_points(10, (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), 0.05, seed=4)
    rec = Receivers(d, pts, "cuda:0")
    dt = 0.5 * estimate_rk4_timestep(d, 1.3)
    solver = EulerAdjointSolver(d, prob.params[0], dt, 8, rec, "cuda:0", segment=3)
    q0 = torch.from_numpy(prob.fields).cuda()
    rng = np.random.default_rng(2)
    obs = EulerMisfitFunction.apply(q0 * (1 + 0.01 * torch.from_numpy(
        rng.standard_normal(q0.shape)).cuda()), solver).detach()

    def loss(qq):
        return 0.5 * torch.sum((EulerMisfitFunction.apply(qq, solver) - obs) ** 2)

    qv = q0.clone().requires_grad_(True)
    loss(qv).backward()
    dq = torch.from_numpy(rng.standard_normal(tuple(q0.shape))).cuda()
    eps = 1e-6
    with torch.no_grad():
        fd = (float(loss(q0 + eps * dq)) - float(loss(q0 - eps * dq))) / (2 * eps)
    an = float(torch.sum(qv.grad * dq))
    assert abs(an - fd) <= 1e-5 * abs(fd), (an, fd)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("alias", ["none", "x_is_lam", "rbar_in_place"])
def test_fused_vjp_stage_matches_composition(order, alias):
    """dg_rhs_vjp_stage == the same reverse stage composed from dg_rhs_vjp and
    elementwise operations: lam += dt L'(q)^T rbar, rbar_out = a rbar + b lam,
    with a per-element scale and the aliasing the reverse sweep uses (x = lam
    on its first stage, rbar updated in place)."""
    prob, plan = _plan("euler", order, seed=20 + order)
    rng = np.random.default_rng(40 + order)
    shape = prob.fields.shape
    q = torch.from_numpy(_euler_state(shape, rng)).cuda()
    plan.set_element_scale(torch.from_numpy(rng.uniform(0.5, 1.5, shape[1])).cuda())
    lam = torch.from_numpy(rng.standard_normal(shape)).cuda()
    x = lam.clone() if alias == "x_is_lam" else torch.from_numpy(
        rng.standard_normal(shape)).cuda()
    xscale, a, b, dt = (0.7, -0.4, 0.3, 1e-2)
    rb = xscale * x
    lam_ref = lam + dt * plan.vjp(q, rb)
    rbar_ref = a * rb + b * lam_ref
    ysc = torch.empty_like(x)
    if alias == "x_is_lam":
        xin, out = lam, torch.empty_like(x)
    elif alias == "rbar_in_place":
        xin = out = x
    else:
        xin, out = x, torch.empty_like(x)
    plan.vjp_stage(q, xin, xscale, lam, out, a, b, dt, ysc)
    plan.finish()
    for got, ref in ((lam, lam_ref), (out, rbar_ref)):
        err = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
        assert err <= 1e-14, err


def test_vjp_stage_wave_plan_and_overlap_errors():
    """On a wave plan dg_rhs_vjp_stage is dg_rhs_adjoint_stage without the
    element-scale gradient; overlapping q or scratch arrays are refused."""
    from actx_dgfem_suite_gb300._lib import DGError
    prob, plan = _plan("wave", 2)
    rng = np.random.default_rng(1)
    shape = prob.fields.shape
    lam = torch.from_numpy(rng.standard_normal(shape)).cuda()
    x = torch.from_numpy(rng.standard_normal(shape)).cuda()
    lam2 = lam.clone()
    out1, out2, ysc = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    plan.vjp_stage(x, x, 0.5, lam, out1, 0.2, 0.3, 1e-2, ysc)
    plan.adjoint_stage(x, 0.5, lam2, out2, None, None, 0.2, 0.3, 1e-2, ysc)
    plan.finish()
    assert torch.equal(lam, lam2) and torch.equal(out1, out2)
    eprob, eplan = _plan("euler", 2)
    eshape = eprob.fields.shape
    q = torch.from_numpy(_euler_state(eshape, rng)).cuda()
    ex = torch.from_numpy(rng.standard_normal(eshape)).cuda()
    elam, eysc = torch.zeros_like(ex), torch.empty_like(ex)
    with pytest.raises(DGError):
        eplan.vjp_stage(q, ex, 1.0, q, None, 0.2, 0.3, 1e-2, eysc)      # lam is q
    with pytest.raises(DGError):
        eplan.vjp_stage(q, ex, 1.0, elam, None, 0.2, 0.3, 1e-2, elam)   # scratch is lam

"""Hand-written adjoint of the wave RHS and the misfit gradient."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from tests._helpers import jittered_box_mesh, make_problem

pytestmark = pytest.mark.gpu


def _plan(disc, c=1.0):
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    return DevicePlan(DeviceMesh(disc, "cuda:0", with_partner=True), "wave", (c,))


@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("scaled", [False, True])
def test_dot_product(order, scaled):
    """<L x, y> = <x, L^T y> to round-off (with and without c_e)."""
    prob = make_problem("wave", jittered_box_mesh(3), order)
    plan = _plan(prob.disc, 1.3)
    g = torch.Generator(device="cuda:0").manual_seed(order)
    shape = plan.shape
    x = torch.randn(shape, dtype=torch.float64, device="cuda:0", generator=g)
    y = torch.randn(shape, dtype=torch.float64, device="cuda:0", generator=g)
    if scaled:
        c = 0.8 + 0.4 * torch.rand(shape[1], dtype=torch.float64, device="cuda:0",
                                   generator=g)
        plan.set_element_scale(c)
    lx = plan.rhs(x)
    lty = plan.adjoint(y)
    plan.finish()
    a = float(torch.sum(lx * y))
    b = float(torch.sum(x * lty))
    scale = float(torch.linalg.norm(lx) * torch.linalg.norm(y))
    assert abs(a - b) <= 1e-13 * scale, (a, b)


def test_adjoint_matches_oracle_matrix():
    """L^T y equals the transpose of the oracle's operator, assembled column
    by column from the CPU oracle (P1, 6 * 2^3 tets)."""
    from tests._helpers import oracle_rhs
    from oracle.geometry import build_oracle_disc
    import copy
    prob = make_problem("wave", jittered_box_mesh(2), 1)
    d = prob.disc
    od = build_oracle_disc(d.mesh.vertices, d.mesh.elements, 1)
    n = prob.fields.size
    cols = []
    p2 = copy.copy(prob)
    for k in range(n):
        e = np.zeros(n)
        e[k] = 1.0
        p2.fields = e.reshape(prob.fields.shape)
        cols.append(oracle_rhs(p2, od).reshape(-1))
    A = np.stack(cols, axis=1)
    y = np.random.default_rng(0).standard_normal(n)
    ref = A.T @ y
    plan = _plan(d)
    got = plan.adjoint(torch.from_numpy(y.reshape(prob.fields.shape)).cuda())
    plan.finish()
    got = got.cpu().numpy().reshape(-1)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-12


def _small_solver(nsteps=12, order=2, checkpointing="binomial", slots=None):
    from actx_dgfem_suite_gb300.adjoint import (Receivers, WaveAdjointSolver,
                                                random_interior_points)
    from actx_dgfem_suite_gb300.equations.wave import wave_problem
    from actx_dgfem_suite_gb300.timestepping import estimate_rk4_timestep
    prob = wave_problem(order, 3, "baseline")
    d = prob.disc
    pts = random_interior_points(8, (-1, -1, -1), (1, 1, 1), 0.1, seed=4)
    rec = Receivers(d, pts, "cuda:0")
    dt = 0.5 * estimate_rk4_timestep(d, 1.2)
    solver = WaveAdjointSolver(d, dt, nsteps, rec, "cuda:0", segment=5,
                               checkpointing=checkpointing, slots=slots)
    q0 = torch.from_numpy(prob.fields).cuda()
    rng = np.random.default_rng(1)
    c = torch.from_numpy(rng.uniform(0.8, 1.2, d.nelements)).cuda()
    return solver, q0, c


@pytest.mark.parametrize("checkpointing", ["binomial", "segments"])
def test_gradient_matches_finite_differences(checkpointing):
    from actx_dgfem_suite_gb300.adjoint import WaveMisfitFunction
    solver, q0, c = _small_solver(checkpointing=checkpointing)
    obs = WaveMisfitFunction.apply(q0, c * 1.05, solver).detach()

    def loss(qq, cc):
        t = WaveMisfitFunction.apply(qq, cc, solver)
        return 0.5 * torch.sum((t - obs) ** 2)

    qv = q0.clone().requires_grad_(True)
    cv = c.clone().requires_grad_(True)
    J = loss(qv, cv)
    J.backward()
    gq, gc = qv.grad, cv.grad
    rng = np.random.default_rng(7)
    dc = torch.from_numpy(rng.standard_normal(c.shape[0])).cuda()
    dq = torch.from_numpy(rng.standard_normal(tuple(q0.shape))).cuda()
    for (dirq, dirc) in ((None, dc), (dq, None)):
        eps = 1e-5
        with torch.no_grad():
            qp = q0 + eps * dirq if dirq is not None else q0
            qm = q0 - eps * dirq if dirq is not None else q0
            cp = c + eps * dirc if dirc is not None else c
            cm = c - eps * dirc if dirc is not None else c
            fd = (float(loss(qp, cp)) - float(loss(qm, cm))) / (2 * eps)
        an = float(torch.sum(gq * dirq)) if dirq is not None else float(torch.sum(gc * dirc))
        tol = 1e-9 if dirq is not None else 2e-5  # loss is quadratic in q0
        assert abs(fd - an) <= tol * max(abs(an), 1e-30), (fd, an)


def test_gradient_deterministic():
    from actx_dgfem_suite_gb300.adjoint import WaveMisfitFunction
    solver, q0, c = _small_solver(nsteps=7)
    grads = []
    for _ in range(2):
        qv = q0.clone().requires_grad_(True)
        cv = c.clone().requires_grad_(True)
        t = WaveMisfitFunction.apply(qv, cv, solver)
        (t ** 2).sum().backward()
        grads.append((qv.grad.clone(), cv.grad.clone()))
    assert torch.equal(grads[0][0], grads[1][0])
    assert torch.equal(grads[0][1], grads[1][1])


def test_checkpointing_schemes_agree():
    """Binomial (few slots, many recomputations) and segment checkpointing
    give the same gradient."""
    from actx_dgfem_suite_gb300.adjoint import WaveMisfitFunction
    grads = []
    for scheme, slots in (("segments", None), ("binomial", 2), ("binomial", 5)):
        solver, q0, c = _small_solver(nsteps=17, checkpointing=scheme, slots=slots)
        qv = q0.clone().requires_grad_(True)
        cv = c.clone().requires_grad_(True)
        t = WaveMisfitFunction.apply(qv, cv, solver)
        (0.5 * (t ** 2).sum()).backward()
        grads.append((qv.grad.clone(), cv.grad.clone()))
        if scheme == "binomial":
            assert solver.stats["peak_stored_states"] <= slots + 1
    for gq, gc in grads[1:]:
        assert float(torch.linalg.norm(gq - grads[0][0])) <= 1e-12 * float(torch.linalg.norm(grads[0][0]))
        assert float(torch.linalg.norm(gc - grads[0][1])) <= 1e-12 * float(torch.linalg.norm(grads[0][1]))


@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("alias", ["none", "x_is_lam", "rbar_in_place"])
def test_fused_adjoint_stage_matches_composition(order, alias):
    """dg_rhs_adjoint_stage == the same stage composed from the plain
    transpose and elementwise operations: lam += dt L^T rbar, rbar_out =
    a rbar + b lam, cbar_e += dt <rbar, lq>_e, including the aliasing the
    reverse sweep uses (x = lam on its first stage, rbar updated in place)."""
    prob = make_problem("wave", jittered_box_mesh(3), order)
    plan = _plan(prob.disc, 1.3)
    g = torch.Generator(device="cuda:0").manual_seed(10 + order)
    shape, nel = plan.shape, plan.shape[1]
    rnd = lambda: torch.randn(shape, dtype=torch.float64, device="cuda:0", generator=g)  # noqa: E731
    c = 0.8 + 0.4 * torch.rand(nel, dtype=torch.float64, device="cuda:0", generator=g)
    plan.set_element_scale(c)
    lam, lq = rnd(), rnd()
    x = lam.clone() if alias == "x_is_lam" else rnd()
    cbar = torch.rand(nel, dtype=torch.float64, device="cuda:0", generator=g)
    xscale, a, b, dt = (0.7, -0.4, 0.3, 1e-2)
    rb = xscale * x
    lam_ref = lam + dt * plan.adjoint(rb)
    rbar_ref = a * rb + b * lam_ref
    cbar_ref = cbar + dt * (rb * lq).sum(dim=(0, 2))
    ysc = torch.empty_like(x)
    if alias == "x_is_lam":
        xin, out = lam, torch.empty_like(x)
    elif alias == "rbar_in_place":
        xin = out = x
    else:
        xin, out = x, torch.empty_like(x)
    plan.adjoint_stage(xin, xscale, lam, out, lq, cbar, a, b, dt, ysc)
    plan.finish()
    for got, ref in ((lam, lam_ref), (out, rbar_ref), (cbar, cbar_ref)):
        err = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
        assert err <= 1e-14, err

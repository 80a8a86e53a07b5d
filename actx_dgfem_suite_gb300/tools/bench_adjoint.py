"""Adjoint benchmark: gradient of a receiver misfit through the wave solve.

Default configuration: wave P3 on [-1, 1]^3 with 6 * 40^3 tetrahedra,
per-element wave speed c_e ~ U[0.8, 1.2] (seed 0), Gaussian-pulse initial
pressure, 300 LSRK45 steps, 256 receivers at random interior points (seed 1),
loss = 1/2 sum (traces - observations)^2 with observations computed from a
perturbed speed c_e (1 + 0.05 xi_e), xi_e ~ U[-1, 1] (seed 2).

Reports the forward and adjoint cost per step, the checkpoint memory, and
central finite-difference checks of the gradient with respect to c_e and the
initial state along random directions (FP64).

``--equation euler``: the Euler P3 adjoint instead (6 * 24^3 tetrahedra,
100 LSRK45 steps, 64 density receivers, gradient with respect to the initial
state, see :func:`run_euler`).

``python -m actx_dgfem_suite_gb300.tools.bench_adjoint [--equation euler] [--n N --steps S]``
prints one JSON line.
"""

from __future__ import annotations

import argparse
import json


def run(n: int = 40, order: int = 3, nsteps: int = 300, nrec: int = 256,
        cfl: float = 0.5, fd_eps: float = 1e-5, compare_binomial: bool = True) -> dict:
    import time

    import numpy as np
    import torch

    from actx_dgfem_suite_gb300.adjoint import (Receivers, WaveAdjointSolver,
                                                WaveMisfitFunction,
                                                random_interior_points)
    from actx_dgfem_suite_gb300.equations.wave import wave_problem
    from actx_dgfem_suite_gb300.perf_model import RhsCost
    from actx_dgfem_suite_gb300.timestepping import estimate_rk4_timestep

    t0 = time.perf_counter()
    prob = wave_problem(order, n, "baseline")
    d = prob.disc
    pts = random_interior_points(nrec, (-1, -1, -1), (1, 1, 1), 0.05, seed=1)
    rec = Receivers(d, pts, "cuda")
    dt = estimate_rk4_timestep(d, 1.2, cfl)
    solver = WaveAdjointSolver(d, dt, nsteps, rec)
    q0 = torch.from_numpy(prob.fields).to(solver.device)
    rng = np.random.default_rng(0)
    c = torch.from_numpy(rng.uniform(0.8, 1.2, d.nelements)).to(solver.device)
    xi = np.random.default_rng(2).uniform(-1, 1, d.nelements)
    c_obs = c * torch.from_numpy(1 + 0.05 * xi).to(solver.device)
    setup_s = time.perf_counter() - t0

    with torch.no_grad():
        obs = WaveMisfitFunction.apply(q0, c_obs, solver)

    def loss(qq, cc):
        t = WaveMisfitFunction.apply(qq, cc, solver)
        return 0.5 * torch.sum((t - obs) ** 2)

    # warm-up of every piece the timed solve uses (kernels, receiver products,
    # allocator) on a short solver over the same mesh: the first gradient of
    # a process otherwise ran up to 1.3x slower per step
    warm = WaveAdjointSolver(d, dt, 2 * solver.segment, rec)
    qw = q0.clone().requires_grad_(True)
    cw = c.clone().requires_grad_(True)
    WaveMisfitFunction.apply(qw, cw, warm).square().sum().backward()
    del warm, qw, cw

    qv = q0.clone().requires_grad_(True)
    cv = c.clone().requires_grad_(True)
    torch.cuda.synchronize()
    s = time.perf_counter()
    J = loss(qv, cv)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - s
    s = time.perf_counter()
    J.backward()
    torch.cuda.synchronize()
    t_bwd = time.perf_counter() - s
    gq, gc = qv.grad, cv.grad

    checks = {}
    r2 = np.random.default_rng(7)
    dirs = {"c": (None, torch.from_numpy(r2.standard_normal(d.nelements)).to(solver.device)),
            "q0": (torch.from_numpy(r2.standard_normal(tuple(q0.shape))).to(solver.device), None)}
    for name, (dq, dc) in dirs.items():
        with torch.no_grad():
            qp = q0 + fd_eps * dq if dq is not None else q0
            qm = q0 - fd_eps * dq if dq is not None else q0
            cp = c + fd_eps * dc if dc is not None else c
            cm = c - fd_eps * dc if dc is not None else c
            fd = (float(loss(qp, cp)) - float(loss(qm, cm))) / (2 * fd_eps)
        an = float(torch.sum(gq * dq)) if dq is not None else float(torch.sum(gc * dc))
        checks[name] = {"adjoint": an, "finite_difference": fd,
                        "rel_diff": abs(an - fd) / max(abs(fd), 1e-300)}

    cost = RhsCost("wave", order, d.nelements)
    state_bytes = 4 * d.nelements * d.np_ * 8
    # the same gradient with binomial checkpointing (sqrt(N) state slots)
    binom = None
    if compare_binomial:
        bsolver = WaveAdjointSolver(d, dt, nsteps, rec, checkpointing="binomial")
        qb = q0.clone().requires_grad_(True)
        cb = c.clone().requires_grad_(True)
        torch.cuda.synchronize()
        s = time.perf_counter()
        tb = WaveMisfitFunction.apply(qb, cb, bsolver)
        Jb = 0.5 * torch.sum((tb - obs) ** 2)
        torch.cuda.synchronize()
        tb_fwd = time.perf_counter() - s
        s = time.perf_counter()
        Jb.backward()
        torch.cuda.synchronize()
        tb_bwd = time.perf_counter() - s
        binom = {"slots": bsolver.slots,
                 "peak_stored_states": bsolver.stats["peak_stored_states"],
                 "peak_extra_states": bsolver.stats["peak_stored_states"] + 5,
                 "recomputed_steps": bsolver.stats["recomputed_steps"],
                 "adjoint_over_forward": tb_bwd / tb_fwd,
                 "grad_rel_diff_vs_segments": {
                     "q0": float(torch.linalg.norm(qb.grad - gq) / torch.linalg.norm(gq)),
                     "c": float(torch.linalg.norm(cb.grad - gc) / torch.linalg.norm(gc))}}

    if solver.schedule is not None:
        ck = {"checkpointing": "binomial", "slots": solver.slots,
              "recomputed_steps": solver.stats.get("recomputed_steps"),
              "peak_stored_states": solver.stats.get("peak_stored_states"),
              "peak_extra_states": solver.stats.get("peak_stored_states", 0) + 5}
    else:
        nck = (nsteps - 1) // solver.segment + 1
        ck = {"checkpointing": "segments", "checkpoint_segment": solver.segment,
              "checkpoint_states": nck, "peak_extra_states": nck + 5 * solver.segment}
    return {
        "workload": (f"wave P{order}, 6*{n}^3 tets, {nsteps} LSRK45 steps, "
                     f"{nrec} receivers, c_e ~ U[0.8,1.2]"),
        "nelements": d.nelements,
        "dt": dt,
        "loss": float(J.detach()),
        "forward_ms_per_step": 1e3 * t_fwd / nsteps,
        "adjoint_ms_per_step": 1e3 * t_bwd / nsteps,
        "adjoint_over_forward": t_bwd / t_fwd,
        "forward_dof_updates_per_s": 5 * nsteps * cost.dofs / t_fwd,
        **ck,
        "binomial_checkpointing": binom,
        "state_mb": state_bytes / 1e6,
        "fd_checks": checks,
        "setup_s": setup_s,
    }


def run_euler(n: int = 24, order: int = 3, nsteps: int = 100, nrec: int = 64,
              cfl: float = 0.5, fd_eps: float = 1e-6) -> dict:
    """Euler P3 adjoint: gradient of a density-receiver misfit with respect to
    the initial state through ``nsteps`` LSRK45 steps (one fused reverse
    stage, ``dg_rhs_vjp_stage``, per stage), with its cost against the
    forward sweep and a central finite-difference check along a random
    direction."""
    import time

    import numpy as np
    import torch

    from actx_dgfem_suite_gb300.adjoint import (EulerAdjointSolver, EulerMisfitFunction,
                                                Receivers, random_interior_points)
    from actx_dgfem_suite_gb300.equations.euler import euler_problem
    from actx_dgfem_suite_gb300.timestepping import estimate_rk4_timestep

    prob = euler_problem(order, n, "baseline")
    d = prob.disc
    pts = random_interior_points(nrec, (-0.5,) * 3, (0.5,) * 3, 0.05, seed=1)
    rec = Receivers(d, pts, "cuda")
    dt = estimate_rk4_timestep(d, 1.3, cfl)
    solver = EulerAdjointSolver(d, prob.params[0], dt, nsteps, rec)
    q0 = torch.from_numpy(prob.fields).to(solver.device)
    rng = np.random.default_rng(3)
    pert = torch.from_numpy(1 + 0.01 * rng.standard_normal(tuple(q0.shape))).to(solver.device)
    with torch.no_grad():
        obs = EulerMisfitFunction.apply(q0 * pert, solver)

    def loss(qq):
        return 0.5 * torch.sum((EulerMisfitFunction.apply(qq, solver) - obs) ** 2)

    # one gradient on a short solver over the same mesh first, as for the wave
    warm = EulerAdjointSolver(d, prob.params[0], dt, 2 * solver.segment, rec)
    qw = q0.clone().requires_grad_(True)
    EulerMisfitFunction.apply(qw, warm).square().sum().backward()
    del warm, qw

    qv = q0.clone().requires_grad_(True)
    torch.cuda.synchronize()
    s = time.perf_counter()
    J = loss(qv)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - s
    s = time.perf_counter()
    J.backward()
    torch.cuda.synchronize()
    t_bwd = time.perf_counter() - s
    dq = torch.from_numpy(rng.standard_normal(tuple(q0.shape))).to(solver.device)
    with torch.no_grad():
        fd = (float(loss(q0 + fd_eps * dq)) - float(loss(q0 - fd_eps * dq))) / (2 * fd_eps)
    an = float(torch.sum(qv.grad * dq))
    return {
        "workload": (f"Euler P{order}, 6*{n}^3 tets, {nsteps} LSRK45 steps, {nrec} "
                     "density receivers, gradient wrt the initial state"),
        "nelements": d.nelements,
        "forward_ms_per_step": 1e3 * t_fwd / nsteps,
        "adjoint_ms_per_step": 1e3 * t_bwd / nsteps,
        "adjoint_over_forward": t_bwd / t_fwd,
        "checkpoint_segment": solver.segment,
        "fd_check_q0": {"adjoint": an, "finite_difference": fd,
                        "rel_diff": abs(an - fd) / max(abs(fd), 1e-300)},
    }


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m actx_dgfem_suite_gb300.tools.bench_adjoint")
    ap.add_argument("--equation", choices=("wave", "euler"), default="wave")
    ap.add_argument("--n", type=int, default=None,
                    help="hexahedra per axis (default 40 for wave, 24 for Euler)")
    ap.add_argument("--order", type=int, default=3)
    ap.add_argument("--steps", type=int, default=None,
                    help="LSRK45 steps (default 300 for wave, 100 for Euler)")
    ap.add_argument("--receivers", type=int, default=None,
                    help="receivers (default 256 for wave, 64 for Euler)")
    a = ap.parse_args(argv)
    if a.equation == "wave":
        res = run(a.n or 40, a.order, a.steps or 300, a.receivers or 256)
    else:
        res = run_euler(a.n or 24, a.order, a.steps or 100, a.receivers or 64)
    print(json.dumps(res))


if __name__ == "__main__":
    main()

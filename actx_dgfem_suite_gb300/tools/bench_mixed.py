"""Mixed-precision vs FP64 time integration benchmark.

Euler P3 on a box of 6 n^3 tetrahedra (n = 56 by default: 1,053,696 elements,
21 M DOFs per variable), benchmark initial state (density pulse on a uniform
flow), ``nsteps`` LSRK(5,4) steps run twice from the same state: once with the
FP64 plan and once with the FP32-arithmetic plan (FP64 state, FP64 pressure
recovery, FP64 RK accumulation).  After every step the relative L2 error of the
mixed state against the FP64 state is recorded, both relative to ||q|| and
relative to ||q(t) - q(0)||, the part of the state that actually evolves.

``python -m actx_dgfem_suite_gb300.tools.bench_mixed [--n 56 --steps 100]``
prints one JSON line.
"""

from __future__ import annotations

import argparse
import json


def run(n: int = 56, order: int = 3, nsteps: int = 100, cfl: float = 0.5,
        problem=None, device=None) -> dict:
    import torch

    from actx_dgfem_suite_gb300.perf_model import RhsCost
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    from actx_dgfem_suite_gb300.rhs_builder import get_problem
    from actx_dgfem_suite_gb300.timestepping import LSRK45, estimate_rk4_timestep

    if problem is None:
        try:
            from actx_dgfem_suite_gb300.device_setup import device_problem
            problem = device_problem("euler", order, n, "baseline", device)
        except Exception:
            problem = get_problem("euler", 3, order, definition="baseline", nel_1d=n)
    disc = problem.disc
    mesh = DeviceMesh(disc, device)
    plans = {p: DevicePlan(mesh, "euler", problem.params, p)
             for p in ("fp64", "fp32-mixed")}
    # max wave speed of the benchmark state ~ |u| + c = 0.1 + sqrt(1.4) < 1.3
    dt = estimate_rk4_timestep(disc, 1.3, cfl)
    q0 = (problem.fields if isinstance(problem.fields, torch.Tensor)
          else torch.from_numpy(problem.fields)).to(mesh.device)
    qs = {p: q0.clone() for p in plans}
    integ = {p: LSRK45(plans[p], dt) for p in plans}
    # warm-up: one stage each, on scratch copies
    for p in plans:
        tmp = q0.clone()
        LSRK45(plans[p], dt).step(tmp)
    torch.cuda.synchronize()

    stream = torch.cuda.current_stream()
    times = {p: 0.0 for p in plans}
    err_q, err_dq = [], []
    nq0 = float(torch.linalg.norm(q0))
    for _ in range(nsteps):
        for p in plans:
            s, e = torch.cuda.Event(True), torch.cuda.Event(True)
            s.record(stream)
            integ[p].step(qs[p])
            e.record(stream)
            e.synchronize()
            times[p] += s.elapsed_time(e) * 1e-3
        d = qs["fp32-mixed"] - qs["fp64"]
        nd = float(torch.linalg.norm(d))
        err_q.append(nd / float(torch.linalg.norm(qs["fp64"])))
        err_dq.append(nd / max(float(torch.linalg.norm(qs["fp64"] - q0)), 1e-300))
    for p in plans:
        plans[p].finish()
    cost = RhsCost("euler", order, disc.nelements)
    rates = {p: 5 * nsteps * cost.dofs / times[p] for p in plans}
    return {
        "workload": f"Euler P{order}, 6*{n}^3 tets, {nsteps} LSRK45 steps, dt={dt:.3e}",
        "nelements": disc.nelements,
        "dof_updates_per_s": rates,
        "speedup_vs_fp64": rates["fp32-mixed"] / rates["fp64"],
        "ms_per_step": {p: 1e3 * times[p] / nsteps for p in plans},
        "max_rel_err_vs_fp64": max(err_q),
        "max_rel_err_of_change_vs_fp64": max(err_dq),
        "final_rel_err_vs_fp64": err_q[-1],
        "err_per_step": err_q,
        "input_norm": nq0,
    }


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m actx_dgfem_suite_gb300.tools.bench_mixed")
    ap.add_argument("--n", type=int, default=56)
    ap.add_argument("--order", type=int, default=3)
    ap.add_argument("--steps", type=int, default=100)
    a = ap.parse_args(argv)
    print(json.dumps(run(a.n, a.order, a.steps)))


if __name__ == "__main__":
    main()

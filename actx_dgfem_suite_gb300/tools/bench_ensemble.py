"""Ensemble benchmark: many Maxwell members in one launch vs one FP64 call
per member.

Default configuration: 64 Maxwell P3 members on boxes [0,1]^3 with
n ~ U[12, 40] hexahedra per axis (seed 0; uneven element counts), each member
with its own seeded plane-wave state, upwind flux (alpha = 1), PEC walls.
The batched RHS (FP32 arithmetic, FP64 state) is one persistent launch over
the concatenated members, captured in a CUDA graph and replayed; the
baseline is 64 sequential plain FP64 RHS calls on the members' own plans.

``python -m actx_dgfem_suite_gb300.tools.bench_ensemble [--members 64]``
prints one JSON line.
"""

from __future__ import annotations

import argparse
import json


def run(members: int = 64, lo: int = 12, hi: int = 40, order: int = 3,
        reps: int = 10, seed: int = 0, precision: str = "fp32-mixed",
        device_setup: bool = True, max_rel_l2: float | None = 1e-5) -> dict:
    import time

    import numpy as np
    import torch

    from actx_dgfem_suite_gb300.discretization import clear_box_cache
    from actx_dgfem_suite_gb300.ensemble import Ensemble, random_box_sizes
    from actx_dgfem_suite_gb300.equations.maxwell import maxwell_problem
    from actx_dgfem_suite_gb300.perf_model import RhsCost
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan

    t0 = time.perf_counter()
    sizes = random_box_sizes(members, lo, hi, seed)
    order_of_build = sorted(range(members), key=lambda k: sizes[k])
    probs = [None] * members
    if device_setup:
        from actx_dgfem_suite_gb300.device_setup import device_problem
        for k in range(members):
            probs[k] = device_problem("maxwell", order, sizes[k], "baseline",
                                      seed=seed + 1 + k)
    else:
        for k in order_of_build:      # equal sizes consecutively: mesh cache hits
            probs[k] = maxwell_problem(order, sizes[k], "baseline", seed=seed + 1 + k)
    clear_box_cache()
    ens = Ensemble([p.disc for p in probs], "maxwell", probs[0].params, precision)
    q = ens.stack_states([p.fields for p in probs])
    out = torch.empty_like(q)
    member_plans, member_q, member_out = [], [], []
    for p in probs:
        plan = DevicePlan(DeviceMesh(p.disc), "maxwell", p.params, "fp64")
        member_plans.append(plan)
        qq = (p.fields if isinstance(p.fields, torch.Tensor)
              else torch.from_numpy(p.fields)).cuda()
        member_q.append(qq)
        member_out.append(torch.empty_like(qq))
    for p in probs:
        if hasattr(p.disc, "_cache"):
            p.disc._cache.clear()
    setup_s = time.perf_counter() - t0

    tuning = ens.autotune(q, reps=3, max_rel_l2=max_rel_l2)
    ens.capture(q, out)
    stream = torch.cuda.current_stream()
    for _ in range(3):
        ens.replay()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(True), torch.cuda.Event(True)
    s.record(stream)
    for _ in range(reps):
        ens.replay()
    e.record(stream)
    torch.cuda.synchronize()
    t_ens = s.elapsed_time(e) * 1e-3 / reps

    for k in range(members):
        member_plans[k].rhs(member_q[k], member_out[k])
    torch.cuda.synchronize()
    nrep64 = max(1, reps // 3)
    s.record(stream)
    for _ in range(nrep64):
        for k in range(members):
            member_plans[k].rhs(member_q[k], member_out[k])
    e.record(stream)
    torch.cuda.synchronize()
    t_seq = s.elapsed_time(e) * 1e-3 / nrep64
    ens.plan.finish()
    for pl in member_plans:
        pl.finish()

    num = den = 0.0
    for k in range(members):
        a = ens.member(out, k)
        b = member_out[k]
        num += float(torch.sum((a - b) ** 2))
        den += float(torch.sum(b ** 2))
    nel = int(ens.union.nelements)
    dofs = RhsCost("maxwell", order, nel).dofs
    return {
        "workload": (f"{members} Maxwell P{order} members, n ~ U[{lo},{hi}] "
                     f"(seed {seed}), one graph-replayed launch ({precision}) vs "
                     f"{members} sequential FP64 calls"),
        "nelements_total": nel,
        "member_sizes": sizes,
        "dof_updates_per_s": dofs / t_ens,
        "fp64_sequential_dof_updates_per_s": dofs / t_seq,
        "speedup_vs_sequential_fp64": t_seq / t_ens,
        "ms_per_rhs": t_ens * 1e3,
        "ms_per_rhs_fp64_sequential": t_seq * 1e3,
        "rel_l2_err_vs_fp64": float(np.sqrt(num / den)),
        "setup_s": setup_s,
        "plan": ens.plan.info(),
        "autotune": tuning,
    }


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m actx_dgfem_suite_gb300.tools.bench_ensemble")
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--lo", type=int, default=12)
    ap.add_argument("--hi", type=int, default=40)
    ap.add_argument("--order", type=int, default=3)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--precision", default="fp32-mixed")
    a = ap.parse_args(argv)
    print(json.dumps(run(a.members, a.lo, a.hi, a.order, a.reps,
                         precision=a.precision)))


if __name__ == "__main__":
    main()

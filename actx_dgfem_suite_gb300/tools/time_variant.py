"""Time one benchmark case under a given precision and launch variant, and
report its error against the FP64 plan.

The case is built through the public API (``get_rhs(..., definition="baseline")``
with ``nel_1d`` hexahedra per axis, 6 tetrahedra each); the plan's launch
variant is set explicitly (``DevicePlan.VARIANTS``: 0 persistent, 1
tensor-core persistent, 2 one CTA per tile, 3 tensor-core one CTA per tile,
4 tcgen05 exact digits, 5 tcgen05 3xTF32, 6 the same at its other CTA size,
7-10 the tensor-core kernel at 128- and 512-thread tiles) instead of
autotuned, so a profiler can capture one kernel.  ``--dim 2`` times the
triangle-mesh kernel (``n`` squares per axis, 2 triangles each; FP64, one
variant).

``python -m actx_dgfem_suite_gb300.tools.time_variant maxwell 3 --n 28 --variant 5``
prints one JSON line.
"""

from __future__ import annotations

import argparse
import json


def run(equation: str, order: int, n: int, precision: str = "fp32-mixed",
        variant: int = 0, reps: int = 5, dim: int = 3) -> dict:
    import torch

    from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs

    actx = GB300DGArrayContext("cuda:0")
    rhs, call_args = get_rhs(equation, actx, dim, order, definition="baseline", nel_1d=n)
    op = rhs.dg_operator
    compiled = actx.compile(rhs)
    q = compiled.stage(call_args[-1])
    op.precision = "fp64"
    ref = op.plan_for(actx).rhs(q)
    op.precision = precision
    plan = op.plan_for(actx)
    plan.set_variant(variant)
    out = torch.empty_like(q)
    for _ in range(2):
        plan.rhs(q, out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
    e0.record()
    for _ in range(reps):
        plan.rhs(q, out)
    e1.record()
    torch.cuda.synchronize()
    info = plan.info()
    return {"equation": equation, "dim": dim, "order": order, "n": n,
            "nelements": info["nelements"],
            "dof_updates_per_s": out.numel() / (e0.elapsed_time(e1) / reps * 1e-3),
            "precision": precision, "variant": plan.VARIANTS[variant],
            "ms": e0.elapsed_time(e1) / reps,
            "rel_l2_err_vs_fp64": float(torch.linalg.norm(out - ref) / torch.linalg.norm(ref)),
            "grid": info["grid"], "block": info["block"], "smem_bytes": info["smem_bytes"]}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("equation", choices=("wave", "euler", "maxwell"))
    ap.add_argument("order", type=int)
    ap.add_argument("--n", type=int, default=20)
    ap.add_argument("--precision", default="fp32-mixed",
                    choices=("fp64", "fp64-tc", "fp32-mixed"))
    ap.add_argument("--variant", type=int, default=0)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--dim", type=int, default=3, choices=(2, 3))
    args = ap.parse_args()
    print(json.dumps(run(args.equation, args.order, args.n, args.precision,
                         args.variant, args.reps, args.dim)))


if __name__ == "__main__":
    main()

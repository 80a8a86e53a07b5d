"""Wave-operator DOF-throughput sweep, mirroring
``actx_dgfem_suite/tools/wave_dof_scaling.py``.

For each degree and DOF budget per field, builds the wave RHS, runs the
suite's warm-up / timing protocol (``wave_dof_scaling.py:128-160``) and
reports GDOF/s counting all ``dim + 1`` fields (``wave_dof_scaling.py:162-169``).
``python -m actx_dgfem_suite_gb300.tools.wave_dof_scaling --degrees 1,2,3,4``
"""

from __future__ import annotations

import argparse
import gc
import json
from time import time

#: DOF budgets per field for the GB300 sweep (the reference's list for
#: H200 NVL is 1M..27M, ``wave_dof_scaling.py:58-73``)
GB300_NDOFS = (1_000_000, 5_000_000, 10_000_000, 15_000_000, 20_000_000,
               25_000_000, 27_000_000)


def sweep(degrees, ndofs_list, precision: str = "fp64", dim: int = 3,
          device_setup: bool = False, events: bool = False):
    """GDOF/s per (degree, DOF budget).  ``device_setup``: build the mesh and
    initial state on the GPU (``device_problem``) instead of on the host;
    ``events``: time 3 warm-up and 10 timed RHS with CUDA events instead of
    the suite's wall-clock protocol (a quick sweep)."""
    import torch

    from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext
    from actx_dgfem_suite_gb300.equations.wave import wave_problem
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    from actx_dgfem_suite_gb300.utils import (get_ndof_for_regular_rect_mesh,
                                              get_nel_1d_for_regular_rect_mesh)
    actx = GB300DGArrayContext()
    out = {}
    for degree in degrees:
        for ndofs in ndofs_list:
            nel_1d = get_nel_1d_for_regular_rect_mesh(dim, degree, int(ndofs))
            if device_setup:
                if dim != 3:
                    raise NotImplementedError("device-side setup builds 3D meshes only")
                from actx_dgfem_suite_gb300.device_setup import device_problem
                prob = device_problem("wave", degree, nel_1d, "reference", actx.device)
            else:
                prob = wave_problem(degree, nel_1d, "reference", dim=dim)
            plan = DevicePlan(DeviceMesh(prob.disc, actx.device), "wave",
                              prob.params, precision)
            q = torch.as_tensor(prob.fields).to(actx.device)
            o = torch.empty_like(q)
            plan.rhs(q, o)
            actual = get_ndof_for_regular_rect_mesh(dim, degree, nel_1d)
            if events:
                for _ in range(3):
                    plan.rhs(q, o)
                e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
                e0.record()
                for _ in range(10):
                    plan.rhs(q, o)
                e1.record()
                plan.finish()
                out[(degree, ndofs)] = actual * (dim + 1) / (e0.elapsed_time(e1) * 1e-4)
                del plan, q, o, prob
                gc.collect()
                continue
            i_warmup, t_warmup = 0, 0.0
            while i_warmup < 5 and t_warmup < 2:
                plan.finish()
                t0 = time()
                plan.rhs(q, o)
                plan.finish()
                t_warmup += time() - t0
                i_warmup += 1
            i_timing, t_rhs = 0, 0.0
            while i_timing < 50 and t_rhs < 4:
                plan.finish()
                t0 = time()
                for _ in range(3):
                    plan.rhs(q, o)
                plan.finish()
                t_rhs += time() - t0
                i_timing += 3
            out[(degree, ndofs)] = actual * (dim + 1) / (t_rhs / i_timing)
            del plan, q, o, prob
            gc.collect()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m actx_dgfem_suite_gb300.tools.wave_dof_scaling")
    ap.add_argument("--degrees", default="1,2,3,4")
    ap.add_argument("--ndofs", default=",".join(str(n) for n in GB300_NDOFS))
    ap.add_argument("--precision", default="fp64", choices=("fp64", "fp32-mixed"))
    ap.add_argument("--dim", type=int, default=3, choices=(2, 3),
                    help="topological dimension (the reference's --dim; 2: "
                         "triangles, FP64)")
    ap.add_argument("--json", action="store_true")
    a = ap.parse_args(argv)
    degrees = [int(x) for x in a.degrees.split(",")]
    ndofs = [int(float(x)) for x in a.ndofs.split(",")]
    res = sweep(degrees, ndofs, a.precision, dim=a.dim)
    if a.json:
        print(json.dumps({f"P{d}@{n}": v for (d, n), v in res.items()}))
        return res
    print(f"GDOFS/s for {a.dim}D-wave:")
    print("      " + "".join(f"{n / 1e6:>10.1f}M" for n in ndofs))
    for d in degrees:
        print(f"P{d:<5d}" + "".join(f"{res[(d, n)] * 1e-9:>11.3f}" for n in ndofs))
    return res


if __name__ == "__main__":
    main()

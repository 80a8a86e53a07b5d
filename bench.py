#!/usr/bin/env python
"""Benchmark of the plain FP64 DG-FEM RHS on GB300.

Workload (one "step"): one RHS evaluation of each of the 12 benchmark cases
-- wave, Euler and Maxwell at P1/P2/P3/P4 on box meshes of 6 n^3 tetrahedra
with n = 95/70/56/46 (the suite's ``large_`` sizes), benchmark ("baseline")
problem definitions, FP64.  Metric: RHS DOF-updates/s (nfields * Nel * Np per
RHS), whole job.

* ``value``: device-resident inputs; per-case CUDA events on the launch
  stream; every case's state is larger than L2 (129 MB), so no L2 flush is
  needed between launches.
* ``e2e``: the same step through the public API with host buffers:
  ``compiled(t, host_state)`` for every case (host->device copy of each
  page-locked state on the context's copy stream, overlapping the kernels of
  the cases before it; the calls go in descending kernel time per input
  byte, so the copy-heavy low-order cases upload behind the long kernels),
  then ``actx.to_numpy_batch(results)`` in the same order (device->host
  copy of each result into a new page-locked array behind its own kernel,
  one wait at the end), all inside the timed
  region; 3-4 untimed steps (the first ones pay the host allocations), then
  min(steps, 5) timed steps.  ``logged_steps``: as many steps again with
  the array context's transfer log on (the copies' busy times and rates, the
  span to the last copy, the end of the last kernel, the wall time);
  ``split_ms``: the logged step of median wall time, beside the kernels'
  time of the device-resident step.
* ``parity``: every case at the CPU sample's size (n // cpu-scale) through
  the public API against the CPU oracle's RHS of the same run.
* ``--impl reference``: the CPU FP64 oracle (a restatement of the
  reference's operators; the reference itself cannot run here) on a bounded
  sample of every case, one process per case over the host's cores.

Multi-GPU (torchrun): every rank runs an independent replica (the operator
does not shard without a halo exchange); value = all ranks' DOF updates over
the max-over-ranks time, ``scaling`` = "weak".
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

CASES = [(eq, p, n) for eq in ("wave", "euler", "maxwell")
         for p, n in ((1, 95), (2, 70), (3, 56), (4, 46))]
METRIC = "RHS DOF-updates/s (plain FP64, wave+Euler+Maxwell P1-P4 sweep)"
UNIT = "DOF-updates/s"
#: relative L2 bound of the mixed-precision results against FP64
MIXED_RTOL = 1e-5
WORKLOAD = ("plain FP64 RHS sweep: {wave, euler, maxwell} x P1-P4 on box meshes "
            "of 6 n^3 tets, n = 95/70/56/46; one RHS per case per step")


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float, device) -> float:
    """The maximum of a per-rank time over all ranks of the initialised
    process group (the replica that finished last sets the job's time);
    ``value`` itself for a single process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank: float, seconds: float, world: int) -> float:
    """Whole-job rate of ``world`` independent replicas that each process
    ``units_per_rank`` in at most ``seconds`` (the max over ranks)."""
    return world * units_per_rank / seconds


# {{{ clocks sampling


class ClockSampler:
    """Samples SM clock and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# }}}


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def _ncu_traffic(path: str) -> dict:
    """DRAM bytes of one RHS (all its launches) from the committed ncu
    summary, keyed by case, for the FP64 path ``path`` ("shared"/"fused")."""
    out = {}
    p = ROOT / "profiles" / "dram_traffic_fp64_rhs.txt"
    if p.exists():
        for ln in p.read_text().splitlines():
            f = ln.split()
            if len(f) >= 4 and f[0] == "traffic" and f[3] == path:
                out[f[1]] = float(f[2])
    return out


def fp64_peak_tflops(torch) -> float:
    """FP64 FMA throughput of the device (library probe, CUDA events)."""
    import ctypes

    from actx_dgfem_suite_gb300 import _lib
    L = _lib.lib()
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    grid, block, iters = nsm * 8, 256, 4000
    buf = torch.empty(grid * block, dtype=torch.float64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    best = 0.0
    for _ in range(2):   # let the clocks settle before timing
        _lib.check(L.dg_fp64_fma_probe(ctypes.c_void_p(buf.data_ptr()), iters,
                                       grid, block, st))
    for _ in range(5):
        s, e = torch.cuda.Event(True), torch.cuda.Event(True)
        s.record()
        _lib.check(L.dg_fp64_fma_probe(ctypes.c_void_p(buf.data_ptr()), iters,
                                       grid, block, st))
        e.record()
        torch.cuda.synchronize()
        best = max(best, 16.0 * iters * grid * block / (s.elapsed_time(e) * 1e-3))
    return best / 1e12


def bench_config(args, world: int) -> dict:
    """The workload description both arms print (the reference arm times a
    bounded sample of it, described in its ``cpu_baseline.sample``)."""
    return {"workload": WORKLOAD, "problem": "baseline definitions",
            "precision": args.precision,
            "l2": "inputs larger than L2 (every case's state > 129 MB)",
            "parallelism": f"replicas x{world}",
            "scale_divisor": args.scale}


# {{{ reference arm (CPU oracle)


def _oracle_case(args):
    """One case of the CPU oracle sweep: (DOF updates, seconds per RHS, and
    with ``keep`` the oracle's RHS for the parity check)."""
    eq, order, n_sample, reps, keep = args
    import numpy as np

    from actx_dgfem_suite_gb300.rhs_builder import get_problem
    from oracle.geometry import build_oracle_disc
    from oracle.rhs import euler_rhs, maxwell_rhs, wave_rhs
    prob = get_problem(eq, 3, order, definition="baseline", nel_1d=n_sample)
    d = prob.disc
    od = build_oracle_disc(d.mesh.vertices, d.mesh.elements, order)
    q = prob.fields
    t0 = time.perf_counter()
    for _ in range(reps):
        if eq == "wave":
            rhs = wave_rhs(od, q[0], q[1:4], *prob.params)
        elif eq == "euler":
            rhs = euler_rhs(od, q, *prob.params)
        else:
            rhs = maxwell_rhs(od, q, *prob.params)
    dt = (time.perf_counter() - t0) / reps
    dofs = prob.nfields * d.nelements * d.np_
    if not keep:
        return dofs, dt, None
    if eq == "wave":
        rhs = np.concatenate([rhs[0][None], rhs[1]])
    # the product's nodes must sit at the oracle's (independently built) ones
    node_err = float(np.max(np.abs(d.nodes() - od.nodes)))
    return dofs, dt, {"rhs": np.asarray(rhs), "node_err": node_err}


def cpu_sample_sizes(scale: int) -> list[int]:
    return [max(2, n // scale) for (_, _, n) in CASES]


def run_oracle_sweep(scale: int, reps: int = 1, procs: int | None = None,
                     keep: bool = False):
    """Times the oracle on every case at n // scale; returns (dofs, wall
    seconds, busy seconds, cores[, per-case outputs with ``keep``]), one
    process per case."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    sizes = cpu_sample_sizes(scale)
    jobs = [(eq, p, ns, reps, keep) for (eq, p, _), ns in zip(CASES, sizes)]
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"   # one core per worker process
    cores = procs or min(len(jobs), os.cpu_count() or 1)
    t0 = time.perf_counter()
    with ProcessPoolExecutor(max_workers=cores,
                             mp_context=mp.get_context("spawn")) as ex:
        res = list(ex.map(_oracle_case, jobs))
    wall = time.perf_counter() - t0
    dofs = sum(r[0] for r in res)
    busy = sum(r[1] for r in res)
    if keep:
        return dofs, wall, busy, cores, [r[2] for r in res]
    return dofs, wall, busy, cores


def reference_arm(args) -> None:
    rank, world, _ = _dist()
    if rank != 0:
        return
    scale = args.cpu_scale
    # warm-up: spawn cost, imports, operator assembly
    for _ in range(max(0, args.warmup)):
        run_oracle_sweep(scale, reps=1)
    times, dofs, cores = [], 0, 1
    for _ in range(args.steps):
        dofs, wall, busy, cores = run_oracle_sweep(scale, reps=1)
        # per-case evaluation time (excludes process start-up and setup)
        times.append(busy / cores)
    t = statistics.mean(times)
    value = dofs / t
    sample = (f"every case at n // {scale} ({', '.join(str(s) for s in cpu_sample_sizes(scale))}), "
              f"one process per case over {cores} host cores; time = summed "
              f"per-case RHS time / cores")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# }}}


def transfer_split(actx, step_fn, klog: list | None = None) -> dict:
    """One end-to-end step with the array context's transfer log on: the busy
    time of its host->device and device->host copies (sum of the copies'
    event intervals on the copy streams), the span from the step's first
    upload to its last result copy, when its last kernel ended (``kernels``,
    from the timing events ``step_fn`` appends to ``klog``), the copies'
    effective rates and the step's wall time."""
    import torch
    torch.cuda.synchronize()
    actx.transfer_log = []
    if klog is not None:
        klog.clear()
    t0 = torch.cuda.Event(enable_timing=True)
    t0.record(actx.h2d_stream)
    w = time.perf_counter()
    step_fn()
    wall = (time.perf_counter() - w) * 1e3
    torch.cuda.synchronize()
    log, actx.transfer_log = actx.transfer_log, None
    res = {}
    for kind in ("h2d", "d2h"):
        rows = [(a.elapsed_time(b), n) for k, a, b, n in log if k == kind]
        busy = sum(ms for ms, _ in rows)
        res[kind] = busy
        res[kind + "_gbs"] = sum(n for _, n in rows) / (busy * 1e-3) / 1e9 if busy > 0 else None
    ends = [t0.elapsed_time(b) for k, a, b, n in log]
    res["span"] = max(ends) if ends else 0.0
    res["kernels"] = max(t0.elapsed_time(e) for e in klog) if klog else None
    res["wall"] = wall
    return res


def parity_vs_oracle(actx, scale: int, outs: list) -> dict:
    """Every benchmark case at the CPU sample's size (n // scale), evaluated
    through the public API on the GPU (the default FP64 path, and fp64-tc
    at orders 3-4) and compared with the oracle's RHS from the CPU sweep:
    relative L2 error per case (bound 1e-12)."""
    import numpy as np

    from actx_dgfem_suite_gb300.containers import leaves
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs
    cases, worst = {}, 0.0
    for (eq, order, _), ns, o in zip(CASES, cpu_sample_sizes(scale), outs):
        ref = o["rhs"]
        rhs, call_args = get_rhs(eq, actx, 3, order, definition="baseline", nel_1d=ns)
        row = {"n": ns, "node_err": o["node_err"]}
        for prec in (("fp64", "fp64-tc") if order >= 3 else ("fp64",)):
            rhs.dg_operator.precision = prec
            got = np.stack([d[0] for d in leaves(actx.to_numpy(
                actx.compile(rhs)(*call_args)))])
            err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
            row["rel_l2" if prec == "fp64" else "rel_l2_fp64_tc"] = err
            worst = max(worst, err)
        cases[f"{eq}{order}"] = row
        del rhs, call_args
    return {"bound": 1e-12, "max_rel_l2": worst, "ok": bool(worst <= 1e-12),
            "against": "CPU FP64 oracle (independent reference element), same meshes",
            "cases": cases}


def run_extras(args, runs, actx, K, fp64_ms_per_step, fp64_case_ms) -> dict:
    """The forms built beside the plain FP64 path, each measured on its own
    benchmark configuration: mixed precision (the same 12-case sweep with
    FP32 arithmetic, with the accuracy of the exact-digit tcgen05 variant
    beside the autotuned one, and Euler P3 n=56 over 100 LSRK45 steps), FP64
    with the contractions emulated on tcgen05 (the P3/P4 cases), the
    64-member Maxwell ensemble, and the wave and Euler adjoints (gradients
    checked by finite differences).  Each entry reports its error against
    FP64."""
    import torch

    out = {}
    # {{{ mixed-precision sweep on the resident states
    try:
        stream = torch.cuda.current_stream()
        plans = []
        for r in runs:
            op = r["compiled"].op
            op.precision = "fp32-mixed"
            plans.append(op.plan_for(actx))
            op.precision = "fp64"
        outs = [torch.empty_like(r["q"]) for r in runs]
        # the autotuner picks each plan's launch variant (tensor-core or CUDA-core
        # products, persistent or one-CTA-per-tile grid, tcgen05) on the case's
        # own state, among the variants within MIXED_RTOL of the FP64 result
        tuned = [p.autotune(r["q"], reps=2, ref=r["out"], max_rel_l2=MIXED_RTOL)
                 for p, r in zip(plans, runs)]
        for _ in range(2):
            for p, r, o in zip(plans, runs, outs):
                p.rhs(r["q"], o)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(True), torch.cuda.Event(True)) for _ in runs]
        times = [0.0] * len(runs)
        for _ in range(K):
            for k, (p, r, o) in enumerate(zip(plans, runs, outs)):
                ev[k][0].record(stream)
                p.rhs(r["q"], o)
                ev[k][1].record(stream)
            torch.cuda.synchronize()
            for k in range(len(runs)):
                times[k] += ev[k][0].elapsed_time(ev[k][1]) / K
        errs = [float(torch.linalg.norm(o - r["out"]) / torch.linalg.norm(r["out"]))
                for o, r in zip(outs, runs)]
        dofs = sum(r["cost"].dofs for r in runs)
        out["mixed_precision_sweep"] = {
            "value": dofs / (sum(times) * 1e-3), "unit": UNIT,
            "ms_per_step": sum(times),
            "speedup_vs_fp64": fp64_ms_per_step / sum(times),
            "max_rel_l2_err_vs_fp64": max(errs),
            "cases_ms": {f"{r['eq']}{r['order']}": t for r, t in zip(runs, times)},
            "autotuned_variant": {f"{r['eq']}{r['order']}": p.VARIANTS[tu["chosen"]]
                                  for r, p, tu in zip(runs, plans, tuned)},
            "variant_ms": {f"{r['eq']}{r['order']}": tu["ms"] for r, tu in zip(runs, tuned)},
            "variant_rel_l2": {f"{r['eq']}{r['order']}": tu["rel_l2"]
                               for r, tu in zip(runs, tuned)},
            "error_budget": MIXED_RTOL,
            "cases_rel_l2_err_vs_fp64": {f"{r['eq']}{r['order']}": e
                                         for r, e in zip(runs, errs)},
        }
        # the exact-digit tcgen05 variant (4): its accuracy on every case
        tc_err = {}
        for p, r, o, tu in zip(plans, runs, outs, tuned):
            p.set_variant(4)
            p.rhs(r["q"], o)
            tc_err[f"{r['eq']}{r['order']}"] = float(
                torch.linalg.norm(o - r["out"]) / torch.linalg.norm(r["out"]))
            p.set_variant(tu["chosen"])
        out["mixed_precision_sweep"]["tcgen05_variant_rel_l2_err_vs_fp64"] = tc_err
        del outs
    except Exception as exc:  # report, keep the main line
        out["mixed_precision_sweep"] = {"error": repr(exc)}
    # }}}
    # {{{ FP64 with the contractions emulated on tcgen05 (orders 3 and 4)
    try:
        stream = torch.cuda.current_stream()
        rows = {}
        sel = [(k, r) for k, r in enumerate(runs) if r["order"] >= 3]
        for k, r in sel:
            op = r["compiled"].op
            op.precision = "fp64-tc"
            p = op.plan_for(actx)
            op.precision = "fp64"
            o = torch.empty_like(r["q"])
            for _ in range(2):
                p.rhs(r["q"], o)
            e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
            e0.record(stream)
            for _ in range(K):
                p.rhs(r["q"], o)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / K
            rows[f"{r['eq']}{r['order']}"] = {
                "ms": ms, "fp64_fma_ms": fp64_case_ms[k],
                "speedup_vs_fp64_fma": fp64_case_ms[k] / ms,
                "rel_l2_err_vs_fp64": float(torch.linalg.norm(o - r["out"])
                                            / torch.linalg.norm(r["out"]))}
            del p, o
        dofs = sum(r["cost"].dofs for _, r in sel)
        tot = sum(v["ms"] for v in rows.values())
        out["fp64_tcgen05_emulation"] = {
            "value": dofs / (tot * 1e-3), "unit": UNIT, "ms_per_step": tot,
            "fp64_fma_ms_per_step": sum(fp64_case_ms[k] for k, _ in sel),
            "max_rel_l2_err_vs_fp64": max(v["rel_l2_err_vs_fp64"] for v in rows.values()),
            "cases": rows}
    except Exception as exc:
        out["fp64_tcgen05_emulation"] = {"error": repr(exc)}
    torch.cuda.empty_cache()
    # }}}
    # {{{ DOF-throughput sweep of the wave operator (the reference's
    # wave_dof_scaling: P1-P4, 1-27 M DOFs per field)
    try:
        from actx_dgfem_suite_gb300.tools.wave_dof_scaling import GB300_NDOFS, sweep
        t0 = time.perf_counter()
        res = sweep((1, 2, 3, 4), GB300_NDOFS, "fp64", device_setup=True, events=True)
        out["wave_dof_scaling"] = {
            "unit": "G DOF-updates/s (4 fields)", "problem": "reference wave definition",
            "ndofs_per_field": list(GB300_NDOFS),
            "gdof_s": {f"P{d}": [res[(d, n)] * 1e-9 for n in GB300_NDOFS]
                       for d in (1, 2, 3, 4)},
            "timing": "3 warm-up + 10 timed RHS per point, CUDA events",
            "wall_s": time.perf_counter() - t0}
    except Exception as exc:
        out["wave_dof_scaling"] = {"error": repr(exc)}
    torch.cuda.empty_cache()
    # }}}
    for name, mod, kw in (
            ("mixed_precision_euler_p3_lsrk45", "bench_mixed", {}),
            ("ensemble_maxwell_p3_64", "bench_ensemble", {"reps": 5}),
            ("adjoint_wave_p3", "bench_adjoint", {}),
            ("adjoint_euler_p3", "bench_adjoint", {"_fn": "run_euler"})):
        try:
            import importlib
            m = importlib.import_module(f"actx_dgfem_suite_gb300.tools.{mod}")
            kw = dict(kw)
            fn = getattr(m, kw.pop("_fn", "run"))
            res = fn(**kw)
            res.pop("err_per_step", None)
            res.pop("member_sizes", None)
            out[name] = res
        except Exception as exc:
            out[name] = {"error": repr(exc)}
        torch.cuda.empty_cache()
    return out


def our_arm(args) -> None:
    import numpy as np
    import torch
    import torch.distributed as dist

    from actx_dgfem_suite_gb300 import hostmem
    from actx_dgfem_suite_gb300 import perf_model as pm
    from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext
    from actx_dgfem_suite_gb300.containers import leaves
    from actx_dgfem_suite_gb300.discretization import clear_box_cache
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs

    rank, world, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    actx = GB300DGArrayContext(f"cuda:{local}")
    dev = actx.device

    cases = CASES if not args.cases else [c for c in CASES
                                          if f"{c[0]}{c[1]}" in args.cases.split(",")]
    # {{{ setup through the public API (host mesh/geometry/IC, then upload)
    t_setup = time.perf_counter()
    runs = []
    for (eq, order, n) in cases:
        n_eff = max(2, n // args.scale)
        rhs, call_args = get_rhs(eq, actx, 3, order, definition="baseline",
                                 nel_1d=n_eff, device_setup=not args.host_setup)
        rhs.dg_operator.precision = args.precision
        compiled = actx.compile(rhs)
        state = call_args[-1]
        q = compiled.stage(state)
        out = torch.empty_like(q)
        nel = rhs.dg_operator.disc.nelements
        runs.append(dict(eq=eq, order=order, n=n_eff, compiled=compiled,
                         call_args=call_args, q=q, out=out,
                         cost=pm.RhsCost(eq, order, nel,
                                         boundary_faces=12 * n_eff * n_eff)))
        if hasattr(rhs.dg_operator.disc, "_cache"):
            rhs.dg_operator.disc._cache.clear()
    clear_box_cache()
    setup_s = time.perf_counter() - t_setup
    # }}}

    fp64_peak = fp64_peak_tflops(torch)
    stream = torch.cuda.current_stream()
    # launch variant per case (persistent grid or one CTA per tile), picked by
    # the library's autotuner on the case's own state, outside the timed region
    tuned = {f"{r['eq']}{r['order']}": r["compiled"].plan.autotune(r["q"], reps=2)
             for r in runs}

    def step(record=None):
        for k, r in enumerate(runs):
            if record is not None:
                record[k][0].record(stream)
            r["compiled"].plan.rhs(r["q"], r["out"])
            if record is not None:
                record[k][1].record(stream)

    for _ in range(args.warmup):
        step()
    for r in runs:
        r["compiled"].plan.finish()

    K = args.steps
    events = [[(torch.cuda.Event(True), torch.cuda.Event(True)) for _ in runs]
              for _ in range(K)]
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t_all0 = torch.cuda.Event(True)
    t_all1 = torch.cuda.Event(True)
    t_all0.record(stream)
    for s in range(K):
        step(events[s])
    t_all1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clock_info = clocks.stop()
    for r in runs:
        r["compiled"].plan.finish()   # raises on any device-side error flag
    total_ms = t_all0.elapsed_time(t_all1)
    case_ms = [statistics.mean(events[s][k][0].elapsed_time(events[s][k][1])
                               for s in range(K)) for k in range(len(runs))]
    ms_step = max_over_ranks(total_ms / K, dev)
    dofs_step = sum(r["cost"].dofs for r in runs)
    value = replica_rate(dofs_step, ms_step * 1e-3, world)
    flops_step = sum(r["cost"].flops for r in runs)

    # {{{ e2e through the public API with host buffers
    host_states = []
    for r in runs:
        hq = actx.pinned_host_like(r["q"])
        hq.copy_(r["q"])
        tmpl = r["call_args"][-1]
        from actx_dgfem_suite_gb300.containers import from_stacked
        hs = from_stacked(actx, tmpl, hq)
        host_states.append(r["call_args"][:-1] + (hs,))
    h2d = sum(r["q"].numel() * 8 for r in runs)
    d2h = h2d

    # calls in descending kernel time per input byte (highest order first), so
    # that the uploads of the cheap, copy-heavy low-order cases run behind the
    # long kernels: the step then tolerates a host link slowed by other
    # traffic on the shared host (every case is still evaluated once per step)
    order = sorted(range(len(runs)),
                   key=lambda k: -case_ms[k] / (runs[k]["q"].numel() * 8))

    klog: list = []          # kernel-end events of a logged step
    logging = [False]

    def e2e_step():
        # every case's call first (host->device copies on the context's copy
        # stream overlap the kernels of earlier cases), then every result back
        outs = []
        for k in order:
            outs.append(runs[k]["compiled"](*host_states[k]))
            if logging[0]:   # when the step is logged: end of its kernel
                ev = torch.cuda.Event(enable_timing=True)
                ev.record(torch.cuda.current_stream())
                klog.append(ev)
        # read back in the same order, each copy behind its own kernel, with
        # one wait at the end
        host = dict(zip(order, actx.to_numpy_batch(outs)))
        return [host[k] for k in range(len(runs))]

    # warm-up with the timed loop's lifetimes (the previous step's host
    # results stay alive while the next step runs), so the page-locked
    # result blocks the timed steps use are already in the host cache
    host_out = None
    for _ in range(max(3, min(args.warmup, 4))):
        host_out = e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ke = max(1, min(K, 5))
    e2e_step_ms = []
    t0 = time.perf_counter()
    for _ in range(ke):
        ts = time.perf_counter()
        host_out = e2e_step()   # ends in a synchronous device->host copy
        e2e_step_ms.append((time.perf_counter() - ts) * 1e3)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / ke, dev)
    # where the time goes: the same number of steps again with the transfer
    # log on (copy busy times and rates, span, end of the last kernel), beside
    # the kernels' time (the device-resident step above); `split_ms` is the
    # logged step of median wall time
    keep = [host_out]
    host_out = None

    def logged_step():   # the timed loop's lifetimes: the previous results live on
        keep[0] = e2e_step()

    logging[0] = True
    logged = [transfer_split(actx, logged_step, klog) for _ in range(ke)]
    logging[0] = False
    host_out = keep[0]
    split = dict(sorted(logged, key=lambda r: r["wall"])[len(logged) // 2])
    split["compute"] = ms_step
    split["step"] = statistics.median(e2e_step_ms)
    # sanity: the host result equals the device-resident result
    ok = all(np.array_equal(np.stack([d[0] for d in leaves(h)]),
                            r["out"].cpu().numpy())
             for h, r in zip(host_out[:1], runs[:1]))
    e2e_value = replica_rate(dofs_step, e2e_s, world)
    del host_out
    # }}}

    # {{{ roofline of the dominant launch
    peaks = _peaks()
    dom = max(range(len(runs)), key=lambda k: case_ms[k])
    rd = runs[dom]
    c = rd["cost"]
    t_dom = case_ms[dom] * 1e-3
    achieved_gbs = c.bytes / t_dom / 1e9
    info = rd["compiled"].plan.info()
    path = "shared" if info["face_shared"] else "fused"
    if info["tensor_cores"]:
        path = "tc"
    traffic = _ncu_traffic(path).get(f"{rd['eq']}{rd['order']}")
    if traffic is not None and (args.scale != 1 or args.precision == "fp32-mixed"):
        traffic = None
    if info["tensor_cores"]:
        kname = f"dg_rhs_tc_kernel<{rd['order']}, {rd['eq']}, SPLIT>"
    else:
        kname = (f"dg_rhs_kernel<{rd['order']}, {rd['eq']}, "
                 f"{'float' if args.precision == 'fp32-mixed' else 'double'}, "
                 f"{'SPLIT' if info['face_shared'] else 'RHS'}>")
    if info["face_shared"]:
        kname = (f"dg_face_flux_kernel<{rd['order']}, {rd['eq']}>"
                 + (" + dg_euler_aux_kernel" if rd["eq"] == "euler" else "")
                 + " + " + kname + " (one RHS)")
    fp64_achieved = 2.0 * c.fma / t_dom / 1e12
    roofline = {
        "bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"],
        "unit": "GB/s", "frac": achieved_gbs / peaks["hbm_gbs"],
        "traffic": traffic,
        "kernel": kname,
        "peak_source": peaks["source"],
        "fp64_pipe": {"achieved_tflops": fp64_achieved,
                      "peak_tflops": fp64_peak,
                      "frac": fp64_achieved / fp64_peak,
                      "peak_source": "measured live (dg_fp64_fma_probe)"},
        "limiter": "fp64 pipe",
        "suite_model_frac": c.roofline_seconds(fp64_peak * 1e12,
                                               peaks["hbm_gbs"] * 1e9) / t_dom,
    }
    # }}}

    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu:
        dofs_c, wall, busy, cores, outs = run_oracle_sweep(args.cpu_scale, reps=1,
                                                           keep=True)
        cpu = {"value": dofs_c / (busy / cores), "unit": UNIT, "cores": cores,
               "kind": "port",
               "sample": (f"CPU FP64 oracle, every case at n // {args.cpu_scale}, "
                          f"one process per case")}
        parity = parity_vs_oracle(actx, args.cpu_scale, outs)

    extras = None
    if rank == 0 and world == 1 and not args.no_extras:
        extras = run_extras(args, runs, actx, K, ms_step, case_ms)

    per_case = [{"case": f"{r['eq']} P{r['order']} n={r['n']}",
                 "nel": r["cost"].nelements, "ms": case_ms[k],
                 "gdof_s": r["cost"].dofs / case_ms[k] / 1e6,
                 "gflops_suite": r["cost"].flops / case_ms[k] / 1e6,
                 "fp64_frac": 2 * r["cost"].fma / (case_ms[k] * 1e-3) / 1e12 / fp64_peak,
                 "hbm_frac": r["cost"].bytes / (case_ms[k] * 1e-3) / 1e9 / peaks["hbm_gbs"]}
                for k, r in enumerate(runs)]
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": K, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 state)" if args.precision == "fp32-mixed" else "f64",
            "data": "synthetic",
            "config": bench_config(args, world),
            "gflops_suite": world * flops_step / (ms_step * 1e-3) / 1e9,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "host_matches_device": bool(ok),
                    "step_ms": [round(x, 1) for x in e2e_step_ms],
                    "split_ms": {k: (round(v, 2) if v is not None else None)
                                 for k, v in split.items()},
                    "logged_steps": [{k: (round(v, 1) if v is not None else None)
                                      for k, v in r.items()} for r in logged],
                    # page-locked host buffers: on huge pages, or from
                    # cudaHostAlloc where the host granted no huge pages
                    "host_state_buffers": dict(hostmem.stats),
                    "overlap": ("all cases' calls issued before their results are read "
                                "(highest kernel time per input byte first), then every "
                                "result's copy back in the same order (to_numpy_batch, "
                                "one wait): copies run on the context's copy streams "
                                "beside the kernels")},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "parity": parity,
            "clocks": clock_info,
            "gpu_launches": K * sum(r["compiled"].plan.launches_per_rhs for r in runs),
            "autotuned_variant": {k: v["chosen"] for k, v in tuned.items()},
            "setup_s": setup_s,
            "cases": per_case,
            "extras": extras,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--scale", type=int, default=1,
                    help="divide every n by this (quick runs; 1 = benchmark sizes)")
    ap.add_argument("--cpu-scale", type=int, default=4,
                    help="CPU sample: every case at n // cpu-scale")
    ap.add_argument("--cases", default="", help="subset, e.g. wave3,euler4")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the mixed-precision, ensemble and adjoint extras")
    ap.add_argument("--host-setup", action="store_true",
                    help="build meshes on the host (NumPy) instead of on the GPU")
    ap.add_argument("--precision", default="fp64", choices=("fp64", "fp64-tc", "fp32-mixed"),
                    help="arithmetic of the timed RHS (the benchmark metric is fp64)")
    args = ap.parse_args(argv)
    if args.impl == "reference":
        reference_arm(args)
    else:
        our_arm(args)


if __name__ == "__main__":
    main()

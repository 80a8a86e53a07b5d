"""Timing harness, mirroring ``actx_dgfem_suite/run/__main__.py``.

``python -m actx_dgfem_suite_gb300.run --equations wave,euler --dims 3
--degrees 1,2,3,4 --actxs cuda:gb300`` prints GFLOP/s tables (suite FLOP
count) per equation, one column per array context plus the roofline column.
The warm-up (<= 5 calls or 2 s) and timing (batches of 3 calls until >= 50
calls or 4 s) loops follow ``run/__main__.py:101-132``; the rate is
``flops * calls / time`` (``run/__main__.py:134-135``).

Verification against another array context (``run/__main__.py:77-96``) is
not done here: this package ships one array context, and its results are
checked against the CPU oracle by the test suite.
"""

from __future__ import annotations

import argparse
import dataclasses as dc
import gc
from collections.abc import Sequence
from time import time

from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext
from actx_dgfem_suite_gb300.measure import finish_command_queue, instantiate_actx_t
from actx_dgfem_suite_gb300.perf_model import RhsCost
from actx_dgfem_suite_gb300.rhs_builder import get_rhs


class _BiDict(dict):
    """A name -> class map with the inverse lookup ``.inv`` (bidict-like)."""

    @property
    def inv(self) -> dict:
        return {v: k for k, v in self.items()}


#: array-context registry; the reference's is ``run/__main__.py:209-216``
_NAME_TO_ACTX_CLASS = _BiDict({
    "cuda:gb300": GB300DGArrayContext,
})


def register_actx(name: str, actx_t: type) -> None:
    """Add an array context type under a unique name."""
    if name in _NAME_TO_ACTX_CLASS or actx_t in _NAME_TO_ACTX_CLASS.values():
        raise ValueError(f"{name!r} or {actx_t} already registered")
    _NAME_TO_ACTX_CLASS[name] = actx_t


def _boundary_faces(disc) -> int:
    bd = getattr(disc, "is_boundary", None)
    if bd is None:          # a mesh built on the device keeps no host mask:
        return 0            # the wave boundary term (1 per boundary point) is left out
    return int(bd.sum()) if hasattr(bd, "sum") else 0


def _flops(equation: str, dim: int, degree: int, rhs) -> int:
    base = equation.split("_", 1)[-1] if equation.startswith(("tiny_", "large_")) \
        else equation
    disc = rhs.dg_operator.disc
    return RhsCost(base, degree, disc.nelements, dim,
                   boundary_faces=_boundary_faces(disc)).flops


def peak_flop_rate(equation: str, dim: int, degree: int, nelements: int,
                   peak_flops: float, peak_bw: float) -> float:
    """Roofline rate ``F / max(F/peakF, B/peakBW)`` (``perf_analysis.py:624-653``)."""
    base = equation.split("_", 1)[-1] if equation.startswith(("tiny_", "large_")) \
        else equation
    c = RhsCost(base, degree, nelements, dim)
    return c.flops / c.roofline_seconds(peak_flops, peak_bw)


def get_flop_rate(actx_t, equation: str, dim: int, degree: int,
                  definition: str = "reference") -> tuple[float, int]:
    actx = instantiate_actx_t(actx_t)
    rhs, args = get_rhs(equation, actx, dim, degree, definition=definition)
    compiled_rhs = actx.compile(rhs)
    compiled_rhs(*args)

    i_warmup, t_warmup = 0, 0.0
    while i_warmup < 5 and t_warmup < 2:
        finish_command_queue(actx)
        t_start = time()
        compiled_rhs(*args)
        finish_command_queue(actx)
        t_warmup += time() - t_start
        i_warmup += 1

    i_timing, t_rhs = 0, 0.0
    while i_timing < 50 and t_rhs < 4:
        finish_command_queue(actx)
        t_start = time()
        for _ in range(3):
            compiled_rhs(*args)
        finish_command_queue(actx)
        t_rhs += time() - t_start
        i_timing += 3

    nel = rhs.dg_operator.disc.nelements
    return _flops(equation, dim, degree, rhs) * i_timing / t_rhs, nel


def _fmt(flops: float) -> str:
    return "N/A" if flops != flops else f"{flops * 1e-9:.1f}"


def _table(rows: list[list[str]]) -> str:
    widths = [max(len(r[k]) for r in rows) for k in range(len(rows[0]))]
    line = "+" + "+".join("-" * (w + 2) for w in widths) + "+"
    out = [line]
    for r in rows:
        out.append("| " + " | ".join(c.rjust(w) for c, w in zip(r, widths)) + " |")
        out.append(line)
    return "\n".join(out)


def main(equations: Sequence[str], dims: Sequence[int], degrees: Sequence[int],
         actx_ts: Sequence[type], definition: str = "reference",
         peak_flops: float | None = None, peak_bw: float | None = None) -> dict:
    from actx_dgfem_suite_gb300.consts import (DEV_TO_PEAK_BW,
                                               DEV_TO_PEAK_F64_GFLOPS)
    results = {}
    nels = {}
    for actx_t in actx_ts:
        for dim in dims:
            for eq in equations:
                for deg in degrees:
                    rate, nel = get_flop_rate(actx_t, eq, dim, deg, definition)
                    results[(actx_t, dim, eq, deg)] = rate
                    nels[(dim, eq, deg)] = nel
                    gc.collect()
    pf = peak_flops or DEV_TO_PEAK_F64_GFLOPS["NVIDIA GB300"] * 1e9
    pb = peak_bw or DEV_TO_PEAK_BW["NVIDIA GB300"] * 1e9
    names = _NAME_TO_ACTX_CLASS.inv
    for dim in dims:
        for eq in equations:
            print(f"GFLOPS/s for {dim}D-{eq}:")
            rows = [["", *[names.get(t, t.__name__) for t in actx_ts], "Roofline"]]
            for deg in degrees:
                rows.append([f"P{deg}",
                             *[_fmt(results[(t, dim, eq, deg)]) for t in actx_ts],
                             _fmt(peak_flop_rate(eq, dim, deg, nels[(dim, eq, deg)],
                                                 pf, pb))])
            print(_table(rows))
    return results


@dc.dataclass(frozen=True)
class CLIArgs:
    equations: str
    dims: str
    degrees: str
    actxs: str
    definition: str


def cli(argv=None):
    parser = argparse.ArgumentParser(
        prog="python -m actx_dgfem_suite_gb300.run",
        description="Run DG-FEM RHS benchmarks for array contexts")
    parser.add_argument("--equations", required=True,
                        help="comma separated, e.g. 'wave,euler,maxwell'; prefix "
                             "'tiny_' (1K DOFs/field) or 'large_' (20M)")
    parser.add_argument("--dims", required=True, help="comma separated, e.g. 3")
    parser.add_argument("--degrees", required=True, help="e.g. 1,2,3,4")
    parser.add_argument("--actxs", default="cuda:gb300")
    parser.add_argument("--definition", default="reference",
                        choices=("reference", "baseline"))
    parser.add_argument("--no-verify", action="store_true",
                        help="accepted for compatibility; see module docstring")
    a = parser.parse_args(argv)
    return main(equations=[k.strip() for k in a.equations.split(",")],
                dims=[int(k) for k in a.dims.split(",")],
                degrees=[int(k) for k in a.degrees.split(",")],
                actx_ts=[_NAME_TO_ACTX_CLASS[k.strip()] for k in a.actxs.split(",")],
                definition=a.definition)


if __name__ == "__main__":
    cli()

"""FLOP count and roofline tables, mirroring
``actx_dgfem_suite/tools/print_ngflops.py`` and ``print_roofline.py``.

``python -m actx_dgfem_suite_gb300.tools.print_roofline --equations wave,euler
--dims 2,3 --degrees 1,2,3,4 [--peak-gflops G --peak-gbs B]`` prints, per
dimension, equation and degree, the suite-rule GFLOP count of one RHS, the
algorithmic bytes, and the roofline rate ``F / max(F/peakF, B/peakBW)``
(``perf_analysis.py:624-653``).  No GPU is needed.
"""

from __future__ import annotations

import argparse

from actx_dgfem_suite_gb300.consts import DEV_TO_PEAK_BW, DEV_TO_PEAK_F64_GFLOPS
from actx_dgfem_suite_gb300.perf_model import RhsCost
from actx_dgfem_suite_gb300.rhs_builder import split_equation_name
from actx_dgfem_suite_gb300.utils import get_nel_1d_for_regular_rect_mesh


def table(equations, degrees, peak_gflops: float, peak_gbs: float, dims=(3,)):
    rows = []
    for dim in dims:
        for eq in equations:
            base, ndofs = split_equation_name(eq)
            for d in degrees:
                n = get_nel_1d_for_regular_rect_mesh(dim, d, ndofs)
                nel = 6 * n**3 if dim == 3 else 2 * n**2
                bfaces = 12 * n**2 if dim == 3 else 4 * n
                c = RhsCost(base, d, nel, dim, boundary_faces=bfaces)
                t = c.roofline_seconds(peak_gflops * 1e9, peak_gbs * 1e9)
                rows.append((dim, eq, d, n, c.flops / 1e9, c.bytes / 1e9,
                             c.flops / t / 1e9))
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m actx_dgfem_suite_gb300.tools.print_roofline")
    ap.add_argument("--equations", default="wave,euler,maxwell")
    ap.add_argument("--degrees", default="1,2,3,4")
    ap.add_argument("--dims", default="3", help="comma separated, e.g. 2,3")
    ap.add_argument("--peak-gflops", type=float,
                    default=DEV_TO_PEAK_F64_GFLOPS["NVIDIA GB300"])
    ap.add_argument("--peak-gbs", type=float, default=DEV_TO_PEAK_BW["NVIDIA GB300"])
    a = ap.parse_args(argv)
    rows = table([e.strip() for e in a.equations.split(",")],
                 [int(x) for x in a.degrees.split(",")], a.peak_gflops, a.peak_gbs,
                 dims=[int(x) for x in a.dims.split(",")])
    print(f"{'dim':>3} {'equation':<16}{'P':>3}{'n':>6}{'GFLOP':>10}{'GB':>9}"
          f"{'roofline GFLOP/s':>19}")
    for dim, eq, d, n, gf, gb, rate in rows:
        print(f"{dim:>3} {eq:<16}{d:>3}{n:>6}{gf:>10.2f}{gb:>9.3f}{rate:>19.1f}")
    return rows


if __name__ == "__main__":
    main()

"""Golden vectors from the reference's own importable modules.

``actx_dgfem_suite/utils.py`` (the DOF budget -> elements per axis helpers
behind ``get_rhs``) and ``actx_dgfem_suite/consts.py`` (the roofline's device
peak table) import nothing outside the standard library, so the reference
itself can be run here; the DOF budgets of ``rhs_builder.py`` (a module that
needs the reference's numeric stack) are read from its source text.  This script imports them from a checkout of the
reference and records their outputs over a grid of arguments in
``reference_utils.json``; ``tests/test_reference_utils.py`` checks the
package's helpers against that file (the reference cannot travel with the
tests, the file does).

Usage, from the repository root, with the reference checked out at
``$REF`` (default ``/root/reference``)::

    python tests/golden/make_reference_utils.py
"""

from __future__ import annotations

import json
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent

#: DOF budgets: the suite's tiny/full/large budgets, the DOF-scaling sweep's
#: sizes, and values around them
NDOFS = sorted({10**3, 4 * 10**6, 2 * 10**7, 1_000_000, 5_000_000, 10_000_000,
                15_000_000, 20_000_000, 25_000_000, 27_000_000}
               | {int(1.37**k) for k in range(10, 60, 3)})
NEL_1D = list(range(1, 13)) + [20, 33, 46, 56, 70, 95]


def main() -> None:
    ref = os.environ.get("REF", "/root/reference")
    sys.path.insert(0, ref)
    from actx_dgfem_suite import consts, utils
    nel = [[dim, order, n, utils.get_nel_1d_for_regular_rect_mesh(dim, order, n)]
           for dim in (2, 3) for order in (1, 2, 3, 4) for n in NDOFS]
    ndof = [[dim, order, k, utils.get_ndof_for_regular_rect_mesh(dim, order, k)]
            for dim in (2, 3) for order in (1, 2, 3, 4) for k in NEL_1D]
    # rhs_builder.py imports the reference's numeric stack at module level;
    # its DOF budgets are read from the source text instead
    import ast
    tree = ast.parse((Path(ref) / "actx_dgfem_suite" / "rhs_builder.py").read_text())
    budgets = {node.targets[0].id: ast.literal_eval(node.value)
               for node in tree.body
               if isinstance(node, ast.Assign) and len(node.targets) == 1
               and isinstance(node.targets[0], ast.Name)
               and node.targets[0].id.startswith("_NDOFS_")}
    out = {"source": "actx_dgfem_suite/utils.py:15-74, actx_dgfem_suite/consts.py:1-12, "
                     "actx_dgfem_suite/rhs_builder.py:9-11",
           "get_nel_1d_for_regular_rect_mesh": nel,
           "get_ndof_for_regular_rect_mesh": ndof,
           "DEV_TO_PEAK_F64_GFLOPS": consts.DEV_TO_PEAK_F64_GFLOPS,
           "DEV_TO_PEAK_BW": consts.DEV_TO_PEAK_BW,
           "rhs_builder_budgets": budgets}
    (HERE / "reference_utils.json").write_text(json.dumps(out) + "\n")


if __name__ == "__main__":
    main()

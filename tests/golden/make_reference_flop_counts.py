"""Pointwise operation counts of the reference's own wave operator.

Imports ``actx_dgfem_suite/equations/wave.py`` from a checkout of the
reference on the stand-in modules of ``tests/golden/reference_stubs.py`` and
runs ``wave_operator`` (``wave.py:121-200``, with ``wave_flux`` at
``wave.py:80-114``) with operation counting on: every +, -, *, / (and
unary minus) on DOF arrays adds its output size, the rule by which the
reference counts the pointwise nodes of its DAG
(``actx_dgfem_suite/perf_analysis.py:250-377``).  The counts are recorded per
volume node and per face point of each domain -- the boundary trace pair
(``BTAG_ALL``), the interior trace pairs (``int_faces``) and the all-faces
fluxes -- in ``reference_wave_flops.json``; ``perf_model`` takes the wave
equation's pointwise count from them (``tests/test_perf_model.py`` checks).

The einsums (weak derivatives, face mass, inverse mass) are not in these
counts: the stand-ins evaluate them with the oracle, and the FLOP model
counts them by the einsum rule.  What the counts cannot see is what the
reference's DAG transformations (common-subexpression merging, constant
folding) do to the pointwise nodes.

Usage, from the repository root, with the reference checked out at ``$REF``
(default ``/root/reference``)::

    python tests/golden/make_reference_flop_counts.py
"""

from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))


def main() -> None:
    from tests.golden import reference_stubs as rs
    rs.install()
    sys.path.insert(0, os.environ.get("REF", "/root/reference"))
    from actx_dgfem_suite.equations import wave as ref_wave

    from actx_dgfem_suite_gb300.mesh import generate_box_tet_mesh, generate_box_tri_mesh
    from oracle.geometry import build_oracle_disc, build_oracle_disc_2d

    actx = rs.StubActx()
    out = {"mesh": "box, 2 hexahedra per axis (48 tetrahedra)", "orders": {},
           "mesh_2d": "square, 2 squares per axis (8 triangles)", "orders_2d": {}}
    for dim, build, mesh, key in (
            (3, build_oracle_disc, generate_box_tet_mesh(0.0, 1.0, 2), "orders"),
            (2, build_oracle_disc_2d, generate_box_tri_mesh(0.0, 1.0, 2), "orders_2d")):
        for order in (1, 2, 3, 4):
            d = build(mesh.vertices, mesh.elements, order)
            dcoll = rs.StubDcoll(d, actx)
            rng = np.random.default_rng(order)
            shape = d.nodes.shape[1:]
            w = ref_wave.WaveState(u=rs.DOF(rng.standard_normal(shape)),
                                   v=rs.objarr([rs.DOF(rng.standard_normal(shape))
                                                for _ in range(dim)]))
            with rs.counting() as counts:
                ref_wave.wave_operator(actx, dcoll, c=1, w=w, quad_tag=None)
            nvol = d.nel * d.nodes.shape[2]
            nface = d.int_idx.size      # the stand-ins keep every face array full size
            out[key][str(order)] = {
                "per_node": counts.get("vol", 0) / nvol,
                "per_boundary_face_point": counts.get("bdry", 0) / nface,
                "per_interior_face_point": counts.get("int", 0) / nface,
                "per_all_faces_point": counts.get("all", 0) / nface,
            }
    (HERE / "reference_wave_flops.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()

"""Golden vectors from the reference's own equation code.

Imports ``actx_dgfem_suite/equations/wave.py`` and ``euler.py`` from a
checkout of the reference, on the stand-in modules of
``tests/golden/reference_stubs.py`` (the reference's numeric stack is absent
here), and records in ``reference_equations.npz``:

* the initial states of the reference's problem definitions at the oracle's
  node coordinates of a box mesh: ``bump`` (``wave.py:216-236``) and
  ``acoustic_pulse_condition`` (``euler.py:119-137``);
* the RHS of ``wave_operator`` (``wave.py:121-200``, with its ``wave_flux``
  and boundary pair) for a seeded random state on a jittered mesh, with the
  oracle's grudge primitives underneath, at orders 1-4.

``tests/test_reference_equations.py`` checks the package's initial states,
the oracle's restated wave operator and (on a GPU) the product against them.

``--dim 2`` writes ``reference_equations_2d.npz`` instead: the same records
on triangle meshes (the reference's ``wave.py`` is dimension-generic: the
bump's centre is its first ``dim`` entries, v has ``dim`` components).

Usage, from the repository root, with the reference checked out at ``$REF``
(default ``/root/reference``)::

    python tests/golden/make_reference_equations.py
"""

from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

#: jittered box mesh of the wave-operator cases (elements per axis)
WAVE_MESH_N = 2
#: box mesh of the initial-state cases: reference definition, [-0.5, 0.5]^3
IC_MESH_N, IC_ORDER = 3, 3


def main() -> None:
    from tests.golden import reference_stubs as rs
    rs.install()
    sys.path.insert(0, os.environ.get("REF", "/root/reference"))
    from actx_dgfem_suite.equations import euler as ref_euler
    from actx_dgfem_suite.equations import wave as ref_wave

    from actx_dgfem_suite_gb300.mesh import generate_box_tet_mesh
    from oracle.geometry import build_oracle_disc
    from tests._helpers import jittered_box_mesh

    out = {}
    actx = rs.StubActx()

    # {{{ initial states of the reference definitions
    mesh = generate_box_tet_mesh(-0.5, 0.5, IC_MESH_N)
    d = build_oracle_disc(mesh.vertices, mesh.elements, IC_ORDER)
    dcoll = rs.StubDcoll(d, actx)
    out["ic_vertices"] = mesh.vertices
    out["ic_elements"] = mesh.elements
    out["ic_nodes"] = d.nodes
    out["ic_wave_u"] = ref_wave.bump(actx, dcoll).a
    q = ref_euler.acoustic_pulse_condition(dcoll.nodes())
    out["ic_euler"] = np.stack([q.mass.a, q.energy.a]
                               + [np.broadcast_to(m.a, q.mass.a.shape) for m in q.momentum])
    # }}}

    # {{{ wave operator on a jittered mesh, random state
    mesh = jittered_box_mesh(WAVE_MESH_N)
    out["wave_vertices"] = mesh.vertices
    out["wave_elements"] = mesh.elements
    rng = np.random.default_rng(0)
    for order in (1, 2, 3, 4):
        d = build_oracle_disc(mesh.vertices, mesh.elements, order)
        dcoll = rs.StubDcoll(d, actx)
        shape = d.nodes.shape[1:]
        u = rng.standard_normal(shape)
        v = rng.standard_normal((3,) + shape)
        w = ref_wave.WaveState(u=rs.DOF(u), v=rs.objarr([rs.DOF(v[x]) for x in range(3)]))
        r = ref_wave.wave_operator(actx, dcoll, c=1, w=w, quad_tag=None)
        out[f"wave_P{order}_state"] = np.concatenate([u[None], v])
        out[f"wave_P{order}_rhs"] = np.stack([r.u.a] + [r.v[x].a for x in range(3)])
    # }}}

    np.savez_compressed(HERE / "reference_equations.npz", **out)


def main_2d() -> None:
    from tests.golden import reference_stubs as rs
    rs.install()
    sys.path.insert(0, os.environ.get("REF", "/root/reference"))
    from actx_dgfem_suite.equations import euler as ref_euler
    from actx_dgfem_suite.equations import wave as ref_wave

    from actx_dgfem_suite_gb300.mesh import generate_box_tri_mesh
    from oracle.geometry import build_oracle_disc_2d
    from tests._helpers import jittered_square_mesh

    out = {}
    actx = rs.StubActx()
    mesh = generate_box_tri_mesh(-0.5, 0.5, 4)      # reference definition's square
    d = build_oracle_disc_2d(mesh.vertices, mesh.elements, IC_ORDER)
    dcoll = rs.StubDcoll(d, actx)
    out["ic_vertices"] = mesh.vertices
    out["ic_elements"] = mesh.elements
    out["ic_nodes"] = d.nodes
    out["ic_wave_u"] = ref_wave.bump(actx, dcoll).a
    q = ref_euler.acoustic_pulse_condition(dcoll.nodes())
    out["ic_euler"] = np.stack([q.mass.a, q.energy.a]
                               + [np.broadcast_to(m.a, q.mass.a.shape) for m in q.momentum])

    mesh = jittered_square_mesh(3)
    out["wave_vertices"] = mesh.vertices
    out["wave_elements"] = mesh.elements
    rng = np.random.default_rng(0)
    for order in (1, 2, 3, 4):
        d = build_oracle_disc_2d(mesh.vertices, mesh.elements, order)
        dcoll = rs.StubDcoll(d, actx)
        shape = d.nodes.shape[1:]
        u = rng.standard_normal(shape)
        v = rng.standard_normal((2,) + shape)
        w = ref_wave.WaveState(u=rs.DOF(u), v=rs.objarr([rs.DOF(v[x]) for x in range(2)]))
        r = ref_wave.wave_operator(actx, dcoll, c=1, w=w, quad_tag=None)
        out[f"wave_P{order}_state"] = np.concatenate([u[None], v])
        out[f"wave_P{order}_rhs"] = np.stack([r.u.a] + [r.v[x].a for x in range(2)])
    np.savez_compressed(HERE / "reference_equations_2d.npz", **out)


if __name__ == "__main__":
    main_2d() if "--dim" in sys.argv and sys.argv[-1] == "2" else main()

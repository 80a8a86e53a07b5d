"""The DOF-budget helpers and the roofline's device table against golden
vectors recorded from the reference's own modules
(``tests/golden/make_reference_utils.py`` imports
``actx_dgfem_suite/utils.py`` and ``consts.py``, which need nothing outside
the standard library)."""

from __future__ import annotations

import json
from pathlib import Path

from actx_dgfem_suite_gb300 import consts, utils

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" /
                     "reference_utils.json").read_text())


def test_nel_1d_matches_the_reference():
    rows = GOLDEN["get_nel_1d_for_regular_rect_mesh"]
    assert len(rows) > 100
    for dim, order, ndofs, want in rows:
        assert utils.get_nel_1d_for_regular_rect_mesh(dim, order, ndofs) == want, \
            (dim, order, ndofs)


def test_ndof_matches_the_reference_except_its_p1_factor():
    """Equal everywhere but 3D P1, where the reference multiplies the element
    count by 6 instead of Np = 4 (``utils.py:50``); the helper here returns
    Nel * Np, i.e. 4/6 of the reference's number."""
    rows = GOLDEN["get_ndof_for_regular_rect_mesh"]
    for dim, order, nel_1d, want in rows:
        got = utils.get_ndof_for_regular_rect_mesh(dim, order, nel_1d)
        if dim == 3 and order == 1:
            assert got * 6 == want * 4, nel_1d
        else:
            assert got == want, (dim, order, nel_1d)


def test_device_table_extends_the_reference():
    for name, ref in (("DEV_TO_PEAK_F64_GFLOPS", consts.DEV_TO_PEAK_F64_GFLOPS),
                      ("DEV_TO_PEAK_BW", consts.DEV_TO_PEAK_BW)):
        for dev, val in GOLDEN[name].items():
            assert ref[dev] == val, (name, dev)


def test_dof_budgets_and_benchmark_sizes():
    """The suite's tiny / full / large DOF budgets, and the elements per axis
    they give per order (the large sizes are the benchmark's n = 95/70/56/46)."""
    from actx_dgfem_suite_gb300 import rhs_builder
    for name, val in GOLDEN["rhs_builder_budgets"].items():
        assert getattr(rhs_builder, name) == val, name
    large = GOLDEN["rhs_builder_budgets"]["_NDOFS_LARGE"]
    assert [utils.get_nel_1d_for_regular_rect_mesh(3, p, large)
            for p in (1, 2, 3, 4)] == [95, 70, 56, 46]

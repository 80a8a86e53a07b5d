"""The suite's CI invocation of its timing harness, on this array context:
``python -m actx_dgfem_suite.run --equations tiny_* --dims 2,3 --degrees
1,2,3,4`` (``.github/workflows/ci.yml:94-100``), here
``actx_dgfem_suite_gb300.run`` with the ``cuda:gb300`` context."""

from __future__ import annotations

import math

import pytest

pytestmark = pytest.mark.gpu


def test_ci_tiny_operators_dims_2_and_3(capsys):
    from actx_dgfem_suite_gb300.run import _NAME_TO_ACTX_CLASS, cli
    results = cli(["--equations", "tiny_euler,tiny_maxwell,tiny_wave",
                   "--dims", "2,3", "--degrees", "1,2,3,4", "--actxs", "cuda:gb300"])
    actx_t = _NAME_TO_ACTX_CLASS["cuda:gb300"]
    assert len(results) == 3 * 2 * 4
    for dim in (2, 3):
        for eq in ("tiny_euler", "tiny_maxwell", "tiny_wave"):
            for deg in (1, 2, 3, 4):
                rate = results[(actx_t, dim, eq, deg)]
                assert math.isfinite(rate) and rate > 0, (dim, eq, deg)
    out = capsys.readouterr().out
    for dim in (2, 3):
        for eq in ("tiny_euler", "tiny_maxwell", "tiny_wave"):
            assert f"GFLOPS/s for {dim}D-{eq}:" in out

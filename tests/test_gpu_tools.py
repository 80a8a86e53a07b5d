"""The DOF-throughput sweep tool (the reference's ``tools/wave_dof_scaling.py``
with its ``--dim``) on both dimensions, with small DOF budgets."""

from __future__ import annotations

import math

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim", [2, 3])
def test_wave_dof_scaling_sweep(dim):
    from actx_dgfem_suite_gb300.tools.wave_dof_scaling import sweep
    res = sweep([1, 3], [100_000, 400_000], dim=dim, events=True)
    assert set(res) == {(d, n) for d in (1, 3) for n in (100_000, 400_000)}
    assert all(math.isfinite(v) and v > 1e8 for v in res.values())

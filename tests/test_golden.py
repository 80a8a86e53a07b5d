"""Golden fixtures (oracle outputs for the reference problem definitions on
tiny meshes, see tests/golden/make_golden.py)."""

import numpy as np
import pytest

from tests._helpers import FP64_RTOL, parity_error
from tests.golden.make_golden import CASES, compute, fixture_path


@pytest.mark.parametrize("eq,order,n", CASES)
def test_oracle_reproduces_fixture(eq, order, n):
    fx = np.load(fixture_path(eq, order, n))
    prob, rhs, scale = compute(eq, order, n)
    assert np.isclose(np.linalg.norm(prob.fields), float(fx["input_l2"]), rtol=1e-14)
    assert parity_error(rhs, fx["rhs"], float(fx["scale"])) < 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("eq,order,n", CASES)
def test_gpu_matches_fixture(eq, order, n, actx):
    from actx_dgfem_suite_gb300.containers import leaves
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs
    fx = np.load(fixture_path(eq, order, n))
    rhs, args = get_rhs(eq, actx, 3, order, nel_1d=n)
    out = actx.to_numpy(actx.compile(rhs)(*args))
    got = np.stack([d[0] for d in leaves(out)])
    assert parity_error(got, fx["rhs"], float(fx["scale"])) <= FP64_RTOL

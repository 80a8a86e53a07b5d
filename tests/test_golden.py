"""Golden fixtures (oracle outputs for the reference problem definitions on
tiny meshes, see tests/golden/make_golden.py)."""

import numpy as np
import pytest

from tests._helpers import FP64_RTOL, parity_error, scaled_error
from tests.golden.make_golden import CASES, compute, fixture_path


@pytest.mark.parametrize("eq,order,n", CASES)
def test_oracle_reproduces_fixture(eq, order, n):
    fx = np.load(fixture_path(eq, order, n))
    prob, rhs, scale = compute(eq, order, n)
    assert np.isclose(np.linalg.norm(prob.fields), float(fx["input_l2"]), rtol=1e-14)
    # the fixtures were written by an earlier construction of the oracle's
    # matrices (FP64 quadrature over an orthonormal simplex basis); the
    # current extended-precision one agrees with it to round-off (<= 1.1e-14
    # of the volume and surface terms; relative to ||rhs|| the near-cancelling
    # Euler cases amplify that round-off)
    assert scaled_error(rhs, fx["rhs"], float(fx["scale"])) < 1e-13


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


@pytest.mark.gpu
def test_gpu_results_are_independent_host_arrays(actx):
    """to_numpy returns a new host array per call (page-locked by default,
    pageable with pinned_results=False), equal either way."""
    from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext
    from actx_dgfem_suite_gb300.containers import leaves
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs
    eq, order, n = CASES[0]
    rhs, args = get_rhs(eq, actx, 3, order, nel_1d=n)
    compiled = actx.compile(rhs)
    first = np.stack([d[0] for d in leaves(actx.to_numpy(compiled(*args)))])
    held = actx.to_numpy(compiled(*args))
    again = np.stack([d[0] for d in leaves(actx.to_numpy(compiled(*args)))])
    held_arr = np.stack([d[0] for d in leaves(held)])
    held_arr0 = held_arr.copy()
    leaves(held)[0][0][...] = 0.0          # writing one result leaves the others
    assert np.array_equal(first, again) and np.array_equal(first, held_arr0)
    plain = GB300DGArrayContext(actx.device, pinned_results=False)
    rhs2, args2 = get_rhs(eq, plain, 3, order, nel_1d=n)
    got = np.stack([d[0] for d in leaves(plain.to_numpy(plain.compile(rhs2)(*args2)))])
    assert np.array_equal(got, first)

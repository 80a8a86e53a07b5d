"""The allocation-free adjoint entry point, called through the C ABI.

``dg_rhs_adjoint_noalloc`` serves callers that may not allocate device memory
while they run (a host application that owns the whole memory budget, or a
latency-critical caller that cannot afford cudaMalloc's implicit
synchronisation): it works in a static 64 MiB device array instead of a
caller-supplied scratch buffer.  These tests check it against the allocating
entry point ``dg_rhs_adjoint`` on two calls in a row, and that meshes larger
than the static buffer are refused.  The file sorts last so that a run stopping
at the first failure has already run every other test.
"""

from __future__ import annotations

import ctypes

import pytest
import torch

from tests._helpers import jittered_box_mesh, make_problem

pytestmark = pytest.mark.gpu

#: same bound as the adjoint's dot-product test
RTOL = 1e-13


def _plan(disc):
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    return DevicePlan(DeviceMesh(disc, "cuda:0", with_partner=True), "wave", (1.3,))


def _noalloc(plan, x, y):
    from actx_dgfem_suite_gb300 import _lib
    L = _lib.lib()
    return L.dg_rhs_adjoint_noalloc(
        plan._handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_noalloc_adjoint_matches_allocating_entry_point():
    from actx_dgfem_suite_gb300 import _lib
    torch.cuda.set_device(0)
    prob = make_problem("wave", jittered_box_mesh(3), 3)
    plan = _plan(prob.disc)
    g = torch.Generator(device="cuda:0").manual_seed(11)
    c = 0.8 + 0.4 * torch.rand(prob.disc.nelements, dtype=torch.float64,
                               device="cuda:0", generator=g)
    plan.set_element_scale(c)
    for _ in range(2):  # two calls in a row, different inputs
        x = torch.randn(plan.shape, dtype=torch.float64, device="cuda:0", generator=g)
        ref = plan.adjoint(x)
        y = torch.full_like(x, float("nan"))
        assert _noalloc(plan, x, y) == _lib.DG_OK
        plan.finish()
        err = float(torch.linalg.norm(y - ref) / torch.linalg.norm(ref))
        assert err <= RTOL, err


def test_noalloc_adjoint_rejects_meshes_above_the_limit():
    from actx_dgfem_suite_gb300 import _lib
    from actx_dgfem_suite_gb300.discretization import make_box_discretization
    torch.cuda.set_device(0)
    disc = make_box_discretization(4, 23)          # 73,002 P4 elements > 69,905
    plan = _plan(disc)
    x = torch.zeros(plan.shape, dtype=torch.float64, device="cuda:0")
    y = torch.empty_like(x)
    assert _noalloc(plan, x, y) == _lib.DG_ERR_ARGUMENT
    assert b"static adjoint scratch" in _lib.lib().dg_last_error()

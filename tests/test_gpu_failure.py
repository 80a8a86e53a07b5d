"""Failure detection without a GPU fault: every device-side wait of the
kernels is bounded (1 s) and reports DG_ERR_TIMEOUT through a status word the
host reads.  Here a wait is made to run out (an mbarrier whose arrival never
comes); the status comes back and the context keeps working."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from tests._helpers import FP64_RTOL, oracle_rhs, parity_error

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives():
    from actx_dgfem_suite_gb300 import _lib
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    from actx_dgfem_suite_gb300.rhs_builder import get_problem
    L = _lib.lib()
    torch.cuda.set_device(0)
    status = ctypes.c_int32(-1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(L.dg_wait_probe(ctypes.byref(status), stream))
    assert status.value == _lib.DG_ERR_TIMEOUT
    # the context is intact: a plan still evaluates an RHS correctly
    prob = get_problem("wave", 3, 2, definition="reference", nel_1d=2)
    plan = DevicePlan(DeviceMesh(prob.disc, "cuda:0"), "wave", prob.params, "fp64")
    got = plan.rhs(torch.from_numpy(prob.fields).cuda())
    plan.finish()
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got.cpu().numpy(), ref, scale) <= FP64_RTOL

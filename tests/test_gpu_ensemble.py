"""Ensemble batching: one launch over uneven member meshes equals the
members evaluated one by one."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _members(nmembers=5, order=3):
    from actx_dgfem_suite_gb300.equations.maxwell import maxwell_problem
    from actx_dgfem_suite_gb300.ensemble import random_box_sizes
    sizes = random_box_sizes(nmembers, 2, 5, seed=3)
    return [maxwell_problem(order, n, "baseline") for n in sizes]


@pytest.mark.parametrize("precision", ["fp64", "fp32-mixed"])
def test_ensemble_equals_members(precision):
    from actx_dgfem_suite_gb300.ensemble import Ensemble
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    probs = _members()
    ens = Ensemble([p.disc for p in probs], "maxwell", probs[0].params, precision)
    q = ens.stack_states([p.fields for p in probs])
    out = ens.rhs(q)
    ens.plan.finish()
    for k, p in enumerate(probs):
        plan = DevicePlan(DeviceMesh(p.disc), "maxwell", p.params, precision)
        ref = plan.rhs(torch.from_numpy(p.fields).cuda())
        plan.finish()
        assert torch.equal(ens.member(out, k), ref)


def test_ensemble_graph_replay():
    from actx_dgfem_suite_gb300.ensemble import Ensemble
    probs = _members(3, 2)
    ens = Ensemble([p.disc for p in probs], "maxwell", probs[0].params)
    q = ens.stack_states([p.fields for p in probs])
    out = torch.empty_like(q)
    ens.capture(q, out)
    ref = ens.rhs(q)
    q.mul_(2.0)
    ens.replay()
    torch.cuda.synchronize()
    assert torch.allclose(out, 2.0 * ref, rtol=1e-6, atol=1e-12)

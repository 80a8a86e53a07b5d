"""Box meshes built on the GPU agree with the host setup."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_device_box_matches_host(order):
    from actx_dgfem_suite_gb300.device_setup import DeviceBoxDiscretization
    from actx_dgfem_suite_gb300.discretization import make_discretization
    from actx_dgfem_suite_gb300.mesh import generate_box_tet_mesh
    n, a, b = (3, 2, 4), (-1.0, 0.0, 0.5), (1.0, 0.5, 2.0)
    host = make_discretization(generate_box_tet_mesh(a, b, n), order)
    dev = DeviceBoxDiscretization(order, n, a, b, "cuda:0", with_partner=True)
    torch.cuda.synchronize()
    assert dev.nelements == host.nelements
    np.testing.assert_allclose(dev.metric.cpu().numpy(), host.metric_flat(),
                               rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(dev.face_geom.cpu().numpy(), host.face_geometry(),
                               rtol=1e-13, atol=1e-14)
    assert np.array_equal(dev.gather.cpu().numpy().view(np.uint32), host.gather_index())
    assert np.array_equal(dev.partner.cpu().numpy(), host.face_partner())
    np.testing.assert_allclose(dev.nodes().cpu().numpy(), host.nodes(),
                               rtol=0, atol=1e-14)


@pytest.mark.parametrize("equation", ["wave", "euler", "maxwell"])
def test_device_problem_rhs_matches_host(equation):
    from actx_dgfem_suite_gb300.device_setup import device_problem
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    from actx_dgfem_suite_gb300.rhs_builder import get_problem
    hp = get_problem(equation, 3, 3, definition="baseline", nel_1d=4)
    dp = device_problem(equation, 3, 4, "baseline", "cuda:0")
    np.testing.assert_allclose(dp.fields.cpu().numpy(), hp.fields, rtol=0, atol=1e-13)
    q = torch.from_numpy(hp.fields).cuda()
    r_host = DevicePlan(DeviceMesh(hp.disc), equation, hp.params).rhs(q)
    r_dev = DevicePlan(DeviceMesh(dp.disc), equation, dp.params).rhs(q)
    torch.cuda.synchronize()
    err = float(torch.linalg.norm(r_dev - r_host) / torch.linalg.norm(r_host))
    assert err < 1e-13, err


def test_device_union_matches_host_union():
    from actx_dgfem_suite_gb300.device_setup import (DeviceBoxDiscretization,
                                                     device_union)
    from actx_dgfem_suite_gb300.discretization import (make_box_discretization,
                                                       union_discretization)
    sizes = [2, 3, 2]
    hosts = [make_box_discretization(2, n, 0.0, 1.0) for n in sizes]
    devs = [DeviceBoxDiscretization(2, n, 0.0, 1.0, "cuda:0", with_partner=True)
            for n in sizes]
    hu, hoffs = union_discretization(hosts)
    du, doffs = device_union(devs)
    assert list(hoffs) == list(doffs)
    assert np.array_equal(du.gather.cpu().numpy().view(np.uint32), hu.gather_index())
    assert np.array_equal(du.partner.cpu().numpy(), hu.face_partner())


def test_get_rhs_device_setup_through_actx(actx):
    from actx_dgfem_suite_gb300.containers import leaves
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs
    r1, a1 = get_rhs("tiny_maxwell", actx, 3, 3, definition="baseline")
    r2, a2 = get_rhs("tiny_maxwell", actx, 3, 3, definition="baseline",
                     device_setup=True)
    o1 = np.stack([d[0] for d in leaves(actx.to_numpy(actx.compile(r1)(*a1)))])
    o2 = np.stack([d[0] for d in leaves(actx.to_numpy(actx.compile(r2)(*a2)))])
    assert np.linalg.norm(o1 - o2) <= 1e-13 * np.linalg.norm(o1)


def test_timestep_estimate_device_mesh_matches_host():
    from actx_dgfem_suite_gb300.device_setup import DeviceBoxDiscretization
    from actx_dgfem_suite_gb300.discretization import make_discretization
    from actx_dgfem_suite_gb300.mesh import generate_box_tet_mesh
    from actx_dgfem_suite_gb300.timestepping import estimate_rk4_timestep
    n, a, b = (3, 2, 4), (-1.0, 0.0, 0.5), (1.0, 0.5, 2.0)
    host = make_discretization(generate_box_tet_mesh(a, b, n), 3)
    dev = DeviceBoxDiscretization(3, n, a, b, "cuda:0")
    dt_h = estimate_rk4_timestep(host, 1.3, 0.5)
    dt_d = estimate_rk4_timestep(dev, 1.3, 0.5)
    assert abs(dt_d - dt_h) <= 1e-13 * dt_h

"""FP64 parity of the CUDA RHS kernels against the CPU oracle, through the
C ABI (DevicePlan -> dg_rhs).  Bound: relative L2 <= 1e-12.

All FP64 paths are covered: ``tc`` (``fp64-tc``, mesh uploaded with face
partners: face kernel evaluates each glued pair's flux once, then volume +
LIFT with the contractions on the tensor cores as an exact FP64 emulation),
``shared`` (the same split with FP64-FMA contractions, the ``fp64`` default) and
``fused`` (no partners: one launch computes every face point's flux)."""

from __future__ import annotations

import numpy as np
import pytest

from tests._helpers import (FP64_RTOL, jittered_box_mesh, make_problem, oracle_rhs,
                           parity_error, single_tet_mesh)
from actx_dgfem_suite_gb300.mesh import generate_box_tet_mesh
from actx_dgfem_suite_gb300.rhs_builder import get_problem

pytestmark = pytest.mark.gpu

EQUATIONS = ("wave", "euler", "maxwell")
ORDERS = (1, 2, 3, 4)
PATHS = ("tc", "shared", "fused")


def _gpu_rhs(problem, path="tc"):
    import torch

    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    dm = DeviceMesh(problem.disc, "cuda:0", with_partner=(path != "fused"))
    plan = DevicePlan(dm, problem.equation, problem.params,
                      "fp64-tc" if path == "tc" else "fp64")
    info = plan.info()
    assert info["face_shared"] == (path != "fused")
    # tensor-core products are built for orders 3 and 4 (FP64 FMAs below)
    assert info["tensor_cores"] == (path == "tc" and problem.disc.order >= 3)
    q = torch.from_numpy(problem.fields).to("cuda:0")
    out = plan.rhs(q)
    plan.finish()
    return out.cpu().numpy(), plan


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("definition", ("reference", "baseline"))
@pytest.mark.parametrize("path", PATHS)
def test_parity_box(equation, order, definition, path):
    prob = get_problem(equation, 3, order, definition=definition, nel_1d=3)
    got, _ = _gpu_rhs(prob, path)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
def test_parity_tiny_benchmark_config(equation):
    """The tiny benchmark configuration as stated: P2 tetrahedra on 6^3 hexes
    x 6 tets (1296 elements), benchmark definitions (wave: [-1,1]^3,
    p = exp(-|x|^2/0.1^2), v = 0, upwind, Dirichlet pressure; Euler and
    Maxwell at the same size).  The public builder and compiled callable with
    a host state (the default FP64 path and fp64-tc), and every FP64 path
    through the plans, checked against the oracle."""
    from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext
    from actx_dgfem_suite_gb300.containers import leaves
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs
    actx = GB300DGArrayContext("cuda:0")
    rhs, args = get_rhs(equation, actx, 3, 2, definition="baseline", nel_1d=6)
    prob = rhs.dg_operator.problem
    assert prob.disc.nelements == 1296 and prob.disc.np_ == 10
    ref, scale = oracle_rhs(prob, parts=True)
    for precision in ("fp64", "fp64-tc"):
        rhs.dg_operator.precision = precision
        out = actx.to_numpy(actx.compile(rhs)(*args))
        got = np.stack([d[0] for d in leaves(out)])
        assert parity_error(got, ref, scale) <= FP64_RTOL, precision
    for path in PATHS:
        got, _ = _gpu_rhs(prob, path)
        assert parity_error(got, ref, scale) <= FP64_RTOL, path
    if equation == "wave":
        v = prob.disc.mesh.vertices
        assert (v.min(), v.max()) == (-1.0, 1.0)
        x = prob.disc.nodes()
        assert np.allclose(prob.fields[0], np.exp(-(x ** 2).sum(axis=0) / 0.01))
        assert not prob.fields[1:].any()


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("path", PATHS)
def test_parity_jittered_mesh(equation, order, path):
    prob = make_problem(equation, jittered_box_mesh(4), order, seed=order)
    got, _ = _gpu_rhs(prob, path)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("path", PATHS)
def test_parity_single_element(equation, order, path):
    prob = make_problem(equation, single_tet_mesh(), order)
    got, _ = _gpu_rhs(prob, path)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("path", PATHS)
def test_parity_single_hex(equation, path):
    prob = make_problem(equation, generate_box_tet_mesh(0.0, 1.0, 1), 3)
    got, _ = _gpu_rhs(prob, path)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("path", PATHS)
def test_parity_anisotropic_box(equation, path):
    """n = (5, 2, 3) hexahedra per axis: a tile tail and uneven neighbours."""
    prob = make_problem(equation, generate_box_tet_mesh((0, 0, 0), (2.0, 0.5, 1.0),
                                                        (5, 2, 3)), 2, seed=3)
    got, _ = _gpu_rhs(prob, path)
    ref, scale = oracle_rhs(prob, parts=True)
    assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("path", PATHS)
def test_deterministic_bitwise(path):
    prob = make_problem("euler", jittered_box_mesh(4), 3)
    a, plan = _gpu_rhs(prob, path)
    b, _ = _gpu_rhs(prob, path)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("equation", EQUATIONS)
def test_paths_agree_and_launch_counts(equation):
    """The two FP64 paths agree to round-off; the shared path reports its
    extra launches and owns each interior face once."""
    prob = make_problem(equation, jittered_box_mesh(4), 2, seed=5)
    a, plan_s = _gpu_rhs(prob, "shared")
    b, plan_f = _gpu_rhs(prob, "fused")
    c, plan_t = _gpu_rhs(prob, "tc")
    d4, plan_t4 = _gpu_rhs(make_problem(equation, jittered_box_mesh(4), 4, seed=5), "tc")
    e4, _ = _gpu_rhs(make_problem(equation, jittered_box_mesh(4), 4, seed=5), "fused")
    assert np.linalg.norm(a - b) <= 1e-13 * np.linalg.norm(b)
    assert np.linalg.norm(c - b) <= 1e-13 * np.linalg.norm(b)
    assert np.linalg.norm(d4 - e4) <= 1e-13 * np.linalg.norm(e4)
    assert plan_t4.info()["tensor_cores"]
    assert plan_t.info()["launches_per_rhs"] == plan_s.info()["launches_per_rhs"]
    info_s, info_f = plan_s.info(), plan_f.info()
    assert info_s["launches_per_rhs"] == (3 if equation == "euler" else 2)
    assert info_f["launches_per_rhs"] == 1 and not info_f["face_shared"]
    d = prob.disc
    nbdry = int((d.neighbor < 0).sum())
    assert info_s["owned_faces"] == nbdry + (4 * d.nelements - nbdry) // 2


def test_inconsistent_partner_rejected():
    """A partner table that does not pair whole faces consistently with the
    gather index is refused at plan creation (checked by the ownership
    kernel, which reads only in-range indices)."""
    import torch

    from actx_dgfem_suite_gb300._lib import DGError
    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    prob = make_problem("wave", jittered_box_mesh(3), 2)
    dm = DeviceMesh(prob.disc, "cuda:0", with_partner=True)
    part = prob.disc.face_partner().copy()
    inner = np.flatnonzero(part.reshape(-1) >= 0)
    bad = part.reshape(-1)
    i, j = inner[0], inner[-1]
    bad[i], bad[j] = bad[j], bad[i]          # two points now point at wrong faces
    dm.partner = torch.from_numpy(bad.reshape(part.shape)).to("cuda:0")
    with pytest.raises(DGError, match="face_partner"):
        DevicePlan(dm, "wave", prob.params)
    bad2 = part.reshape(-1).copy()
    bad2[inner[0]] = 10**9                    # out of range: rejected, never read
    dm.partner = torch.from_numpy(bad2.reshape(part.shape)).to("cuda:0")
    with pytest.raises(DGError, match="face_partner"):
        DevicePlan(dm, "wave", prob.params)


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", (3, 4))
@pytest.mark.parametrize("drop", (1, 7))
def test_parity_odd_element_count(equation, order, drop):
    """A box mesh with ``drop`` elements removed (their faces become walls):
    an odd element count leaves partial tiles whose sizes are no multiple of
    16 bytes, which the order-3 tensor-core kernel loads with plain loads
    instead of its bulk-copy prefetch; both paths against the oracle."""
    from actx_dgfem_suite_gb300.mesh import TetMesh
    box = jittered_box_mesh(4)
    keep = np.ones(box.nelements, dtype=bool)
    keep[np.linspace(0, box.nelements - 1, drop).astype(int)] = False
    mesh = TetMesh(box.vertices, box.elements[keep])
    assert mesh.nelements % 2 == 1
    prob = make_problem(equation, mesh, order, seed=order + drop)
    ref, scale = oracle_rhs(prob, parts=True)
    for path in ("tc", "shared"):
        got, _ = _gpu_rhs(prob, path)
        assert parity_error(got, ref, scale) <= FP64_RTOL


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", (3, 4))
def test_tc_rk_stage_matches_fma_path(equation, order):
    """The fused RK stage of the tensor-core kernel (at order 3 its state
    comes from the prefetched input buffer) against the FP64-FMA kernel, with
    a nonzero residual, a per-element scale and the unscaled RHS output."""
    import torch

    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    prob = make_problem(equation, jittered_box_mesh(4), order, seed=11 + order)
    dm = DeviceMesh(prob.disc, "cuda:0", with_partner=True)
    q = torch.from_numpy(prob.fields).to("cuda:0")
    nel = prob.disc.nelements
    scale = torch.linspace(0.9, 1.1, nel, dtype=torch.float64, device="cuda:0")
    res0 = torch.rand(q.shape, dtype=q.dtype, device=q.device,
                      generator=torch.Generator(device=q.device).manual_seed(3))
    outs = []
    for prec in ("fp64-tc", "fp64"):
        plan = DevicePlan(dm, equation, prob.params, prec)
        assert plan.info()["tensor_cores"] == (prec == "fp64-tc")
        plan.set_element_scale(scale)
        res, qo, un = res0.clone(), torch.empty_like(q), torch.empty_like(q)
        plan.rk_stage(q, qo, res, 0.4, 0.3, 2e-3, rhs_unscaled=un)
        plan.finish()
        outs.append((qo, res, un))
    for a, b in zip(outs[0], outs[1]):
        assert float(torch.linalg.norm(a - b)) <= FP64_RTOL * float(torch.linalg.norm(b))


@pytest.mark.parametrize("equation", EQUATIONS)
@pytest.mark.parametrize("order", (3, 4))
def test_tc_nan_propagates_like_fp64(equation, order):
    """A NaN in one element's state: the tensor-core FP64 emulation returns
    NaN where the FMA path does (that element and its face neighbours), not
    finite values from the fixed-point split, and the same RHS elsewhere."""
    import torch

    from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
    prob = make_problem(equation, jittered_box_mesh(5), order, seed=2)
    dm = DeviceMesh(prob.disc, "cuda:0", with_partner=True)
    q = torch.from_numpy(prob.fields).to("cuda:0")
    q[1, 11, 2] = float("nan")
    outs = {}
    for prec in ("fp64-tc", "fp64"):
        plan = DevicePlan(dm, equation, prob.params, prec)
        outs[prec] = plan.rhs(q)
        plan.finish()
    tc, fma = outs["fp64-tc"], outs["fp64"]
    bad_tc = ~torch.isfinite(tc).all(dim=(0, 2))
    bad_fma = ~torch.isfinite(fma).all(dim=(0, 2))
    assert bool(bad_fma[11]) and torch.equal(bad_tc, bad_fma)
    ok = ~bad_fma
    n = float(torch.linalg.norm(fma[:, ok]))
    assert float(torch.linalg.norm(tc[:, ok] - fma[:, ok])) <= FP64_RTOL * n

"""Shared test helpers: oracle evaluation of a problem and small meshes."""

from __future__ import annotations

import numpy as np

from actx_dgfem_suite_gb300.discretization import make_discretization
from actx_dgfem_suite_gb300.discretization2d import make_discretization_2d
from actx_dgfem_suite_gb300.equations.common import Problem
from actx_dgfem_suite_gb300.mesh import (
    TetMesh,
    TriMesh,
    generate_box_tet_mesh,
    generate_box_tri_mesh,
)

#: relative L2 parity bound for the FP64 path against the CPU oracle
FP64_RTOL = 1e-12


def oracle_rhs(problem: Problem, od=None, parts: bool = False):
    """Oracle RHS of ``problem``; with ``parts=True`` returns
    ``(rhs, scale)``, ``scale`` the L2 norm of the volume and surface terms
    that cancel into the RHS (see :func:`parity_error`)."""
    from oracle.geometry import build_oracle_disc, build_oracle_disc_2d
    from oracle.rhs import euler_rhs, maxwell_rhs, wave_rhs
    d = problem.disc
    dim = getattr(d, "dim", 3)
    if od is None:
        build = build_oracle_disc if dim == 3 else build_oracle_disc_2d
        od = build(d.mesh.vertices, d.mesh.elements, d.order)
    check_node_layout(d, od)
    q = problem.fields
    if problem.equation == "wave":
        rhs, vol, surf = wave_rhs(od, q[0], q[1:1 + dim], *problem.params, parts=True)
    elif problem.equation == "euler":
        rhs, vol, surf = euler_rhs(od, q, *problem.params, parts=True)
    else:
        rhs, vol, surf = maxwell_rhs(od, q, *problem.params, parts=True)
    if parts:
        return rhs, float(np.sqrt(np.linalg.norm(vol) ** 2 + np.linalg.norm(surf) ** 2))
    return rhs


def check_node_layout(disc, od) -> None:
    """The product's volume nodes must sit at the oracle's node coordinates,
    in the same order: the oracle builds its node set independently, so this
    pins the product's node family, node order and element geometry before
    any state in the product's layout is handed to the oracle."""
    x = disc.nodes()
    if not isinstance(x, np.ndarray):      # a mesh built on the device
        x = x.detach().cpu().numpy()
    err = float(np.max(np.abs(np.asarray(x) - od.nodes)))
    assert err <= 1e-12, f"product nodes differ from the oracle's by {err:.3e}"


def rel_l2(a, b) -> float:
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


#: below this ratio ||rhs|| / ||(volume, surface)|| the RHS counts as a
#: near-cancellation of its volume and surface terms
CANCELLATION_RATIO = 1e-2


def parity_error(got, ref, scale: float) -> float:
    """Plain relative L2 error ||got - ref|| / ||ref|| of ``got`` against the
    oracle ``ref`` -- except where the RHS is a near-cancellation of its
    volume and surface terms (||ref|| below ``CANCELLATION_RATIO`` times
    ``scale``, the norm of those terms; e.g. the reference Euler pulse on a
    state at rest, ratio 2e-4 to 2e-3): there ||ref|| sits near round-off
    level, a plain relative error would compare round-off with round-off,
    and the error is normalised by ``scale`` instead."""
    diff = float(np.linalg.norm(np.asarray(got) - np.asarray(ref)))
    nref = float(np.linalg.norm(ref))
    if nref >= CANCELLATION_RATIO * scale:
        return diff / nref
    return diff / scale


def scaled_error(got, ref, scale: float) -> float:
    """||got - ref|| / max(||ref||, scale): the error relative to the size of
    the RHS's volume and surface terms, for comparing two oracle
    constructions whose matrices differ by round-off in those terms."""
    diff = float(np.linalg.norm(np.asarray(got) - np.asarray(ref)))
    return diff / max(float(np.linalg.norm(ref)), scale)


def jittered_box_mesh(n: int, amp: float = 0.15, seed: int = 1) -> TetMesh:
    """Box mesh on [0,1]^3 with interior vertices moved randomly (non-uniform
    affine elements, still positively oriented for amp < 0.25)."""
    m = generate_box_tet_mesh(0.0, 1.0, n)
    v = m.vertices.copy()
    h = 1.0 / n
    interior = np.all((v > 1e-12) & (v < 1 - 1e-12), axis=1)
    rng = np.random.default_rng(seed)
    v[interior] += amp * h * rng.uniform(-1, 1, size=(interior.sum(), 3))
    return TetMesh(vertices=v, elements=m.elements)


def jittered_square_mesh(n: int, amp: float = 0.15, seed: int = 1) -> TriMesh:
    """Triangle mesh on [0,1]^2 with interior vertices moved randomly
    (counter-clockwise elements for amp < 0.25)."""
    m = generate_box_tri_mesh(0.0, 1.0, n)
    v = m.vertices.copy()
    h = 1.0 / n
    interior = np.all((v > 1e-12) & (v < 1 - 1e-12), axis=1)
    rng = np.random.default_rng(seed)
    v[interior] += amp * h * rng.uniform(-1, 1, size=(interior.sum(), 2))
    return TriMesh(vertices=v, elements=m.elements)


def single_tet_mesh() -> TetMesh:
    v = np.array([[0.0, 0, 0], [1.0, 0.1, 0], [0.2, 0.9, 0.1], [0.1, 0.2, 0.8]])
    return TetMesh(vertices=v, elements=np.array([[0, 1, 2, 3]], dtype=np.int64))


def smooth_fields(disc, nfields: int, equation: str, seed: int = 0) -> np.ndarray:
    """Smooth random-ish state; Euler gets positive density and pressure."""
    x = disc.nodes()
    dim = x.shape[0]
    rng = np.random.default_rng(seed)
    out = np.empty((nfields,) + x.shape[1:])
    for k in range(nfields):
        a = rng.uniform(0.5, 2.0, size=3)
        ph = rng.uniform(0, 2 * np.pi, size=3)
        out[k] = np.sin(a[0] * 3 * x[0] + ph[0]) * np.cos(a[1] * 2 * x[1] + ph[1]) \
            + 0.3 * np.sin(a[2] * 4 * x[dim - 1] + ph[2])
    if equation == "euler":
        out[0] = 1.0 + 0.2 * out[0] ** 2
        out[2:2 + dim] *= 0.2
        kinetic = 0.5 * (out[2:2 + dim] ** 2).sum(axis=0) / out[0]
        out[1] = 2.5 + 0.3 * out[1] ** 2 + kinetic
    return out


def make_problem(equation: str, mesh: TetMesh, order: int, fields=None,
                 params=None, seed: int = 0) -> Problem:
    disc = make_discretization(mesh, order)
    nf = {"wave": 4, "euler": 5, "maxwell": 6}[equation]
    if params is None:
        params = {"wave": (1.0,), "euler": (1.4,), "maxwell": (0.5, 1.0, 1.0)}[equation]
    if fields is None:
        fields = smooth_fields(disc, nf, equation, seed)
    return Problem(equation, disc, fields, params,
                   None if equation == "wave" else 0.5, "test")


def make_problem_2d(equation: str, mesh: TriMesh, order: int, fields=None,
                    params=None, seed: int = 0) -> Problem:
    """A problem on a triangle mesh: fields (3, 4, 3) for wave, Euler and
    Maxwell (TM)."""
    disc = make_discretization_2d(mesh, order)
    nf = {"wave": 3, "euler": 4, "maxwell": 3}[equation]
    if params is None:
        params = {"wave": (1.0,), "euler": (1.4,), "maxwell": (0.5, 1.0, 1.0)}[equation]
    if fields is None:
        fields = smooth_fields(disc, nf, equation, seed)
    return Problem(equation, disc, fields, params,
                   None if equation == "wave" else 0.5, "test")

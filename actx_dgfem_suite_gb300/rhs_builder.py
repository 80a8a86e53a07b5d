"""Dispatch helper that builds ``(rhs, call_args)`` for each equation,
mirroring ``actx_dgfem_suite/rhs_builder.py:14-45``.

``tiny_`` / ``large_`` / unprefixed names select 1e3 / 2e7 / 4e6 DOFs per
field (``rhs_builder.py:9-11``).  ``definition`` picks the reference's own
problem setup (default) or the benchmark ("baseline") setup; ``nel_1d``
overrides the element count per axis.
"""

from __future__ import annotations

from typing import Any

_NDOFS_FULL = 4_000_000
_NDOFS_TINY = 1_000
_NDOFS_LARGE = 20_000_000


def split_equation_name(equation: str) -> tuple[str, int]:
    if equation.startswith("tiny_"):
        return equation.removeprefix("tiny_"), _NDOFS_TINY
    if equation.startswith("large_"):
        return equation.removeprefix("large_"), _NDOFS_LARGE
    return equation, _NDOFS_FULL


def get_rhs(equation: str, actx, dim: int, degree: int, *,
            definition: str = "reference", nel_1d: int | None = None,
            device_setup: bool = False) -> tuple[Any, tuple[Any, ...]]:
    """Return ``(rhs_callable, call_args)`` for ``equation``.

    ``dim`` 3 builds tetrahedral box meshes, 2 triangle meshes (the suite's
    CI runs both, ``--dims 2,3``).  ``device_setup=True`` builds the 3D box
    mesh, geometry, connectivity and initial state on the array context's
    GPU instead of on the host."""
    base, ndofs = split_equation_name(equation)
    if device_setup:
        from actx_dgfem_suite_gb300.device_setup import device_problem
        from actx_dgfem_suite_gb300.equations.common import make_rhs_and_args
        from actx_dgfem_suite_gb300.utils import get_nel_1d_for_regular_rect_mesh
        if dim != 3:
            raise NotImplementedError("device-side setup builds 3D meshes only")
        if base not in ("wave", "euler", "maxwell"):
            raise NotImplementedError(f"equation '{equation}' not supported")
        n = nel_1d or get_nel_1d_for_regular_rect_mesh(dim, degree, ndofs)
        return make_rhs_and_args(device_problem(base, degree, n, definition,
                                                actx.device), actx)
    kw = dict(actx=actx, dim=dim, order=degree, ndofs=ndofs,
              definition=definition, nel_1d=nel_1d)
    if base == "wave":
        from actx_dgfem_suite_gb300.equations.wave import get_wave_rhs
        return get_wave_rhs(**kw)
    if base == "euler":
        from actx_dgfem_suite_gb300.equations.euler import get_euler_rhs
        return get_euler_rhs(**kw)
    if base == "maxwell":
        from actx_dgfem_suite_gb300.equations.maxwell import get_maxwell_rhs
        return get_maxwell_rhs(**kw)
    raise NotImplementedError(f"equation '{equation}' not supported")


def get_problem(equation: str, dim: int, degree: int, *,
                definition: str = "reference", nel_1d: int | None = None):
    """Host-side setup only (mesh, geometry, initial state), no device."""
    from actx_dgfem_suite_gb300.utils import get_nel_1d_for_regular_rect_mesh
    if dim not in (2, 3):
        raise NotImplementedError("dim must be 2 or 3")
    base, ndofs = split_equation_name(equation)
    if nel_1d is None:
        nel_1d = get_nel_1d_for_regular_rect_mesh(dim, degree, ndofs)
    if base == "wave":
        from actx_dgfem_suite_gb300.equations.wave import wave_problem
        return wave_problem(degree, nel_1d, definition, dim=dim)
    if base == "euler":
        from actx_dgfem_suite_gb300.equations.euler import euler_problem
        return euler_problem(degree, nel_1d, definition, dim=dim)
    if base == "maxwell":
        from actx_dgfem_suite_gb300.equations.maxwell import maxwell_problem
        return maxwell_problem(degree, nel_1d, definition, dim=dim)
    raise NotImplementedError(f"equation '{equation}' not supported")

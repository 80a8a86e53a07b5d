"""Mesh-size helpers, mirroring ``actx_dgfem_suite/utils.py:15-74``."""

from __future__ import annotations

from math import cbrt, ceil, sqrt

#: nodes per element of the P1..P4 simplices, 3D and 2D
_NP3 = {1: 4, 2: 10, 3: 20, 4: 35}
_NP2 = {1: 3, 2: 6, 3: 10, 4: 15}


def get_nel_1d_for_regular_rect_mesh(dim: int, order: int, ndofs: int) -> int:
    """Elements per axis so that a box of ``6 n^3`` tets (3D) or ``2 n^2``
    triangles (2D) holds about ``ndofs`` DOFs per field
    (``actx_dgfem_suite/utils.py:15-43``)."""
    if dim == 3:
        if order not in _NP3:
            raise NotImplementedError(order)
        return int(ceil(cbrt((ndofs / _NP3[order]) / 6)))
    if dim == 2:
        if order not in _NP2:
            raise NotImplementedError(order)
        return int(ceil(sqrt((ndofs / _NP2[order]) / 2)))
    raise NotImplementedError


def get_ndof_for_regular_rect_mesh(dim: int, order: int, nel_1d: int) -> int:
    """DOFs per field of the box mesh (``actx_dgfem_suite/utils.py:46-74``).

    The reference multiplies the 3D P1 element count by 6 instead of Np = 4
    (``utils.py:50``), over-counting P1 DOFs by 1.5x in its DOF-scaling tool;
    this helper returns the true count Nel * Np."""
    if dim == 3:
        if order not in _NP3:
            raise NotImplementedError(order)
        return 6 * nel_1d**3 * _NP3[order]
    if dim == 2:
        if order not in _NP2:
            raise NotImplementedError(order)
        return 2 * nel_1d**2 * _NP2[order]
    raise NotImplementedError

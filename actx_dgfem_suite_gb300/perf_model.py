"""Analytic FLOP and byte model of one RHS evaluation.

The reference counts FP64 operations on its transformed pytato DAG
(``actx_dgfem_suite/perf_analysis.py:535-576``): every einsum along the
``opt_einsum`` "optimal" contraction path at one multiply plus one add per
iteration point of a reducing contraction and one multiply per point of an
outer product (``perf_analysis.py:380-417``), and one operation per output
element for each pointwise +, -, *, /, where, max, min and sqrt
(``perf_analysis.py:265-377``).  That DAG cannot be built here, so this module
applies the same rules to the einsums the mass-inverse fusion produces
(``actx_dgfem_suite/arraycontext/mass_inverse_fuser.py:20-76``), which are
exact, plus per-node / per-face-point pointwise counts.  For the wave
equation those are counted from the reference's own ``wave_operator`` run
on stand-ins for its dependencies (``tests/golden/make_reference_flop_counts.py``:
8 per node, 38 per face point of a trace pair's flux plus 1 per boundary
face point for the mirrored state, and 8 per face point for summing the
boundary and interior fluxes on all faces); what the reference's DAG
transformations merge is not visible there.  Euler and Maxwell, whose
operators live in grudge (absent), use estimates from the restated flux
and volume-flux expressions.

Bytes are the algorithmic minimum a fused implementation moves per RHS:
state in and RHS out (FP64), the per-element metric (9 doubles), per-face
normal + sJ/J (16 doubles) and one 4-byte gather index per face node.  The
reference's ``get_footprint_bytes`` (``perf_analysis.py:581-619``) sums kernel
arguments of its own kernel split instead.

``dim=2`` (triangles, 3 edges) applies the same rules: the einsums have two
reference axes, the state holds 3 (wave), 4 (Euler) or 3 (Maxwell TM)
fields, the metric is 2x2 and each edge carries a 2-vector normal and sJ/J.
"""

from __future__ import annotations

from dataclasses import dataclass

NFIELDS = {"wave": 4, "euler": 5, "maxwell": 6}
NFIELDS_2D = {"wave": 3, "euler": 4, "maxwell": 3}


def np_of(order: int, dim: int = 3) -> int:
    if dim == 2:
        return (order + 1) * (order + 2) // 2
    return (order + 1) * (order + 2) * (order + 3) // 6


def nfp_of(order: int, dim: int = 3) -> int:
    if dim == 2:
        return order + 1
    return (order + 1) * (order + 2) // 2


# {{{ einsum counts per element (suite rules; exact)


def grad_flops(order: int, dim: int = 3) -> int:
    """``re,rji,ej->ei``: 3 Np + 6 Np^2 (2D: 2 Np + 4 Np^2)."""
    n = np_of(order, dim)
    return dim * n + 2 * dim * n * n


def div_flops(order: int, dim: int = 3) -> int:
    """``xre,rji,xej->ei``: 18 Np + 6 Np^2 (2D: 8 Np + 4 Np^2)."""
    n = np_of(order, dim)
    return 2 * dim * dim * n + 2 * dim * n * n


def lift_flops(order: int, dim: int = 3) -> int:
    """``jfi,fe,fej->ei``: 4 Nfp + 8 Nfp Np (2D, 3 edges: 3 Nfp + 6 Nfp Np)."""
    nf = dim + 1
    return nf * nfp_of(order, dim) + 2 * nf * nfp_of(order, dim) * np_of(order, dim)


# }}}

#: pointwise operations per face point and per volume node: wave counted
#: from the reference's wave_operator (38 flux + 8 all-faces sum per face
#: point), Euler and Maxwell estimated from the restated expressions
_POINTWISE = {
    "wave": (46, 8),
    "euler": (251, 48),
    "maxwell": (72, 30),
}
#: the wave boundary pair's extra operation per boundary face point (the
#: mirrored exterior state -u)
WAVE_BOUNDARY_EXTRA = 1
#: the same on triangles: wave counted from the reference's wave_operator
#: with dim = 2 (27 flux + 6 all-faces sum per face point, 6 per node);
#: Maxwell TM counted from the 2D flux expressions (the TM components of the
#: alpha flux and the PEC mirror); Euler scaled from 3D by its flux
#: components (8 of 15)
_POINTWISE_2D = {
    "wave": (33, 6),
    "euler": (134, 26),
    "maxwell": (28, 10),
}


def einsum_flops_per_element(equation: str, order: int, dim: int = 3) -> int:
    g, d, li = grad_flops(order, dim), div_flops(order, dim), lift_flops(order, dim)
    if dim == 2:
        if equation == "wave":      # 1 div + 2 grad + 3 LIFT
            return d + 2 * g + 3 * li
        if equation == "euler":     # 4 div + 4 LIFT
            return 4 * d + 4 * li
        if equation == "maxwell":   # 4 TM curl derivatives + 3 LIFT
            return 4 * g + 3 * li
        raise ValueError(equation)
    if equation == "wave":      # 1 div (u) + 3 grad (v) + 4 LIFT
        return d + 3 * g + 4 * li
    if equation == "euler":     # 5 div + 5 LIFT
        return 5 * d + 5 * li
    if equation == "maxwell":   # 12 curl derivatives + 6 LIFT
        return 12 * g + 6 * li
    raise ValueError(equation)


def flops_per_element(equation: str, order: int, dim: int = 3) -> int:
    """Per element, boundary terms aside (see :attr:`RhsCost.flops`)."""
    face, vol = (_POINTWISE_2D if dim == 2 else _POINTWISE)[equation]
    return (einsum_flops_per_element(equation, order, dim)
            + face * (dim + 1) * nfp_of(order, dim) + vol * np_of(order, dim))


def bytes_per_element(equation: str, order: int, dim: int = 3) -> int:
    if dim == 2:   # metric 2x2, 3 edges x (n_x, n_y, sJ/J), 3 Nfp indices
        return (16 * NFIELDS_2D[equation] * np_of(order, 2) + 4 * 8 + 9 * 8
                + 3 * 4 * nfp_of(order, 2))
    return (16 * NFIELDS[equation] * np_of(order) + 9 * 8 + 16 * 8
            + 4 * 4 * nfp_of(order))


def fp64_fma_per_element(equation: str, order: int) -> int:
    """FP64 fused multiply-adds the CUDA kernel issues per element in its
    contractions (the reference derivatives of a field are shared by its
    gradient components; see ``csrc/dg_rhs_fp64.cuh``)."""
    n, nf = np_of(order), 4 * nfp_of(order)
    lift = NFIELDS[equation] * n * nf
    if equation == "wave":
        return 6 * n * n + lift          # 3 D_r u + sum_r D_r (G v)_r
    if equation == "euler":
        return 15 * n * n + lift         # 5 fields x sum_r D_r (G F)_r
    if equation == "maxwell":
        return 18 * n * n + lift         # 6 fields x 3 D_r
    raise ValueError(equation)


@dataclass(frozen=True)
class RhsCost:
    equation: str
    order: int
    nelements: int
    dim: int = 3
    #: faces on the boundary (box of n^3 hexahedra: 12 n^2), for the wave
    #: boundary pair's extra operation; 0 leaves it out
    boundary_faces: int = 0

    @property
    def dofs(self) -> int:
        """DOF updates per RHS: nfields * Nel * Np."""
        nf = (NFIELDS_2D if self.dim == 2 else NFIELDS)[self.equation]
        return nf * self.nelements * np_of(self.order, self.dim)

    @property
    def flops(self) -> int:
        extra = 0
        if self.equation == "wave":
            extra = WAVE_BOUNDARY_EXTRA * self.boundary_faces * nfp_of(self.order, self.dim)
        return self.nelements * flops_per_element(self.equation, self.order, self.dim) + extra

    @property
    def bytes(self) -> int:
        return self.nelements * bytes_per_element(self.equation, self.order, self.dim)

    @property
    def fma(self) -> int:
        return self.nelements * fp64_fma_per_element(self.equation, self.order)

    def roofline_seconds(self, peak_flops: float, peak_bytes: float) -> float:
        """``max(F / peak_F, B / peak_BW)`` (``perf_analysis.py:643-651``)."""
        return max(self.flops / peak_flops, self.bytes / peak_bytes)

"""Box meshes built on the GPU.

The host setup (``discretization.make_discretization``) spends tens of
seconds on a 5 M-element box in NumPy (face sorting, node coordinates).  For
the suite's box meshes (``meshmode.mesh.generation.generate_regular_rect_mesh``
at ``actx_dgfem_suite/equations/wave.py:250-252``) the connectivity is known
in closed form, so ``dg_box_mesh_build`` writes geometry, gather index,
face partners and node coordinates straight into device memory, one thread
per element.  The only host work is a 6 x 4 neighbour table of the
hexahedron split, derived once here from a 3 x 3 x 3 host box so that the
device mesh is the host mesh element for element.
"""

from __future__ import annotations

import ctypes
from functools import lru_cache

import numpy as np
import torch

from actx_dgfem_suite_gb300 import _lib
from actx_dgfem_suite_gb300.discretization import _PERMS, make_discretization
from actx_dgfem_suite_gb300.mesh import HEX_TO_TETS, generate_box_tet_mesh
from actx_dgfem_suite_gb300.refelem import (FACE_OPPOSITE_VERTEX, FACE_VERTICES,
                                            recursive_barycentric_nodes,
                                            reference_tet)


@lru_cache(maxsize=None)
def hex_split_tables() -> tuple[np.ndarray, np.ndarray]:
    """(corner (6, 4, 3), neighbour (6, 4, 6)) int32 tables of the split:
    neighbour[t, f] = (di, dj, dk, t', f', permutation id)."""
    corner = np.array([[[int(ch) for ch in lab] for lab in tet] for tet in HEX_TO_TETS],
                      dtype=np.int32)
    d = make_discretization(generate_box_tet_mesh(0.0, 1.0, 3), 1)
    mid = (1 * 3 + 1) * 3 + 1
    nbr = np.zeros((6, 4, 6), dtype=np.int32)
    for t in range(6):
        e = mid * 6 + t
        for f in range(4):
            e2 = int(d.neighbor[e, f])
            assert e2 >= 0, "the middle hexahedron has no boundary faces"
            hex2, t2 = divmod(e2, 6)
            i2, rem = divmod(hex2, 9)
            j2, k2 = divmod(rem, 3)
            nbr[t, f] = (i2 - 1, j2 - 1, k2 - 1, t2, int(d.neighbor_face[e, f]),
                         int(d.perm_id[e, f]))
    return corner, nbr


@lru_cache(maxsize=None)
def element_tables(order: int):
    ref = reference_tet(order)
    face_nodes = np.ascontiguousarray(ref.face_nodes, dtype=np.int32)
    perm = np.ascontiguousarray(np.stack([ref.face_perm[p] for p in _PERMS]),
                                dtype=np.int32)
    bary = np.ascontiguousarray(recursive_barycentric_nodes(3, order), dtype=np.float64)
    return face_nodes, perm, bary


class DeviceBoxDiscretization:
    """Geometry and connectivity of a box mesh, resident on one device.

    Exposes the attributes a :class:`~actx_dgfem_suite_gb300.plan.DeviceMesh`
    needs (``order``, ``ref``, ``nelements``, ``np_``, ``nfp``) and the device
    arrays in the C ABI's formats; ``nodes()`` returns the (3, Nel, Np) node
    coordinates as a device tensor."""

    def __init__(self, order: int, n, a, b, device=None, with_partner: bool = True,
                 with_nodes: bool = True):
        if np.isscalar(n):
            n = (int(n),) * 3
        a = np.broadcast_to(np.asarray(a, dtype=np.float64), (3,))
        b = np.broadcast_to(np.asarray(b, dtype=np.float64), (3,))
        dev = torch.device(device or "cuda")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        self.order = order
        self.ref = reference_tet(order)
        self.n = tuple(int(k) for k in n)
        self.box = (tuple(a), tuple(b))
        nel = 6 * self.n[0] * self.n[1] * self.n[2]
        npn, nfp = self.ref.np_, self.ref.nfp
        f64 = dict(dtype=torch.float64, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        self.metric = torch.empty((nel, 9), **f64)
        self.face_geom = torch.empty((nel, 4, 4), **f64)
        self.gather = torch.empty((nel, 4, nfp), **i32)
        self.partner = torch.empty((nel, 4, nfp), **i32) if with_partner else None
        self._nodes = torch.empty((3, nel, npn), **f64) if with_nodes else None

        corner, nbr = hex_split_tables()
        face_nodes, perm, bary = element_tables(order)
        fv = np.array(FACE_VERTICES, dtype=np.int32)
        fo = np.array(FACE_OPPOSITE_VERTEX, dtype=np.int32)
        desc = _lib.BoxDesc()
        desc.order = order
        for k in range(3):
            desc.n[k] = self.n[k]
            desc.a[k] = float(a[k])
            desc.b[k] = float(b[k])
        keep = (corner, nbr, fv, fo, face_nodes, perm, bary)
        desc.corner, desc.nbr, desc.face_vert, desc.face_opp = (
            x.ctypes.data for x in keep[:4])
        desc.face_nodes, desc.perm, desc.bary = (x.ctypes.data for x in keep[4:])
        desc.metric = self.metric.data_ptr()
        desc.face_geom = self.face_geom.data_ptr()
        desc.gather = self.gather.data_ptr()
        desc.face_partner = self.partner.data_ptr() if self.partner is not None else None
        desc.nodes = self._nodes.data_ptr() if self._nodes is not None else None
        with torch.cuda.device(dev):
            stream = torch.cuda.current_stream()
            _lib.check(_lib.lib().dg_box_mesh_build(
                ctypes.byref(desc), ctypes.c_void_p(stream.cuda_stream)))
        self.mesh = None

    @property
    def nelements(self) -> int:
        return self.metric.shape[0]

    @property
    def np_(self) -> int:
        return self.ref.np_

    @property
    def nfp(self) -> int:
        return self.ref.nfp

    def nodes(self) -> torch.Tensor:
        if self._nodes is None:
            raise ValueError("built without node coordinates")
        return self._nodes

    def drop_nodes(self) -> None:
        self._nodes = None


def device_problem(equation: str, order: int, nel_1d: int,
                   definition: str = "baseline", device=None, seed: int = 0,
                   with_partner: bool = True):
    """The builders' problem with mesh, geometry and initial state made on
    the device (same definitions as ``equations.*.*_problem``)."""
    from actx_dgfem_suite_gb300.equations import euler, maxwell, wave
    from actx_dgfem_suite_gb300.equations.common import Problem
    mod = {"wave": wave, "euler": euler, "maxwell": maxwell}[equation]
    if definition not in mod.BOXES:
        raise ValueError(f"unknown problem definition {definition!r}")
    lo, hi = mod.BOXES[definition]
    disc = DeviceBoxDiscretization(order, nel_1d, lo, hi, device, with_partner)
    x = disc.nodes()
    if equation == "wave":
        fields, params, t = wave.initial_state(x, definition), (1.0,), None
    elif equation == "euler":
        fields, params, t = (euler.initial_state(x, definition), (euler.GAMMA,), 0.5)
    else:
        fields = maxwell.initial_state(x, definition, seed)
        params, t = (maxwell.ALPHA[definition], 1.0, 1.0), 0.5
    disc.drop_nodes()
    return Problem(equation, disc, fields.contiguous(), params, t, definition)


def device_union(discs: list[DeviceBoxDiscretization]):
    """Members side by side in one device discretisation (as
    ``discretization.union_discretization``); returns (union, offsets)."""
    order = discs[0].order
    if any(d.order != order for d in discs):
        raise ValueError("all members must have the same order")
    npn, nfp = discs[0].np_, discs[0].nfp
    nels = np.array([d.nelements for d in discs], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(nels)])
    if offs[-1] * npn >= 2**31 or offs[-1] * 4 * nfp >= 2**31:
        raise ValueError("union too large for 31-bit indices")
    u = object.__new__(DeviceBoxDiscretization)
    u.device, u.order, u.ref = discs[0].device, order, discs[0].ref
    u.n, u.box, u.mesh, u._nodes = None, None, None, None
    u.metric = torch.cat([d.metric for d in discs])
    u.face_geom = torch.cat([d.face_geom for d in discs])
    flag = torch.tensor(-2**31, dtype=torch.int32, device=u.device)
    low = torch.tensor(2**31 - 1, dtype=torch.int32, device=u.device)
    gathers, partners = [], []
    for k, d in enumerate(discs):
        g = d.gather
        shifted = (g & low) + int(offs[k] * npn)
        gathers.append(torch.where(g < 0, shifted | flag, shifted))
        if d.partner is not None:
            p = d.partner
            partners.append(torch.where(p < 0, p, p + int(offs[k] * 4 * nfp)))
    u.gather = torch.cat(gathers)
    u.partner = torch.cat(partners) if len(partners) == len(discs) else None
    return u, offs

"""Device-resident mesh data and RHS plans over the C ABI.

A :class:`DeviceMesh` holds one discretisation's geometry and gather index in
HBM (shared by every equation on that mesh); a :class:`DevicePlan` is one
``dg_plan`` for (equation, mesh, parameters).  Tensors are PyTorch CUDA
tensors used as plain device buffers; only raw pointers cross the C ABI.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from actx_dgfem_suite_gb300 import _lib
from actx_dgfem_suite_gb300.discretization import DGDiscretization

EQUATIONS = {"wave": _lib.DG_WAVE, "euler": _lib.DG_EULER,
             "maxwell": _lib.DG_MAXWELL}
NFIELDS = {"wave": 4, "euler": 5, "maxwell": 6}
#: fields on triangle meshes: (u, v_x, v_y); (rho, E, m_x, m_y); TM (E_z, H_x, H_y)
NFIELDS_2D = {"wave": 3, "euler": 4, "maxwell": 3}


def _stream_handle(stream) -> ctypes.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


class DeviceMesh:
    """Geometry, gather index and reference operators of one discretisation,
    uploaded once.

    ``with_partner``: also hold the glued face-point index, which FP64 plans
    use for the face-shared path (each glued pair's flux evaluated once) and
    the adjoint needs.  ``None`` (default): whenever the discretisation
    provides it; ``False``: never (FP64 plans then use the single fused
    launch); ``True``: required."""

    def __init__(self, disc: DGDiscretization, device=None,
                 with_partner: bool | None = None):
        if not torch.cuda.is_available():
            raise RuntimeError("DeviceMesh needs a CUDA device")
        self.disc = disc
        #: 3 (tetrahedra) or 2 (triangles)
        self.dim = getattr(disc, "dim", 3)
        dev = torch.device(device or "cuda")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        if isinstance(getattr(disc, "metric", None), torch.Tensor):
            # built on the device (device_setup.DeviceBoxDiscretization)
            if disc.metric.device != dev:
                raise ValueError("device-built mesh lives on another device")
            self.metric, self.face_geom, self.gather = (
                disc.metric, disc.face_geom, disc.gather)
            self.partner = disc.partner if with_partner is not False else None
            if with_partner and self.partner is None:
                raise ValueError("device mesh was built without face partners")
        else:
            self.metric = torch.from_numpy(disc.metric_flat()).to(self.device)
            self.face_geom = torch.from_numpy(
                np.ascontiguousarray(disc.face_geometry())).to(self.device)
            self.gather = torch.from_numpy(
                disc.gather_index().view(np.int32)).to(self.device)
            # glued face-point index (face-shared path, adjoint; 3D only)
            self.partner = None
            if with_partner and self.dim == 2:
                raise ValueError("triangle meshes carry no face partners")
            if (self.dim == 3 and with_partner is not False
                    and (with_partner or disc.perm_id is not None)):
                self.partner = torch.from_numpy(disc.face_partner()).to(self.device)
        ref = disc.ref
        self._weak = np.ascontiguousarray(ref.weak_diff, dtype=np.float64)
        self._strong = np.ascontiguousarray(ref.diff, dtype=np.float64)
        self._lift = np.ascontiguousarray(ref.lift, dtype=np.float64)
        self._fnodes = np.ascontiguousarray(ref.face_nodes, dtype=np.int32)

    @property
    def nelements(self) -> int:
        return self.disc.nelements

    @property
    def np_(self) -> int:
        return self.disc.np_

    def desc(self):
        if self.dim == 2:
            d = _lib.MeshDesc2D()
            d.order = self.disc.order
            d.nelements = self.nelements
            d.metric = self.metric.data_ptr()
            d.face_geom = self.face_geom.data_ptr()
            d.gather = self.gather.data_ptr()
            d.weak_diff = self._weak.ctypes.data
            d.strong_diff = self._strong.ctypes.data
            d.lift = self._lift.ctypes.data
            d.face_nodes = self._fnodes.ctypes.data
            return d
        d = _lib.MeshDesc()
        d.order = self.disc.order
        d.nelements = self.nelements
        d.metric = self.metric.data_ptr()
        d.face_geom = self.face_geom.data_ptr()
        d.gather = self.gather.data_ptr()
        d.weak_diff = self._weak.ctypes.data
        d.strong_diff = self._strong.ctypes.data
        d.lift = self._lift.ctypes.data
        d.face_nodes = self._fnodes.ctypes.data
        d.face_partner = self.partner.data_ptr() if self.partner is not None else None
        return d

    def nbytes(self) -> int:
        return sum(t.numel() * t.element_size()
                   for t in (self.metric, self.face_geom, self.gather))


PRECISIONS = {"fp64": _lib.DG_FP64, "fp32-mixed": _lib.DG_FP32_MIXED,
              "fp64-tc": _lib.DG_FP64_TC}


class DevicePlan:
    """One compiled RHS: ``rhs(q, out)`` with q, out of shape (nfields, Nel, Np).

    ``precision``: ``"fp64"`` (FP64 arithmetic throughout), ``"fp64-tc"``
    (FP64 results; with face partners the contractions run on the tensor
    cores as an exact FP64 emulation) or ``"fp32-mixed"`` (FP32
    derivative/flux arithmetic, FP64 state, FP64 Euler pressure recovery and
    FP64 RK accumulation)."""

    def __init__(self, mesh: DeviceMesh, equation: str, params,
                 precision: str = "fp64"):
        if equation not in EQUATIONS:
            raise ValueError(f"unknown equation {equation!r}")
        if precision not in PRECISIONS:
            raise ValueError(f"unknown precision {precision!r}")
        self.mesh = mesh
        self.equation = equation
        self.precision = precision
        self.dim = mesh.dim
        if self.dim == 2 and precision != "fp64":
            raise ValueError("triangle-mesh plans evaluate in FP64 only")
        self.nfields = (NFIELDS_2D if self.dim == 2 else NFIELDS)[equation]
        self.params = tuple(float(p) for p in params)
        L = _lib.lib()
        handle = ctypes.c_void_p()
        parr = (ctypes.c_double * max(1, len(self.params)))(*self.params)
        with torch.cuda.device(mesh.device):
            if self.dim == 2:
                _lib.check(L.dg_plan_create_2d(ctypes.byref(handle), EQUATIONS[equation],
                                               ctypes.byref(mesh.desc()), parr,
                                               len(self.params)))
            else:
                _lib.check(L.dg_plan_create(ctypes.byref(handle), EQUATIONS[equation],
                                            PRECISIONS[precision],
                                            ctypes.byref(mesh.desc()), parr,
                                            len(self.params)))
        self._handle = handle
        self._lib = L

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.nfields, self.mesh.nelements, self.mesh.np_)

    def info(self) -> dict:
        nel = ctypes.c_int64()
        vals = [ctypes.c_int32() for _ in range(5)]
        _lib.check(self._lib.dg_plan_info(self._handle, ctypes.byref(nel),
                                          *[ctypes.byref(v) for v in vals]))
        order, nf, grid, block, smem = (v.value for v in vals)
        shared, tcores, launches = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        owned = ctypes.c_int64()
        _lib.check(self._lib.dg_plan_path(self._handle, ctypes.byref(shared),
                                          ctypes.byref(tcores), ctypes.byref(launches),
                                          ctypes.byref(owned)))
        return dict(nelements=nel.value, order=order, nfields=nf, grid=grid,
                    block=block, smem_bytes=smem, face_shared=bool(shared.value),
                    tensor_cores=bool(tcores.value),
                    launches_per_rhs=launches.value, owned_faces=owned.value)

    @property
    def launches_per_rhs(self) -> int:
        """Kernel launches of one ``rhs`` or ``rk_stage`` call."""
        return self.info()["launches_per_rhs"]

    def _check_tensor(self, x: torch.Tensor, name: str):
        if x.dtype != torch.float64 or x.device != self.mesh.device:
            raise TypeError(f"{name} must be float64 on {self.mesh.device}")
        if tuple(x.shape) != self.shape or not x.is_contiguous():
            raise ValueError(f"{name} must be a contiguous {self.shape} tensor, "
                             f"got {tuple(x.shape)}")

    def rhs(self, q: torch.Tensor, out: torch.Tensor | None = None,
            stream=None) -> torch.Tensor:
        self._check_tensor(q, "state")
        if out is None:
            out = torch.empty_like(q)
        else:
            self._check_tensor(out, "out")
        _lib.check(self._lib.dg_rhs(self._handle, ctypes.c_void_p(q.data_ptr()),
                                    ctypes.c_void_p(out.data_ptr()),
                                    _stream_handle(stream)))
        return out

    def rk_stage(self, q_in: torch.Tensor, q_out: torch.Tensor,
                 res: torch.Tensor, a: float, b: float, dt: float,
                 rhs_unscaled: torch.Tensor | None = None, stream=None) -> None:
        """res = a res + dt L(q_in); q_out = q_in + b res (one fused launch).
        ``rhs_unscaled`` optionally receives L(q_in) before the element scale."""
        for x, name in ((q_in, "q_in"), (q_out, "q_out"), (res, "res")):
            self._check_tensor(x, name)
        rptr = None
        if rhs_unscaled is not None:
            self._check_tensor(rhs_unscaled, "rhs_unscaled")
            rptr = ctypes.c_void_p(rhs_unscaled.data_ptr())
        _lib.check(self._lib.dg_rk_stage(
            self._handle, ctypes.c_void_p(q_in.data_ptr()),
            ctypes.c_void_p(q_out.data_ptr()), ctypes.c_void_p(res.data_ptr()),
            float(a), float(b), float(dt), rptr, _stream_handle(stream)))

    def set_element_scale(self, scale: torch.Tensor | None) -> None:
        """Multiply each element's RHS by ``scale[e]`` (kept referenced)."""
        if scale is not None:
            if (scale.dtype != torch.float64 or scale.device != self.mesh.device
                    or tuple(scale.shape) != (self.mesh.nelements,)
                    or not scale.is_contiguous()):
                raise ValueError("scale must be a contiguous float64 (Nel,) "
                                 "tensor on the plan's device")
        self._scale = scale
        _lib.check(self._lib.dg_plan_set_element_scale(
            self._handle, None if scale is None else ctypes.c_void_p(scale.data_ptr())))

    def adjoint(self, x: torch.Tensor, out: torch.Tensor | None = None,
                scratch: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """``L^T x`` (FP64 wave plans on meshes uploaded with partners)."""
        self._check_tensor(x, "x")
        if out is None:
            out = torch.empty_like(x)
        else:
            self._check_tensor(out, "out")
        n = self.mesh.nelements * 2 * 4 * self.mesh.disc.nfp
        if scratch is None:
            scratch = getattr(self, "_adj_scratch", None)
            if scratch is None or scratch.numel() != n:
                scratch = torch.empty(n, dtype=torch.float64, device=self.mesh.device)
                self._adj_scratch = scratch
        elif scratch.numel() < n or scratch.dtype != torch.float64:
            raise ValueError(f"scratch needs {n} float64 entries")
        _lib.check(self._lib.dg_rhs_adjoint(
            self._handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(scratch.data_ptr()), _stream_handle(stream)))
        return out

    def adjoint_stage(self, x: torch.Tensor, xscale: float, lam: torch.Tensor,
                      rbar_out: torch.Tensor | None, lq: torch.Tensor | None,
                      cbar: torch.Tensor | None, a: float, b: float, dt: float,
                      y_scratch: torch.Tensor, stream=None) -> None:
        """One fused reverse LSRK stage (``dg_rhs_adjoint_stage``):
        ``lam += dt L^T (xscale x)``; ``rbar_out = a xscale x + b lam``;
        ``cbar[e] += dt <xscale x, lq>_e``.  ``x`` may be ``lam`` or
        ``rbar_out`` itself."""
        for t, name in ((x, "x"), (lam, "lam"), (y_scratch, "y_scratch")):
            self._check_tensor(t, name)
        for t, name in ((rbar_out, "rbar_out"), (lq, "lq")):
            if t is not None:
                self._check_tensor(t, name)
        if cbar is not None and (cbar.dtype != torch.float64 or cbar.device != self.mesh.device
                                 or tuple(cbar.shape) != (self.mesh.nelements,)
                                 or not cbar.is_contiguous()):
            raise ValueError("cbar must be a contiguous float64 (Nel,) tensor on the "
                             "plan's device")
        ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())  # noqa: E731
        _lib.check(self._lib.dg_rhs_adjoint_stage(
            self._handle, ptr(x), float(xscale), ptr(lam), ptr(rbar_out), ptr(lq),
            ptr(cbar), float(a), float(b), float(dt), ptr(y_scratch),
            _stream_handle(stream)))

    #: launch variants: bit 0 tensor-core products (fp32-mixed), bit 1 one CTA per
    #: tile; 4 and 5 the tcgen05 kernel (exact digit pairs, 3xTF32), 6 the
    #: 3xTF32 kernel at its other CTA size; 7-10 the tensor-core (mma.sync)
    #: kernel at its other tile shapes (128 or 512 threads, 128 / Np or
    #: 512 / Np elements per tile; variants 1 and 3 use 256 and 256 / Np)
    VARIANTS = {0: "persistent", 1: "tensor-core, persistent", 2: "one CTA per tile",
                3: "tensor-core, one CTA per tile", 4: "tcgen05, persistent",
                5: "tcgen05 3xTF32, persistent", 6: "tcgen05 3xTF32, other CTA size",
                7: "tensor-core, 128-thread tiles, persistent",
                8: "tensor-core, 128-thread tiles, one CTA per tile",
                9: "tensor-core, 512-thread tiles, persistent",
                10: "tensor-core, 512-thread tiles, one CTA per tile"}

    def set_variant(self, variant: int) -> None:
        _lib.check(self._lib.dg_plan_set_variant(self._handle, int(variant)))

    def autotune(self, q: torch.Tensor, reps: int = 3, stream=None,
                 ref: torch.Tensor | None = None,
                 max_rel_l2: float | None = None) -> dict:
        """Time the supported launch variants on state ``q`` and keep the
        fastest; returns ``{"chosen": v, "ms": {variant: ms or None}}``.

        With ``ref`` (a trusted RHS of ``q``, e.g. the FP64 plan's) and
        ``max_rel_l2``, only variants whose result lies within that relative
        L2 distance of ``ref`` compete (the most accurate one is kept if none
        does); the result then also carries ``"rel_l2": {variant: err}``."""
        self._check_tensor(q, "state")
        out = torch.empty_like(q)
        chosen = ctypes.c_int32()
        nv = _lib.NUM_VARIANTS     # the library writes this many entries
        ms = (ctypes.c_float * nv)()
        if ref is None:
            _lib.check(self._lib.dg_plan_autotune(
                self._handle, ctypes.c_void_p(q.data_ptr()),
                ctypes.c_void_p(out.data_ptr()), int(reps), _stream_handle(stream),
                ctypes.byref(chosen), ms))
            errs = None
        else:
            self._check_tensor(ref, "ref")
            if max_rel_l2 is None:
                raise ValueError("max_rel_l2 is required with ref")
            errs = (ctypes.c_double * nv)()
            _lib.check(self._lib.dg_plan_autotune_bounded(
                self._handle, ctypes.c_void_p(q.data_ptr()),
                ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ref.data_ptr()),
                float(max_rel_l2), int(reps), _stream_handle(stream),
                ctypes.byref(chosen), ms, errs))
        res = {"chosen": chosen.value,
               "ms": {self.VARIANTS[v]: (float(ms[v]) if ms[v] >= 0 else None)
                      for v in range(nv)}}
        if errs is not None:
            res["max_rel_l2"] = float(max_rel_l2)
            res["rel_l2"] = {self.VARIANTS[v]: (float(errs[v]) if errs[v] >= 0 else None)
                             for v in range(nv)}
        return res

    def vjp(self, q: torch.Tensor, x: torch.Tensor, out: torch.Tensor | None = None,
            stream=None) -> torch.Tensor:
        """``(dL/dq (q))^T x`` (FP64 wave and Euler plans with face partners)."""
        self._check_tensor(q, "q")
        self._check_tensor(x, "x")
        if out is None:
            out = torch.empty_like(x)
        else:
            self._check_tensor(out, "out")
        _lib.check(self._lib.dg_rhs_vjp(
            self._handle, ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(x.data_ptr()),
            ctypes.c_void_p(out.data_ptr()), _stream_handle(stream)))
        return out

    def vjp_stage(self, q: torch.Tensor, x: torch.Tensor, xscale: float,
                  lam: torch.Tensor, rbar_out: torch.Tensor | None, a: float, b: float,
                  dt: float, y_scratch: torch.Tensor, stream=None) -> None:
        """One fused reverse LSRK stage of the operator linearised at the stage
        input ``q`` (``dg_rhs_vjp_stage``): ``lam += dt (dL/dq)^T (xscale x)``;
        ``rbar_out = a xscale x + b lam``.  ``x`` may be ``lam`` or
        ``rbar_out`` itself."""
        for t, name in ((q, "q"), (x, "x"), (lam, "lam"), (y_scratch, "y_scratch")):
            self._check_tensor(t, name)
        if rbar_out is not None:
            self._check_tensor(rbar_out, "rbar_out")
        ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())  # noqa: E731
        _lib.check(self._lib.dg_rhs_vjp_stage(
            self._handle, ptr(q), ptr(x), float(xscale), ptr(lam), ptr(rbar_out),
            float(a), float(b), float(dt), ptr(y_scratch), _stream_handle(stream)))

    def finish(self, stream=None) -> None:
        _lib.check(self._lib.dg_finish(self._handle, _stream_handle(stream)))

    def close(self) -> None:
        if getattr(self, "_handle", None) is not None and self._handle.value:
            self._lib.dg_plan_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

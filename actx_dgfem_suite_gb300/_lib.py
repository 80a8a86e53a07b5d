"""ctypes binding of ``libdgfem_gb300.so`` (C ABI in ``include/dgfem_gb300.h``).

The library is the only compute path: if it is missing or fails to load,
:func:`lib` raises; nothing falls back to a CPU evaluation.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libdgfem_gb300.so"
_lib = None

#: ABI version this binding is written for (dg_abi_version() of the library)
ABI_VERSION = 7

DG_OK = 0
DG_ERR_ARGUMENT = 1
DG_ERR_UNSUPPORTED = 2
DG_ERR_CUDA = 3
DG_ERR_TIMEOUT = 4
DG_ERR_INDEX = 5

DG_WAVE = 0
DG_EULER = 1
DG_MAXWELL = 2

DG_FP64 = 0
DG_FP32_MIXED = 1
DG_FP64_TC = 2
#: DG_NUM_VARIANTS of the header: entries the autotuners write per call
NUM_VARIANTS = 11

#: every entry point declared in include/dgfem_gb300.h
EXPORTED_SYMBOLS = ("dg_plan_create", "dg_plan_create_2d", "dg_rhs", "dg_rk_stage", "dg_finish",
                    "dg_plan_destroy", "dg_plan_set_element_scale",
                    "dg_rhs_adjoint", "dg_rhs_adjoint_noalloc",
                    "dg_rhs_adjoint_stage", "dg_rhs_vjp", "dg_rhs_vjp_stage",
                    "dg_box_mesh_build",
                    "dg_plan_path", "dg_plan_info", "dg_plan_set_variant",
                    "dg_plan_autotune", "dg_plan_autotune_bounded",
                    "dg_fp64_fma_probe", "dg_wait_probe", "dg_stream_copy",
                    "dg_last_error",
                    "dg_abi_version")


class DGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[dg status {code}] {msg}")
        self.code = code


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("order", ctypes.c_int32),
        ("nelements", ctypes.c_int64),
        ("metric", ctypes.c_void_p),
        ("face_geom", ctypes.c_void_p),
        ("gather", ctypes.c_void_p),
        ("weak_diff", ctypes.c_void_p),
        ("strong_diff", ctypes.c_void_p),
        ("lift", ctypes.c_void_p),
        ("face_nodes", ctypes.c_void_p),
        ("face_partner", ctypes.c_void_p),
    ]


class MeshDesc2D(ctypes.Structure):
    """``dg_mesh2d_desc``: a triangle mesh."""
    _fields_ = [
        ("order", ctypes.c_int32),
        ("nelements", ctypes.c_int64),
        ("metric", ctypes.c_void_p),
        ("face_geom", ctypes.c_void_p),
        ("gather", ctypes.c_void_p),
        ("weak_diff", ctypes.c_void_p),
        ("strong_diff", ctypes.c_void_p),
        ("lift", ctypes.c_void_p),
        ("face_nodes", ctypes.c_void_p),
    ]


class BoxDesc(ctypes.Structure):
    _fields_ = [
        ("order", ctypes.c_int32),
        ("n", ctypes.c_int64 * 3),
        ("a", ctypes.c_double * 3),
        ("b", ctypes.c_double * 3),
        ("corner", ctypes.c_void_p),
        ("nbr", ctypes.c_void_p),
        ("face_vert", ctypes.c_void_p),
        ("face_opp", ctypes.c_void_p),
        ("face_nodes", ctypes.c_void_p),
        ("perm", ctypes.c_void_p),
        ("bary", ctypes.c_void_p),
        ("metric", ctypes.c_void_p),
        ("face_geom", ctypes.c_void_p),
        ("gather", ctypes.c_void_p),
        ("face_partner", ctypes.c_void_p),
        ("nodes", ctypes.c_void_p),
    ]


def library_path() -> Path:
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    """Load the CUDA library (building it first when the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    from actx_dgfem_suite_gb300.csrc import build as _build
    rebuild_error = None
    if _build.is_stale():
        try:
            _build.build()
        except Exception as exc:  # no nvcc: the version check below decides
            if not _LIB_PATH.exists():
                raise RuntimeError(
                    f"{_LIB_PATH.name} is missing and could not be built: {exc}"
                ) from exc
            rebuild_error = exc
    if not _LIB_PATH.exists():
        raise RuntimeError(f"{_LIB_PATH} is missing; run __graft_entry__.build()")
    L = ctypes.CDLL(str(_LIB_PATH))
    L.dg_abi_version.argtypes = []
    L.dg_abi_version.restype = ctypes.c_int32
    found = int(L.dg_abi_version())
    if found != ABI_VERSION:
        why = f" (rebuilding the stale library failed: {rebuild_error})" if rebuild_error else ""
        raise RuntimeError(
            f"{_LIB_PATH.name} has ABI version {found}, this binding needs "
            f"{ABI_VERSION}{why}; run __graft_entry__.build()")
    vp = ctypes.c_void_p
    L.dg_plan_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int32,
                                 ctypes.c_int32, ctypes.POINTER(MeshDesc),
                                 ctypes.POINTER(ctypes.c_double), ctypes.c_int32]
    L.dg_plan_create.restype = ctypes.c_int
    L.dg_plan_create_2d.argtypes = [ctypes.POINTER(vp), ctypes.c_int32,
                                    ctypes.POINTER(MeshDesc2D),
                                    ctypes.POINTER(ctypes.c_double), ctypes.c_int32]
    L.dg_plan_create_2d.restype = ctypes.c_int
    L.dg_rhs.argtypes = [vp, vp, vp, vp]
    L.dg_rhs.restype = ctypes.c_int
    dbl = ctypes.c_double
    L.dg_rk_stage.argtypes = [vp, vp, vp, vp, dbl, dbl, dbl, vp, vp]
    L.dg_rk_stage.restype = ctypes.c_int
    L.dg_plan_set_element_scale.argtypes = [vp, vp]
    L.dg_plan_set_element_scale.restype = ctypes.c_int
    L.dg_rhs_adjoint.argtypes = [vp, vp, vp, vp, vp]
    L.dg_rhs_adjoint.restype = ctypes.c_int
    L.dg_rhs_adjoint_stage.argtypes = [vp, vp, dbl, vp, vp, vp, vp, dbl, dbl, dbl,
                                       vp, vp]
    L.dg_rhs_adjoint_stage.restype = ctypes.c_int
    L.dg_rhs_vjp.argtypes = [vp, vp, vp, vp, vp]
    L.dg_rhs_vjp.restype = ctypes.c_int
    L.dg_rhs_vjp_stage.argtypes = [vp, vp, vp, dbl, vp, vp, dbl, dbl, dbl, vp, vp]
    L.dg_rhs_vjp_stage.restype = ctypes.c_int
    L.dg_rhs_adjoint_noalloc.argtypes = [vp, vp, vp, vp]
    L.dg_rhs_adjoint_noalloc.restype = ctypes.c_int
    L.dg_box_mesh_build.argtypes = [ctypes.POINTER(BoxDesc), vp]
    L.dg_box_mesh_build.restype = ctypes.c_int
    L.dg_finish.argtypes = [vp, vp]
    L.dg_finish.restype = ctypes.c_int
    L.dg_plan_destroy.argtypes = [vp]
    L.dg_plan_destroy.restype = ctypes.c_int
    i32p = ctypes.POINTER(ctypes.c_int32)
    L.dg_plan_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), i32p, i32p,
                               i32p, i32p, i32p]
    L.dg_plan_info.restype = ctypes.c_int
    L.dg_plan_path.argtypes = [vp, i32p, i32p, i32p, ctypes.POINTER(ctypes.c_int64)]
    L.dg_plan_set_variant.argtypes = [vp, ctypes.c_int32]
    L.dg_plan_set_variant.restype = ctypes.c_int
    L.dg_plan_autotune.argtypes = [vp, vp, vp, ctypes.c_int32, vp, i32p,
                                   ctypes.POINTER(ctypes.c_float)]
    L.dg_plan_autotune.restype = ctypes.c_int
    L.dg_plan_autotune_bounded.argtypes = [vp, vp, vp, vp, ctypes.c_double,
                                           ctypes.c_int32, vp, i32p,
                                           ctypes.POINTER(ctypes.c_float),
                                           ctypes.POINTER(ctypes.c_double)]
    L.dg_plan_autotune_bounded.restype = ctypes.c_int
    L.dg_plan_path.restype = ctypes.c_int
    L.dg_fp64_fma_probe.argtypes = [vp, ctypes.c_int64, ctypes.c_int32,
                                    ctypes.c_int32, vp]
    L.dg_fp64_fma_probe.restype = ctypes.c_int
    L.dg_stream_copy.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int32, vp]
    L.dg_stream_copy.restype = ctypes.c_int
    L.dg_wait_probe.argtypes = [ctypes.POINTER(ctypes.c_int32), vp]
    L.dg_wait_probe.restype = ctypes.c_int
    L.dg_last_error.argtypes = []
    L.dg_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def check(code: int) -> None:
    if code != DG_OK:
        msg = lib().dg_last_error().decode(errors="replace")
        raise DGError(code, msg)

"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares; argument validation needs no device."""

import ctypes
import re
from pathlib import Path

import pytest

from actx_dgfem_suite_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]


def _declared_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\*?\s*(dg_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_known_symbols():
    declared = _declared_functions()
    assert declared == set(_lib.EXPORTED_SYMBOLS)


def test_library_exports_all_declared_symbols():
    L = _lib.lib()
    for name in _declared_functions():
        assert hasattr(L, name), name
        assert ctypes.cast(getattr(L, name), ctypes.c_void_p).value


def test_variant_count_matches_the_header():
    from actx_dgfem_suite_gb300.plan import DevicePlan
    text = (ROOT / "include" / "dgfem_gb300.h").read_text()
    m = re.search(r"#define\s+DG_NUM_VARIANTS\s+(\d+)", text)
    assert m and int(m.group(1)) == _lib.NUM_VARIANTS == len(DevicePlan.VARIANTS)


def test_version_and_error_strings():
    L = _lib.lib()
    assert L.dg_abi_version() == 7
    assert isinstance(L.dg_last_error(), bytes)


def test_argument_errors_without_device():
    L = _lib.lib()
    h = ctypes.c_void_p()
    # NULL mesh description -> DG_ERR_ARGUMENT, no CUDA call made
    assert L.dg_plan_create(ctypes.byref(h), 0, 0, None, None, 0) == _lib.DG_ERR_ARGUMENT
    assert b"NULL" in L.dg_last_error()
    d = _lib.MeshDesc()
    d.order = 7
    d.nelements = 10
    assert L.dg_plan_create(ctypes.byref(h), 0, 0, ctypes.byref(d), None, 0) \
        == _lib.DG_ERR_UNSUPPORTED
    assert L.dg_plan_create(ctypes.byref(h), 0, 7, ctypes.byref(d), None, 0) \
        == _lib.DG_ERR_ARGUMENT
    d.order = 2
    assert L.dg_plan_create(ctypes.byref(h), 9, 0, ctypes.byref(d), None, 0) \
        == _lib.DG_ERR_ARGUMENT
    assert L.dg_rk_stage(None, None, None, None, 0.0, 0.0, 0.0, None, None) \
        == _lib.DG_ERR_ARGUMENT
    assert L.dg_rhs(None, None, None, None) == _lib.DG_ERR_ARGUMENT
    assert L.dg_finish(None, None) == _lib.DG_ERR_ARGUMENT
    assert L.dg_plan_destroy(None) == _lib.DG_OK
    assert L.dg_fp64_fma_probe(None, 1, 1, 1, None) == _lib.DG_ERR_ARGUMENT
    assert L.dg_plan_set_element_scale(None, None) == _lib.DG_ERR_ARGUMENT
    assert L.dg_rhs_adjoint(None, None, None, None, None) == _lib.DG_ERR_ARGUMENT
    assert L.dg_rhs_vjp(None, None, None, None, None) == _lib.DG_ERR_ARGUMENT
    assert L.dg_rhs_vjp_stage(None, None, None, 1.0, None, None, 0.0, 0.0, 0.0, None,
                              None) == _lib.DG_ERR_ARGUMENT
    assert L.dg_rhs_adjoint_stage(None, None, 1.0, None, None, None, None, 0.0, 0.0, 0.0,
                                  None, None) == _lib.DG_ERR_ARGUMENT
    assert L.dg_plan_set_variant(None, 0) == _lib.DG_ERR_ARGUMENT
    # triangle meshes: the same argument checks before any CUDA call
    assert L.dg_plan_create_2d(None, 0, None, None, 0) == _lib.DG_ERR_ARGUMENT
    assert L.dg_plan_create_2d(ctypes.byref(h), 0, None, None, 0) == _lib.DG_ERR_ARGUMENT
    d2 = _lib.MeshDesc2D()
    d2.order = 5
    d2.nelements = 10
    assert L.dg_plan_create_2d(ctypes.byref(h), 0, ctypes.byref(d2), None, 0) \
        == _lib.DG_ERR_UNSUPPORTED
    d2.order = 2
    assert L.dg_plan_create_2d(ctypes.byref(h), 9, ctypes.byref(d2), None, 0) \
        == _lib.DG_ERR_ARGUMENT
    assert L.dg_plan_create_2d(ctypes.byref(h), 0, ctypes.byref(d2), None, 0) \
        == _lib.DG_ERR_ARGUMENT           # NULL device arrays
    d2.nelements = (1 << 31) // 6 + 1     # Nel * Np >= 2^31 at P2 (Np = 6)
    assert L.dg_plan_create_2d(ctypes.byref(h), 0, ctypes.byref(d2), None, 0) \
        == _lib.DG_ERR_ARGUMENT
    assert b"2^31" in L.dg_last_error()
    d2.nelements = 0
    assert L.dg_plan_create_2d(ctypes.byref(h), 0, ctypes.byref(d2), None, 0) \
        == _lib.DG_ERR_ARGUMENT
    with pytest.raises(_lib.DGError):
        _lib.check(L.dg_rhs(None, None, None, None))

"""Page-locked host buffers backed by transparent huge pages.

The array context moves states to the GPU and results back through
page-locked host memory.  On the GB300 host (Grace, 64 KB base pages) the
GPU reads and writes that memory through the CPU's page tables over the
NVLink-C2C link, and copies that touch many small pages run far below the
link rate: a first pass over a freshly page-locked 1 GiB buffer measured
18-50 GB/s against 211 GB/s once warm, and with tens of GB of such buffers in
use even warm copies fell to ~64 GB/s.  A region that is advised for huge
pages (``madvise(MADV_HUGEPAGE)``) before it is first touched, and only then
registered with CUDA (``cudaHostRegister``), ran at 211 GB/s host->device and
193 GB/s device->host from its first copy.

Used for states that travel host->device (the first copy out of a freshly
page-locked ``cudaHostAlloc`` buffer is the slow one).  Results travel the
other way in the array context's pool of ``cudaHostAlloc`` buffers, whose
first device->host copy already ran at the link rate (193 GB/s).

:func:`host_empty` returns such a buffer as a CPU tensor (``is_pinned()`` is
true, so ``copy_(..., non_blocking=True)`` is asynchronous); the memory is
unregistered and freed when the tensor and every view of it are gone.  The
advice is only a request: on a host whose memory is too fragmented for huge
pages the region stays on base pages, and copies from it measured 10-22
GB/s.  So after the first touch the region's huge-page backing is read from
``/proc/self/smaps``; below :data:`MIN_HUGE_FRACTION` one synchronous
collapse (``MADV_COLLAPSE``) is asked for, and if the backing is still short
the buffer comes from PyTorch's ``pin_memory`` allocation (``cudaHostAlloc``)
instead, as it does where the advice or the registration is unavailable.
:data:`stats` counts the buffers of each kind.
"""

from __future__ import annotations

import ctypes
import os
import weakref

import numpy as np
import torch

_MADV_HUGEPAGE = 14
_MADV_COLLAPSE = 25
_libc = None
#: least fraction of a region on huge pages for it to be used as registered
MIN_HUGE_FRACTION = 0.9
#: buffers handed out: on huge pages ("huge"), or from cudaHostAlloc
#: ("pinned": huge pages not granted, disabled or unavailable)
stats = {"huge": 0, "pinned": 0}


def huge_page_fraction(addr: int, size: int, smaps_text: str | None = None) -> float:
    """Fraction of [addr, addr + size) backed by transparent huge pages, from
    the ``AnonHugePages`` of the mappings in ``/proc/self/smaps`` that
    overlap it (each weighted by its overlap); 0 if that file is unreadable."""
    if smaps_text is None:
        try:
            with open("/proc/self/smaps") as f:
                smaps_text = f.read()
        except OSError:
            return 0.0
    end = addr + size
    huge = 0.0
    lo = hi = None
    for line in smaps_text.splitlines():
        head = line.split(None, 1)[0] if line else ""
        if "-" in head and not head.endswith(":"):
            try:
                a, b = (int(x, 16) for x in head.split("-"))
            except ValueError:
                continue
            lo, hi = a, b
        elif head == "AnonHugePages:" and lo is not None:
            ov = min(hi, end) - max(lo, addr)
            if ov > 0:
                kb = int(line.split()[1])
                huge += kb * 1024.0 * ov / (hi - lo)
    return huge / size if size > 0 else 0.0


def _huge_page_bytes() -> int:
    try:
        with open("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size") as f:
            return int(f.read().strip())
    except (OSError, ValueError):
        return 2 << 20


def _lib_c():
    global _libc
    if _libc is None:
        _libc = ctypes.CDLL(None, use_errno=True)
        _libc.posix_memalign.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t,
                                         ctypes.c_size_t]
        _libc.posix_memalign.restype = ctypes.c_int
        _libc.madvise.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        _libc.madvise.restype = ctypes.c_int
        _libc.free.argtypes = [ctypes.c_void_p]
        _libc.free.restype = None
    return _libc


def _release(addr: int) -> None:
    try:
        torch.cuda.cudart().cudaHostUnregister(addr)
    finally:
        _lib_c().free(ctypes.c_void_p(addr))


def host_empty(nbytes: int) -> torch.Tensor:
    """A page-locked host buffer of ``nbytes`` bytes (uint8 CPU tensor) on
    huge pages where the system allows them."""
    nbytes = int(nbytes)
    if nbytes <= 0:
        return torch.empty(0, dtype=torch.uint8, pin_memory=True)

    def pinned() -> torch.Tensor:
        stats["pinned"] += 1
        return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)

    if os.environ.get("DG_HOST_HUGE_PAGES", "1") == "0":
        return pinned()
    libc = _lib_c()
    page = 64 << 10
    size = (nbytes + page - 1) // page * page
    ptr = ctypes.c_void_p()
    align = min(_huge_page_bytes(), 1 << 30)
    if libc.posix_memalign(ctypes.byref(ptr), align, size) != 0 or not ptr.value:
        return pinned()
    addr = ptr.value
    libc.madvise(ctypes.c_void_p(addr), size, _MADV_HUGEPAGE)   # advice only
    ctypes.memset(addr, 0, size)                                # fault the pages in now
    if huge_page_fraction(addr, size) < MIN_HUGE_FRACTION:
        libc.madvise(ctypes.c_void_p(addr), size, _MADV_COLLAPSE)  # may be unsupported
        if huge_page_fraction(addr, size) < MIN_HUGE_FRACTION:
            libc.free(ctypes.c_void_p(addr))
            return pinned()
    if int(torch.cuda.cudart().cudaHostRegister(addr, size, 0)) != 0:
        libc.free(ctypes.c_void_p(addr))
        return pinned()
    stats["huge"] += 1
    raw = (ctypes.c_ubyte * size).from_address(addr)
    t = torch.frombuffer(raw, dtype=torch.uint8)[:nbytes]
    # free with the last reference to the memory (tensor views keep `raw`)
    weakref.finalize(raw, _release, addr)
    return t


def host_empty_like(t: torch.Tensor) -> torch.Tensor:
    """A page-locked host tensor with ``t``'s shape and dtype."""
    elt = torch.empty((), dtype=t.dtype).element_size()
    n = int(np.prod(tuple(t.shape), dtype=np.int64))
    return host_empty(n * elt).view(t.dtype).view(tuple(t.shape))

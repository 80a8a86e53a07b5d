"""The array context's result-buffer pool: every result is an independent
array; a buffer is reused (same size) only after its array and all views are
gone.  Plain host memory here (page-locking needs a CUDA device)."""

from __future__ import annotations

import gc

import numpy as np
import torch

from actx_dgfem_suite_gb300.array_context import PinnedResultPool


def _free(pool):
    return sum(len(v) for v in pool._free.values())


def test_results_are_independent_and_buffers_return_after_all_views():
    pool = PinnedResultPool(pin=False)
    a, ta = pool.take((3, 4), torch.float64)
    b, tb = pool.take((3, 4), torch.float64)
    ta.fill_(1.0)
    tb.fill_(2.0)
    assert not np.shares_memory(a, b) and a.sum() == 12 and b.sum() == 24
    assert pool.allocated_bytes == 2 * 96
    view = a[1]
    del a, ta
    gc.collect()
    assert _free(pool) == 0            # a view still holds the buffer
    del view
    gc.collect()
    assert _free(pool) == 1
    c, _ = pool.take((4, 3), torch.float64)   # same byte size: reused
    assert _free(pool) == 0 and pool.allocated_bytes == 2 * 96
    d, _ = pool.take((5,), torch.float32)     # other size: allocated
    assert pool.allocated_bytes == 2 * 96 + 20
    del b, tb, c, d
    gc.collect()
    pool.release()
    assert _free(pool) == 0 and pool.allocated_bytes == 0

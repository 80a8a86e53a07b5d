"""Host states through the compiled callable: uploads on the context's
host-to-device stream, results read back on its device-to-host stream, with
several calls in flight before any result is read."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_calls_in_flight_with_host_states(actx):
    from actx_dgfem_suite_gb300.containers import from_stacked, leaves
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs
    cases = [("wave", 3, 4), ("euler", 2, 5), ("maxwell", 4, 3), ("wave", 1, 6)]
    calls, host_args, refs = [], [], []
    for eq, order, n in cases:
        rhs, args = get_rhs(eq, actx, 3, order, definition="baseline", nel_1d=n)
        compiled = actx.compile(rhs)
        q = compiled.stage(args[-1])
        refs.append(compiled.plan.rhs(q).cpu().numpy())
        hq = q.cpu().pin_memory()
        calls.append(compiled)
        host_args.append(args[:-1] + (from_stacked(actx, args[-1], hq),))
    torch.cuda.synchronize()
    for _ in range(3):  # the same callables again: their staging buffers are reused
        outs = [c(*a) for c, a in zip(calls, host_args)]       # all in flight
        got = [np.stack([d[0] for d in leaves(actx.to_numpy(o))]) for o in outs]
        for g, r in zip(got, refs):
            assert np.array_equal(g, r)
    # batched readback: the same arrays, one wait; containers and bare tensors
    for _ in range(2):
        outs = [c(*a) for c, a in zip(calls, host_args)]
        got = actx.to_numpy_batch(outs + [outs[0]])
        for g, r in zip(got, refs + refs[:1]):
            assert np.array_equal(np.stack([d[0] for d in leaves(g)]), r)
    t = torch.arange(12.0, dtype=torch.float64, device=actx.device).reshape(3, 4)
    assert np.array_equal(actx.to_numpy_batch([t])[0], t.cpu().numpy())
    # a state that changes between calls reaches the kernel each time
    c, a = calls[0], host_args[0]
    hq = leaves(a[-1])[0]._stack[0]
    for scale in (2.0, -0.5):
        hq.mul_(scale)
        out = np.stack([d[0] for d in leaves(actx.to_numpy(c(*a)))])
        want = c.plan.rhs(hq.to(actx.device)).cpu().numpy()
        assert np.array_equal(out, want)


def test_pinned_host_buffers(actx):
    """pinned_host_like: page-locked (huge-page backed where available) host
    tensors that round-trip through asynchronous copies, freed with their
    last view."""
    import gc
    dev = torch.arange(3 * 1000 * 35, dtype=torch.float64, device=actx.device).view(3, 1000, 35)
    h = actx.pinned_host_like(dev)
    assert h.is_pinned() and h.shape == dev.shape and h.dtype == dev.dtype
    h.copy_(dev, non_blocking=True)
    torch.cuda.synchronize()
    back = torch.empty_like(dev)
    back.copy_(h, non_blocking=True)
    torch.cuda.synchronize()
    assert torch.equal(back, dev)
    view = h[1]
    del h
    gc.collect()
    assert float(view[0, 0]) == 35000.0      # a view keeps the memory alive
    del view
    gc.collect()


def test_result_readback_waits_only_for_its_own_call(actx):
    """to_numpy of a compiled call's result waits for that call's kernels,
    not for work queued after them: a long kernel issued after the call is
    still running when the result is already on the host."""
    import ctypes

    from actx_dgfem_suite_gb300 import _lib
    from actx_dgfem_suite_gb300.containers import leaves
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs
    rhs, args = get_rhs("wave", actx, 3, 2, definition="baseline", nel_1d=4)
    compiled = actx.compile(rhs)
    ref = np.stack([d[0] for d in leaves(actx.to_numpy(compiled(*args)))])
    out = compiled(*args)
    # then about half a second of FP64 FMAs on the same stream
    L = _lib.lib()
    nsm = torch.cuda.get_device_properties(actx.device).multi_processor_count
    buf = torch.empty(nsm * 4 * 256, dtype=torch.float64, device=actx.device)
    stream = torch.cuda.current_stream(actx.device)
    _lib.check(L.dg_fp64_fma_probe(ctypes.c_void_p(buf.data_ptr()), 200000, nsm * 4, 256,
                                   ctypes.c_void_p(stream.cuda_stream)))
    long_done = torch.cuda.Event()
    long_done.record(stream)
    got = np.stack([d[0] for d in leaves(actx.to_numpy(out))])
    still_running = not long_done.query()
    torch.cuda.synchronize()
    assert np.array_equal(got, ref)
    assert still_running


def test_batched_readback_pageable_and_host_inputs():
    """to_numpy_batch with pageable results (pinned_results=False), and with
    host tensors among the inputs (returned as they are)."""
    from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext
    from actx_dgfem_suite_gb300.containers import leaves
    from actx_dgfem_suite_gb300.rhs_builder import get_rhs
    ctx = GB300DGArrayContext("cuda:0", pinned_results=False)
    rhs, args = get_rhs("euler", ctx, 3, 2, definition="baseline", nel_1d=3)
    compiled = ctx.compile(rhs)
    outs = [compiled(*args) for _ in range(3)]
    ref = np.stack([d[0] for d in leaves(ctx.to_numpy(outs[0]))])
    got = ctx.to_numpy_batch(outs)
    for g in got:
        assert np.array_equal(np.stack([d[0] for d in leaves(g)]), ref)
    h = torch.arange(6.0, dtype=torch.float64)
    assert np.array_equal(ctx.to_numpy_batch([h])[0], h.numpy())

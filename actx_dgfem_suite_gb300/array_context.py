"""``GB300DGArrayContext``: the drop-in array context for the suite's RHS
operators on one GB300 GPU.

It plays the role the reference's array contexts play behind
``_NAME_TO_ACTX_CLASS`` (``actx_dgfem_suite/run/__main__.py:209-216``):
``actx.compile(rhs)`` returns a callable, ``compiled(*args)`` evaluates the RHS
and returns the same container type, ``actx.to_numpy`` brings results to the
host (``actx_dgfem_suite/run/__main__.py:73-96``).  Unlike the tracing
contexts, ``compile`` does not trace grudge code: it recognises the operator
objects built by :mod:`actx_dgfem_suite_gb300.rhs_builder` and binds them to a
:class:`~actx_dgfem_suite_gb300.plan.DevicePlan`, i.e. to the hand-written
sm_103a kernels.  There is no CPU path: constructing the context without a CUDA
device, or without the compiled library, raises.
"""

from __future__ import annotations

import weakref
from typing import Any

import numpy as np
import torch

from actx_dgfem_suite_gb300 import _lib
from actx_dgfem_suite_gb300.containers import (
    DOFArray,
    from_stacked,
    leaves,
    map_leaves,
)
from actx_dgfem_suite_gb300.hostmem import host_empty_like
from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan


class _ActxNumpy:
    """``actx.np``: elementwise functions over DOFArrays and containers."""

    def __init__(self, actx):
        self._actx = actx

    def _unary(self, f, x):
        if isinstance(x, DOFArray):
            return x.map(f)
        if isinstance(x, torch.Tensor):
            return f(x)
        return map_leaves(x, lambda d: d.map(f))

    def exp(self, x):
        return self._unary(torch.exp, x)

    def sqrt(self, x):
        return self._unary(torch.sqrt, x)

    def sin(self, x):
        return self._unary(torch.sin, x)

    def cos(self, x):
        return self._unary(torch.cos, x)

    def abs(self, x):
        return self._unary(torch.abs, x)

    def real(self, x):
        return self._unary(lambda a: a.real if a.is_complex() else a, x)

    def maximum(self, a, b):
        return a._map2(b, lambda u, v: torch.maximum(u, v if torch.is_tensor(v)
                                                      else torch.as_tensor(v, dtype=u.dtype, device=u.device)))

    def minimum(self, a, b):
        return a._map2(b, lambda u, v: torch.minimum(u, v if torch.is_tensor(v)
                                                      else torch.as_tensor(v, dtype=u.dtype, device=u.device)))


def _timing_event(stream) -> torch.cuda.Event:
    ev = torch.cuda.Event(enable_timing=True)
    ev.record(stream)
    return ev


class CompiledRHS:
    """``actx.compile(rhs)``: evaluates the RHS through one DevicePlan.

    A state held on the host is copied on the context's host-to-device
    stream into a device buffer owned by this callable (reused by every call
    whose state is on the host; the copy of call n+1 waits only for the
    kernel of call n that read the buffer), and the RHS kernel on the current
    stream waits for that copy alone.  So a caller that issues several calls
    before reading results back (``to_numpy``) overlaps the copies of one
    call with the kernels of another.  As with any asynchronous array
    context, the host state must not change until the call's result has been
    read or the stream synchronised."""

    def __init__(self, actx: GB300DGArrayContext, op):
        self.actx = actx
        self.op = op
        self.plan: DevicePlan = op.plan_for(actx)
        self._in_buf: torch.Tensor | None = None
        self._in_free: torch.cuda.Event | None = None  # last read of _in_buf

    def _upload(self, host: torch.Tensor) -> torch.Tensor:
        dev = self.actx.device
        cur = torch.cuda.current_stream(dev)
        if (self._in_buf is None or self._in_buf.shape != host.shape):
            self._in_buf = torch.empty(host.shape, dtype=torch.float64, device=dev)
            self._in_free = None
        h2d = self.actx.h2d_stream
        if self._in_free is not None:
            h2d.wait_event(self._in_free)
        else:
            h2d.wait_stream(cur)          # the buffer's allocation
        log = self.actx.transfer_log
        t0 = _timing_event(h2d) if log is not None else None
        with torch.cuda.stream(h2d):
            self._in_buf.copy_(host, non_blocking=True)
        if log is not None:
            log.append(("h2d", t0, _timing_event(h2d), host.numel() * host.element_size()))
        ready = torch.cuda.Event()
        ready.record(h2d)
        cur.wait_event(ready)
        return self._in_buf

    def stage(self, state) -> torch.Tensor:
        """The (nfields, Nel, Np) device tensor holding ``state``; no copy
        when the state is already a view of such a tensor on the device."""
        lv = leaves(state)
        st = lv[0]._stack
        if (st is not None and st[0].shape[0] == len(lv)
                and all(d._stack is not None and d._stack[0] is st[0]
                        and d._stack[1] == k for k, d in enumerate(lv))):
            base = st[0]
            if base.device == self.actx.device and base.is_contiguous():
                return base
            if base.device.type == "cpu":
                return self._upload(base)
            return base.to(self.actx.device)
        arrs = [torch.as_tensor(d[0]) for d in lv]
        if all(a.device == self.actx.device for a in arrs):
            return torch.stack(arrs)
        return self._upload(torch.stack([a.cpu() for a in arrs]))

    def __call__(self, *args, out: torch.Tensor | None = None):
        state = args[self.op.state_argnum]
        q = self.stage(state)
        res = self.plan.rhs(q, out)
        cur = torch.cuda.current_stream(self.actx.device)
        done = torch.cuda.Event()
        done.record(cur)
        if q is self._in_buf:
            self._in_free = done
        res._dg_ready = done              # what to_numpy waits for
        return from_stacked(self.actx, state, res)


class PinnedResultPool:
    """Page-locked host buffers for results, reused by exact size.

    ``take`` returns a new array backed by a free buffer of that byte size
    (allocating one only when every buffer of that size is in use); when the
    array and all its views have been garbage-collected, the buffer goes back
    to the pool.  Page-locking a fresh block costs about as much as copying
    it several times over, and a copy into freshly allocated pageable memory
    is limited by first-touch page faults, so steady-state transfers need
    resident, reused buffers; callers still get independent arrays."""

    def __init__(self, pin: bool = True):
        self.pin = pin                  # page-locked (False: plain host memory)
        self._free: dict[int, list[torch.Tensor]] = {}
        self.allocated_bytes = 0

    def _give(self, nbytes: int, buf: torch.Tensor) -> None:
        self._free.setdefault(nbytes, []).append(buf)

    def take(self, shape, dtype: torch.dtype) -> tuple[np.ndarray, torch.Tensor]:
        view_t = torch.empty((), dtype=dtype)
        nbytes = int(np.prod(shape, dtype=np.int64)) * view_t.element_size()
        free = self._free.get(nbytes)
        if free:
            buf = free.pop()
        else:
            buf = torch.empty(nbytes, dtype=torch.uint8, pin_memory=self.pin)
            self.allocated_bytes += nbytes
        t = buf.view(dtype).view(shape)
        arr = t.numpy()
        weakref.finalize(arr, self._give, nbytes, buf)
        return arr, t

    def release(self) -> None:
        """Drop the free buffers (buffers of live arrays stay with them)."""
        self.allocated_bytes -= sum(b.numel() for lst in self._free.values() for b in lst)
        self._free.clear()


class GB300DGArrayContext:
    """Array context running the suite's RHS operators on one GB300."""

    def __init__(self, device: str | int | torch.device | None = None,
                 pinned_results: bool = True):
        if not torch.cuda.is_available():
            raise RuntimeError("GB300DGArrayContext needs a CUDA device; "
                               "there is no CPU fallback")
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("GB300DGArrayContext runs on CUDA devices only")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        _lib.lib()  # load the kernels now, so a missing library fails here
        self.pinned_results = bool(pinned_results)
        self.host_pool = PinnedResultPool()
        self.np = _ActxNumpy(self)
        self._meshes: dict[int, DeviceMesh] = {}
        # copy streams: host states in, results out, beside the compute stream
        self.h2d_stream = torch.cuda.Stream(self.device)
        self.d2h_stream = torch.cuda.Stream(self.device)
        #: a list to record every host<->device copy of compiled calls and
        #: to_numpy in, as (direction, start event, end event, bytes) with
        #: timing events on the copy streams; None (default) records nothing
        self.transfer_log: list | None = None

    # {{{ device data

    def device_mesh(self, disc) -> DeviceMesh:
        key = id(disc)
        if key not in self._meshes:
            self._meshes[key] = DeviceMesh(disc, self.device)
        return self._meshes[key]

    def from_numpy(self, x):
        if isinstance(x, np.ndarray) and x.dtype != object:
            return torch.from_numpy(np.ascontiguousarray(x)).to(self.device)
        if isinstance(x, DOFArray):
            return DOFArray(self, [self.from_numpy(a) for a in x])
        return map_leaves(x, lambda d: DOFArray(self, [self.from_numpy(np.asarray(a)) for a in d]))

    def _host(self, t: torch.Tensor) -> np.ndarray:
        """A new host array holding ``t``.  Device tensors are copied into a
        page-locked buffer of ``host_pool``: a fresh pageable array would be
        faulted in page by page during the copy (~25 GB/s on a Grace host
        against ~190 GB/s into resident memory), and page-locking a fresh
        block costs more than the copy, so buffers are reused by size and
        return to the pool when the caller drops the array.
        ``pinned_results=False`` keeps plain pageable arrays."""
        arr, pending = self._host_issue(t)
        if pending:
            self.d2h_stream.synchronize()
        return arr

    def _host_issue(self, t: torch.Tensor) -> tuple[np.ndarray, bool]:
        """Start the copy of ``t`` into a new host array; the array is valid
        once the device-to-host stream has drained (the flag says whether a
        copy is pending)."""
        # the event after the kernel that produced t (a compiled call's
        # result), read before detach(), whose new tensor object carries no
        # Python attributes
        ready = getattr(t, "_dg_ready", None)
        if ready is None and t._base is not None:
            ready = getattr(t._base, "_dg_ready", None)
        t = t.detach()
        if not t.is_cuda:
            return t.numpy(), False
        if not self.pinned_results:
            return t.cpu().numpy(), False
        arr, h = self.host_pool.take(tuple(t.shape), t.dtype)
        # the copy runs on the device-to-host stream and waits only for that
        # kernel, so kernels the caller issued after it keep running meanwhile
        d2h = self.d2h_stream
        if ready is not None:
            d2h.wait_event(ready)
        else:
            d2h.wait_stream(torch.cuda.current_stream(t.device))
        log = self.transfer_log
        t0 = _timing_event(d2h) if log is not None else None
        with torch.cuda.stream(d2h):
            h.copy_(t, non_blocking=True)
        if log is not None:
            log.append(("d2h", t0, _timing_event(d2h), t.numel() * t.element_size()))
        t.record_stream(d2h)
        return arr, True

    def pinned_host_like(self, t: torch.Tensor) -> torch.Tensor:
        """A page-locked host tensor shaped like ``t`` (on huge pages where
        the system allows), for states a caller stages on the host: the
        context's copies to and from such buffers run at the link rate."""
        return host_empty_like(t)

    def release_host_buffers(self) -> None:
        """Return the pool's free page-locked result buffers to the system."""
        self.host_pool.release()

    def to_numpy(self, x):
        return self._to_numpy(x, self._host)

    def to_numpy_batch(self, xs) -> list:
        """``[to_numpy(x) for x in xs]`` with one wait: every copy is issued
        on the device-to-host stream behind its own kernel, then the stream is
        drained once, so the host neither waits between copies nor holds the
        copies back while it runs (a stall of the calling thread after the
        copies are issued does not delay them).  The copies also wait for the
        host-to-device copies issued before them, so that the two directions
        do not compete for the host's memory bandwidth while the uploads the
        kernels need are still running."""
        self.d2h_stream.wait_stream(self.h2d_stream)
        pending = [False]

        def issue(t):
            arr, p = self._host_issue(t)
            pending[0] |= p
            return arr

        out = [self._to_numpy(x, issue) for x in xs]
        if pending[0]:
            self.d2h_stream.synchronize()
        return out

    def _to_numpy(self, x, host):
        if isinstance(x, torch.Tensor):
            return host(x)
        if isinstance(x, DOFArray):
            if x._stack is not None:
                h = host(x._stack[0])
                return DOFArray(None, [h[x._stack[1]]])
            return DOFArray(None, [self._to_numpy(a, host) for a in x])
        lv = leaves(x)
        st = lv[0]._stack
        if st is not None and all(d._stack is not None and d._stack[0] is st[0]
                                  for d in lv):
            h = host(st[0])   # one device->host copy
            return map_leaves(x, lambda d: DOFArray(None, [h[d._stack[1]]]))
        return map_leaves(x, lambda d: self._to_numpy(d, host))

    def zeros(self, shape, dtype=torch.float64):
        return torch.zeros(shape, dtype=dtype, device=self.device)

    # }}}

    # {{{ freeze / thaw: device tensors carry no queue, only the context tag

    def freeze(self, x):
        if isinstance(x, DOFArray):
            return DOFArray(None, list(x), stack=x._stack)
        return map_leaves(x, lambda d: DOFArray(None, list(d), stack=d._stack))

    def thaw(self, x):
        if isinstance(x, DOFArray):
            return DOFArray(self, list(x), stack=x._stack)
        return map_leaves(x, lambda d: DOFArray(self, list(d), stack=d._stack))

    def freeze_thaw(self, x):
        return self.thaw(self.freeze(x))

    # }}}

    def compile(self, f) -> CompiledRHS:
        op = getattr(f, "dg_operator", None)
        if op is None:
            raise NotImplementedError(
                "GB300DGArrayContext compiles the RHS operators built by "
                "actx_dgfem_suite_gb300.rhs_builder.get_rhs; got "
                f"{type(f).__name__}")
        return CompiledRHS(self, op)

    def finish(self) -> None:
        torch.cuda.synchronize(self.device)

    def clone(self) -> GB300DGArrayContext:
        return type(self)(self.device)

    def __repr__(self) -> str:
        return f"GB300DGArrayContext(device={self.device})"


def stacked_state(actx: GB300DGArrayContext, template: Any, fields):
    """Fields (nfields, Nel, Np) as one device tensor -- uploaded when given
    on the host -- and a container of views shaped like ``template``."""
    if isinstance(fields, torch.Tensor):
        dev = fields.to(device=actx.device, dtype=torch.float64).contiguous()
    else:
        dev = torch.from_numpy(np.ascontiguousarray(fields, dtype=np.float64)).to(actx.device)
    return from_stacked(actx, template, dev)

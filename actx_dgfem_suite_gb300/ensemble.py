"""Batched evaluation of many independent ensemble members.

Members may live on meshes of different sizes.  Their discretisations are
concatenated into one union (``discretization.union_discretization``), so one
persistent launch of the RHS kernel covers every member: the kernel's tile
loop balances uneven members automatically and no member-level control flow
exists on the device.  The launch can be captured in a CUDA graph and
replayed once per RHS.

The reference has no ensemble path; this is the batched form asked of the
GB300 build (64 Maxwell P3 members on boxes with n ~ U[12, 40]).
"""

from __future__ import annotations

import numpy as np
import torch

from actx_dgfem_suite_gb300.discretization import (DGDiscretization,
                                                   union_discretization)
from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan


class Ensemble:
    """``rhs(q)`` for all members at once; ``q`` is (nfields, sum Nel, Np)."""

    def __init__(self, discs: list, equation: str, params,
                 precision: str = "fp32-mixed", device=None):
        if isinstance(getattr(discs[0], "metric", None), torch.Tensor):
            from actx_dgfem_suite_gb300.device_setup import device_union
            self.union, self.offsets = device_union(discs)   # built on the GPU
        else:
            self.union, self.offsets = union_discretization(discs)
        self.nmembers = len(discs)
        self.mesh = DeviceMesh(self.union, device)
        self.plan = DevicePlan(self.mesh, equation, params, precision)
        self._graph = None
        self._gq = None
        self._gout = None

    @property
    def shape(self):
        return self.plan.shape

    def autotune(self, q: torch.Tensor, reps: int = 3,
                 max_rel_l2: float | None = None) -> dict:
        """Pick the launch variant of the batched kernel (CUDA-core or
        ``mma.sync`` products, the latter at three tile shapes of 128, 256
        or 512 threads and as many nodes per tile; persistent or
        one-CTA-per-tile grid; tcgen05 exact-digit or 3xTF32 products, the
        latter at two CTA sizes) by timing it on the ensemble state ``q``;
        call before :meth:`capture`.
        With ``max_rel_l2``, only variants whose result lies within that
        relative L2 distance of the FP64 RHS of ``q`` (evaluated here by an
        FP64 plan on the same union mesh) compete."""
        ref = None
        if max_rel_l2 is not None:
            p64 = DevicePlan(self.mesh, self.plan.equation, self.plan.params, "fp64")
            ref = p64.rhs(q)
            p64.finish()
            p64.close()
        self.tuning = self.plan.autotune(q, reps, ref=ref, max_rel_l2=max_rel_l2)
        return self.tuning

    def member(self, x: torch.Tensor, k: int) -> torch.Tensor:
        """View of member ``k`` in an ensemble-shaped tensor."""
        return x[:, int(self.offsets[k]):int(self.offsets[k + 1]), :]

    def stack_states(self, states: list) -> torch.Tensor:
        if len(states) != self.nmembers:
            raise ValueError("one state per member expected")
        if isinstance(states[0], torch.Tensor):
            return torch.cat([s.to(self.mesh.device) for s in states], dim=1).contiguous()
        return torch.from_numpy(np.concatenate(states, axis=1)).to(self.mesh.device)

    def rhs(self, q: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        return self.plan.rhs(q, out)

    def capture(self, q: torch.Tensor, out: torch.Tensor) -> None:
        """Capture ``out = L(q)`` as a CUDA graph bound to these tensors."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.plan.rhs(q, out)
        torch.cuda.current_stream().wait_stream(s)
        self._graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self._graph):
            self.plan.rhs(q, out)
        self._gq, self._gout = q, out

    def replay(self) -> torch.Tensor:
        if self._graph is None:
            raise RuntimeError("capture() first")
        self._graph.replay()
        return self._gout


def random_box_sizes(nmembers: int, lo: int, hi: int, seed: int = 0) -> list[int]:
    """Elements per axis of each member, uniform in [lo, hi] from ``seed``."""
    rng = np.random.default_rng(seed)
    return [int(x) for x in rng.integers(lo, hi + 1, size=nmembers)]

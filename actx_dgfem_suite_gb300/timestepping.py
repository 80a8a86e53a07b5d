"""Low-storage Runge-Kutta time integration on the device.

Carpenter & Kennedy's five-stage, fourth-order low-storage scheme (NASA TM
109112, 1994), the integrator of the suite's hand-written baseline
(libparanumal's LSERK4, ``assets/h200nvl.patch``).  Each stage is one fused
launch of the RHS kernel (``dg_rk_stage``): the residual and the state update
happen in the kernel epilogue, so a stage reads the state and residual once and
writes them once.  The reference itself only evaluates RHS operators; its
time-step hook is ``estimate_rk4_timestep`` (``actx_dgfem_suite/equations/wave.py:206-213``).
"""

from __future__ import annotations

import numpy as np
import torch

from actx_dgfem_suite_gb300.discretization import DGDiscretization
from actx_dgfem_suite_gb300.plan import DevicePlan

#: LSRK(5,4) coefficients, Carpenter & Kennedy (1994), solution 3
RK4A = (0.0,
        -567301805773.0 / 1357537059087.0,
        -2404267990393.0 / 2016746695238.0,
        -3550918686646.0 / 2091501179385.0,
        -1275806237668.0 / 842570457699.0)
RK4B = (1432997174477.0 / 9575080441755.0,
        5161836677717.0 / 13612068292357.0,
        1720146321549.0 / 2090206949498.0,
        3134564353537.0 / 4481467310338.0,
        2277821191437.0 / 14882151754819.0)
RK4C = (0.0,
        1432997174477.0 / 9575080441755.0,
        2526269341429.0 / 6820363962896.0,
        2006345519317.0 / 3224310063776.0,
        2802321613138.0 / 2924317926251.0)


def estimate_rk4_timestep(disc: DGDiscretization, c: float = 1.0,
                          cfl: float = 1.0) -> float:
    """Stable step estimate for the explicit RK4 family: the smallest
    element inradius times the smallest reference node spacing ratio, over
    the wave speed ``c``.  Plays the role of grudge's
    ``characteristic_lengthscales`` / ``nodal_min`` used by
    ``actx_dgfem_suite/equations/wave.py:206-213`` (the constants differ)."""
    # inradius = 3 vol / area = 2 / sum_f (sJ_f / J) on the biunit tetrahedron
    # (reference volume 4/3, reference face area 2); works for host meshes
    # and for device-built ones, whose face geometry holds sJ/J directly
    fg = getattr(disc, "face_geom", None)
    if isinstance(fg, torch.Tensor):
        ratio_sum = float(fg[:, :, 3].sum(dim=1).max())
    else:
        ratio_sum = float((disc.face_jac / disc.jac[:, None]).sum(axis=1).max())
    inradius_min = 2.0 / ratio_sum
    x = disc.ref.nodes
    d = np.linalg.norm(x[:, None, :] - x[None, :, :], axis=2)
    dmin = d[d > 0].min() / 2.0       # biunit element: edge length 2
    return float(cfl * inradius_min * dmin / c)


class LSRK45:
    """Integrates ``dq/dt = L(q)`` with one plan; buffers allocated once.

    ``step(q)`` advances ``q`` (a device (nfields, Nel, Np) FP64 tensor) in
    place by one step of size ``dt``.  Set ``use_graph=True`` to capture the
    five stage launches in a CUDA graph and replay it each step."""

    def __init__(self, plan: DevicePlan, dt: float, use_graph: bool = False):
        self.plan = plan
        self.dt = float(dt)
        shape = plan.shape
        dev = plan.mesh.device
        self._buf = torch.empty(shape, dtype=torch.float64, device=dev)
        self.res = torch.zeros(shape, dtype=torch.float64, device=dev)
        self.use_graph = use_graph
        self._graph = None
        self._q_static = None

    def _stages(self, q: torch.Tensor) -> None:
        """Five fused stages; the state ping-pongs between ``q`` and the
        scratch buffer and ends in ``q`` (the last stage writes back)."""
        src, dst = q, self._buf
        for s in range(5):
            self.plan.rk_stage(src, dst, self.res, RK4A[s], RK4B[s], self.dt)
            src, dst = dst, src
        # after 5 (odd) stages the result sits in the scratch buffer
        q.copy_(src)

    def step(self, q: torch.Tensor) -> torch.Tensor:
        if not self.use_graph:
            self._stages(q)
            return q
        if self._graph is None:
            self._q_static = q
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                self._stages(q)          # warm-up outside the capture
            torch.cuda.current_stream().wait_stream(s)
            self._graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self._graph):
                self._stages(q)
            return q                     # the capture did not advance q
        if q.data_ptr() != self._q_static.data_ptr():
            raise ValueError("a captured LSRK45 graph is bound to one state tensor")
        self._graph.replay()
        return q

    def run(self, q: torch.Tensor, nsteps: int, callback=None) -> torch.Tensor:
        for k in range(nsteps):
            self.step(q)
            if callback is not None:
                callback(k + 1, q)
        return q

"""Gradients of a receiver misfit through the wave time integration.

Forward model: the suite's wave operator (``actx_dgfem_suite/equations/wave.py:121-200``)
with a per-element wave speed, ``dq/dt = diag(c_e) L q`` (the operator is linear
in c, so a per-element speed is a per-element factor on the RHS), integrated
with LSRK(5,4) in fused stage launches; receivers sample ``u`` after every
step.  The gradient of any loss of the receiver traces with respect to the
initial state and to ``c_e`` is the discrete adjoint of those steps:

* the operator transpose ``L^T`` is the hand-written adjoint kernel
  (``dg_rhs_adjoint``: transposed D and LIFT, face-gather transpose as a
  deterministic gather over glued face points);
* the reverse of one LSRK step needs only the stage RHS of the forward step
  before the element scale (``L_1 q^(s)``, for the c-gradient term
  ``<rbar, L_1 q>``), which the forward stages write as they recompute the
  step (``rhs_unscaled`` of ``dg_rk_stage``) into buffers allocated once;
  each reverse stage is one fused pair of launches
  (``dg_rhs_adjoint_stage``: the transpose, the state-adjoint update, the
  next residual adjoint and the per-element c-gradient inner products).

Checkpointing (``checkpointing=``):

* ``"binomial"``: Revolve-type binomial checkpointing with
  ``ceil(sqrt(N))`` state slots (:mod:`actx_dgfem_suite_gb300.checkpointing`);
  the forward sweep keeps the states the schedule stores first, the reverse
  sweep recomputes the rest, and each reversed step records its 5 stage
  RHS only while it is being reversed.  Memory: sqrt(N) + 5 states;
  about three forward steps per reversed step at N = 300.
* ``"segments"`` (default): states every ``k`` steps, segments replayed once
  with all their 5 k stage RHS kept; memory ``N/k + 5k`` states, minimal at
  ``k = sqrt(N / 5)``; each forward step recomputed exactly once, so the
  reverse sweep costs one forward sweep plus the adjoint operators.  The
  binomial schedule trades about two more forward steps per step for a
  third of the memory (measured by ``tools/bench_adjoint.py``).

:class:`WaveMisfitFunction` wraps this as a ``torch.autograd.Function``.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from actx_dgfem_suite_gb300.checkpointing import BinomialSchedule, default_slots
from actx_dgfem_suite_gb300.discretization import DGDiscretization
from actx_dgfem_suite_gb300.plan import DeviceMesh, DevicePlan
from actx_dgfem_suite_gb300.refelem import BIUNIT_TET_VERTICES, pkdo_tet
from actx_dgfem_suite_gb300.timestepping import RK4A, RK4B


# {{{ receivers


def locate_points(disc: DGDiscretization, points: np.ndarray, tol: float = 1e-10):
    """Element index and reference coordinates of each point (brute force
    over elements, vectorised; for test- and benchmark-sized point sets)."""
    ev = disc.mesh.vertices[disc.mesh.elements]              # (Nel, 4, 3)
    jm = np.stack([ev[:, 1] - ev[:, 0], ev[:, 2] - ev[:, 0], ev[:, 3] - ev[:, 0]],
                  axis=2)                                    # (Nel, x, k)
    jinv = np.linalg.inv(jm)
    elems = np.empty(len(points), dtype=np.int64)
    bary = np.empty((len(points), 4))
    for p, x in enumerate(points):
        lam = np.einsum("ekx,ex->ek", jinv, x[None, :] - ev[:, 0])  # (Nel, 3)
        l0 = 1.0 - lam.sum(axis=1)
        inside = np.all(lam >= -tol, axis=1) & (l0 >= -tol)
        cand = np.nonzero(inside)[0]
        if cand.size == 0:
            raise ValueError(f"point {x} is outside the mesh")
        e = cand[0]
        elems[p] = e
        bary[p] = np.concatenate([[l0[e]], lam[e]])
    ref = bary @ BIUNIT_TET_VERTICES
    return elems, ref


class Receivers:
    """Point samples of the first field: ``trace = sum_i w_i u[e, i]``."""

    def __init__(self, disc: DGDiscretization, points: np.ndarray, device):
        elems, ref = locate_points(disc, np.asarray(points, dtype=np.float64))
        vinv = np.linalg.inv(disc.ref.vdm)
        w = pkdo_tet(disc.order, ref) @ vinv                 # (R, Np)
        self.npoints = len(points)
        self.elems = torch.from_numpy(elems).to(device)
        self.weights = torch.from_numpy(w).to(device)
        # deterministic adjoint injection: one row per distinct element
        uniq, inv = np.unique(elems, return_inverse=True)
        self.uelems = torch.from_numpy(uniq).to(device)
        inc = np.zeros((len(uniq), len(points)))
        inc[inv, np.arange(len(points))] = 1.0
        self.incidence = torch.from_numpy(inc).to(device)

    def sample(self, q: torch.Tensor) -> torch.Tensor:
        """(R,) values of field 0 of ``q`` (nfields, Nel, Np)."""
        return (q[0, self.elems, :] * self.weights).sum(dim=1)

    def inject(self, lam: torch.Tensor, g: torch.Tensor) -> None:
        """``lam[0] += R^T g`` without atomics."""
        contrib = self.incidence @ (g[:, None] * self.weights)   # (U, Np)
        lam[0, self.uelems, :] += contrib


def random_interior_points(n: int, lo, hi, margin: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, dtype=np.float64) + margin
    hi = np.asarray(hi, dtype=np.float64) - margin
    return lo + (hi - lo) * rng.random((n, 3))


# }}}


class WaveAdjointSolver:
    """Forward traces and their adjoint for one mesh, time step and step count."""

    def __init__(self, disc: DGDiscretization, dt: float, nsteps: int,
                 receivers: Receivers, device=None, segment: int | None = None,
                 checkpointing: str = "segments", slots: int | None = None):
        if checkpointing not in ("binomial", "segments"):
            raise ValueError(f"unknown checkpointing {checkpointing!r}")
        self.checkpointing = checkpointing
        self.mesh = DeviceMesh(disc, device, with_partner=True)
        self.device = self.mesh.device
        self.plan = DevicePlan(self.mesh, "wave", (1.0,), "fp64")
        self.dt = float(dt)
        self.nsteps = int(nsteps)
        self.rec = receivers
        self.segment = segment or max(1, int(round(math.sqrt(self.nsteps / 5.0))))
        self.slots = default_slots(self.nsteps) if slots is None else int(slots)
        self.schedule = (BinomialSchedule(self.nsteps, self.slots)
                         if checkpointing == "binomial" else None)
        shape = self.plan.shape
        self._buf = torch.empty(shape, dtype=torch.float64, device=self.device)
        self._res = torch.zeros(shape, dtype=torch.float64, device=self.device)
        # the reverse sweep's buffers, allocated once: the stage RHS of the
        # steps being reversed (a segment, or one step under the binomial
        # schedule), the residual adjoint and the transpose's scratch
        nrec = 1 if self.schedule is not None else self.segment
        self._lq = torch.empty((nrec, 5) + shape, dtype=torch.float64,
                               device=self.device)
        self._rbar = torch.empty(shape, dtype=torch.float64, device=self.device)
        self._yscr = torch.empty(shape, dtype=torch.float64, device=self.device)
        # touched once here, so that the first reverse sweep does not pay for
        # bringing the buffers into use
        for buf in (self._lq, self._rbar, self._yscr):
            buf.zero_()
        self.stats = {}

    # {{{ forward

    def _step(self, q: torch.Tensor, record: torch.Tensor | None = None) -> None:
        """One LSRK step of q in place; with ``record`` ((5,) + state shape)
        each stage also writes its RHS before the element scale there."""
        src, dst = q, self._buf
        for s in range(5):
            self.plan.rk_stage(src, dst, self._res, RK4A[s], RK4B[s], self.dt,
                               rhs_unscaled=None if record is None else record[s])
            src, dst = dst, src
        q.copy_(src)

    def forward(self, q0: torch.Tensor, c: torch.Tensor):
        """Traces (nsteps, R) and the checkpoints of the reverse sweep."""
        self.plan.set_element_scale(c)
        q = q0.clone()
        ckpts = {0: q0.clone()}
        keep = (set(self.schedule.first_descent()) if self.schedule is not None
                else {n for n in range(self.segment, self.nsteps, self.segment)})
        traces = torch.empty((self.nsteps, self.rec.npoints), dtype=torch.float64,
                             device=self.device)
        for n in range(self.nsteps):
            self._step(q)
            traces[n] = self.rec.sample(q)
            if n + 1 in keep:
                ckpts[n + 1] = q.clone()
        return traces, ckpts

    # }}}

    # {{{ reverse

    def _adjoint_step(self, lam: torch.Tensor, lq: torch.Tensor,
                      cbar: torch.Tensor) -> None:
        """lam <- Phi_q^T lam; cbar += Phi_c^T lam for one forward step whose
        stages had the RHS ``lq[s]`` (before the element scale).  Each stage is
        one fused pair of launches (``dg_rhs_adjoint_stage``): with rbar_4 =
        b_4 lam and rbar_{s-1} = a_s rbar_s + b_{s-1} lam, lam += dt L^T
        rbar_s and cbar_e += dt <rbar_s, lq[s]>_e."""
        rbar = self._rbar
        for s in range(4, -1, -1):
            x, xscale = (lam, RK4B[4]) if s == 4 else (rbar, 1.0)
            self.plan.adjoint_stage(x, xscale, lam, rbar if s > 0 else None, lq[s], cbar,
                                    RK4A[s], RK4B[s - 1] if s > 0 else 0.0, self.dt,
                                    self._yscr)

    def backward(self, grad_traces: torch.Tensor, ckpts: dict, c: torch.Tensor):
        """(dJ/dq0, dJ/dc) for dJ/dtraces = ``grad_traces``."""
        self.plan.set_element_scale(c)
        lam = torch.zeros(self.plan.shape, dtype=torch.float64, device=self.device)
        cbar = torch.zeros_like(c)
        if self.schedule is not None:
            def advance(q, a, b):
                q = q.clone()
                for _ in range(a, b):
                    self._step(q)
                return q

            def reverse_step(q_n, n):
                q = q_n.clone()
                self._step(q, self._lq[0])
                # trace n was sampled after step n, i.e. from q_{n+1}
                self.rec.inject(lam, grad_traces[n])
                self._adjoint_step(lam, self._lq[0], cbar)

            stored = {k: v for k, v in ckpts.items() if k != 0}
            st: dict = {}
            self.schedule.reverse(ckpts[0], advance, reverse_step, stored, st)
            self.stats = {"recomputed_steps": st["advanced"],
                          "peak_stored_states": st["peak_slots"] + 1,
                          "slots": self.slots}
            return lam, cbar
        starts = sorted(ckpts)
        for seg_start in reversed(starts):
            seg_end = min(self.nsteps, seg_start + self.segment)
            q = ckpts[seg_start].clone()
            for n in range(seg_start, seg_end):
                self._step(q, self._lq[n - seg_start])
            for n in range(seg_end - 1, seg_start - 1, -1):
                # trace n was sampled after step n, i.e. from q_{n+1}
                self.rec.inject(lam, grad_traces[n])
                self._adjoint_step(lam, self._lq[n - seg_start], cbar)
        return lam, cbar

    # }}}


class WaveMisfitFunction(torch.autograd.Function):
    """``traces = F(q0, c)`` with the hand-written adjoint as its backward.

    ``q0``: (4, Nel, Np) initial state; ``c``: (Nel,) element wave speeds; the
    third argument is a :class:`WaveAdjointSolver`."""

    @staticmethod
    def forward(ctx, q0, c, solver: WaveAdjointSolver):
        traces, ckpts = solver.forward(q0.detach().contiguous(),
                                       c.detach().contiguous())
        ctx.solver = solver
        ctx.ckpts = ckpts
        ctx.save_for_backward(c)
        return traces

    @staticmethod
    def backward(ctx, grad_traces):
        (c,) = ctx.saved_tensors
        dq0, dc = ctx.solver.backward(grad_traces.contiguous(), ctx.ckpts,
                                      c.contiguous())
        ctx.ckpts = None
        return dq0, dc, None


class RHSFunction(torch.autograd.Function):
    """``L(q)`` of a plan with the hand-written transposed Jacobian as its
    backward (``dg_rhs_vjp``): wave and Euler FP64 plans on meshes with face
    partners.  ``RHSFunction.apply(q, plan)``."""

    @staticmethod
    def forward(ctx, q, plan: DevicePlan):
        q = q.detach().contiguous()
        ctx.plan = plan
        ctx.save_for_backward(q)
        return plan.rhs(q)

    @staticmethod
    def backward(ctx, grad_out):
        (q,) = ctx.saved_tensors
        return ctx.plan.vjp(q, grad_out.contiguous()), None


class EulerAdjointSolver:
    """Gradient of a receiver misfit with respect to the initial state through
    LSRK(5,4) steps of the (nonlinear) Euler operator.

    Receivers sample the density.  The reverse of one step needs the five
    stage input states ``q^(s)``: stage ``s`` computes ``r^s = a_s r^{s-1} + dt
    L(q^(s))`` and ``q^(s+1) = q^(s) + b_s r^s``, so its adjoint applies the
    transposed Jacobian ``L'(q^(s))^T`` to the residual adjoint.  Checkpoints
    every ``segment`` steps; a segment is replayed once with its stage states
    kept (memory ``N/k + 5k`` states): the replayed stages write their output
    states straight into the record, allocated once, so recording costs no
    copies.  Each reverse stage is one fused call (``dg_rhs_vjp_stage``: the
    transposed Jacobian, the state-adjoint update and the next residual
    adjoint)."""

    def __init__(self, disc: DGDiscretization, gamma: float, dt: float, nsteps: int,
                 receivers: Receivers, device=None, segment: int | None = None):
        self.mesh = DeviceMesh(disc, device, with_partner=True)
        self.device = self.mesh.device
        self.plan = DevicePlan(self.mesh, "euler", (float(gamma),), "fp64")
        self.dt = float(dt)
        self.nsteps = int(nsteps)
        self.rec = receivers
        self.segment = segment or max(1, int(round(math.sqrt(self.nsteps / 5.0))))
        shape = self.plan.shape
        self._buf = torch.empty(shape, dtype=torch.float64, device=self.device)
        self._res = torch.zeros(shape, dtype=torch.float64, device=self.device)
        # the reverse sweep's buffers, allocated and touched once: the stage
        # input states of a segment, the residual adjoint and the scratch of
        # the transposed Jacobian
        self._qs = torch.zeros((self.segment, 5) + shape, dtype=torch.float64,
                               device=self.device)
        self._rbar = torch.zeros(shape, dtype=torch.float64, device=self.device)
        self._yscr = torch.zeros(shape, dtype=torch.float64, device=self.device)

    def _step(self, q: torch.Tensor) -> None:
        src, dst = q, self._buf
        for s in range(5):
            self.plan.rk_stage(src, dst, self._res, RK4A[s], RK4B[s], self.dt)
            src, dst = dst, src
        q.copy_(src)

    def _replay(self, q0: torch.Tensor, nsteps: int) -> None:
        """Steps from ``q0`` with every stage input state recorded:
        ``_qs[k, s]`` = q^(s) of the k-th step (stage s of step k reads
        ``_qs[k, s]`` and writes the next stage's input in place).  The last
        step's final stage is not run: the reverse sweep needs stage inputs
        only."""
        qs = self._qs
        qs[0, 0].copy_(q0)
        for k in range(nsteps):
            for s in range(5):
                if s < 4:
                    dst = qs[k, s + 1]
                elif k + 1 < nsteps:
                    dst = qs[k + 1, 0]
                else:
                    break       # its output, the next checkpoint, is not needed
                self.plan.rk_stage(qs[k, s], dst, self._res, RK4A[s], RK4B[s], self.dt)

    def forward(self, q0: torch.Tensor):
        q = q0.clone()
        ckpts = {0: q0.clone()}
        traces = torch.empty((self.nsteps, self.rec.npoints), dtype=torch.float64,
                             device=self.device)
        for n in range(self.nsteps):
            self._step(q)
            traces[n] = self.rec.sample(q)
            if (n + 1) % self.segment == 0 and n + 1 < self.nsteps:
                ckpts[n + 1] = q.clone()
        return traces, ckpts

    def _adjoint_step(self, lam: torch.Tensor, stages: torch.Tensor) -> None:
        """lam <- Phi'^T lam for one forward step with stage inputs
        ``stages[s]``: rbar_4 = b_4 lam, rbar_{s-1} = a_s rbar_s + b_{s-1} lam
        and lam += dt L'(q^(s))^T rbar_s, one fused call per stage."""
        rbar = self._rbar
        for s in range(4, -1, -1):
            x, xscale = (lam, RK4B[4]) if s == 4 else (rbar, 1.0)
            self.plan.vjp_stage(stages[s], x, xscale, lam, rbar if s > 0 else None,
                                RK4A[s], RK4B[s - 1] if s > 0 else 0.0, self.dt,
                                self._yscr)

    def backward(self, grad_traces: torch.Tensor, ckpts: dict) -> torch.Tensor:
        lam = torch.zeros(self.plan.shape, dtype=torch.float64, device=self.device)
        for seg_start in reversed(sorted(ckpts)):
            seg_end = min(self.nsteps, seg_start + self.segment)
            self._replay(ckpts[seg_start], seg_end - seg_start)
            for n in range(seg_end - 1, seg_start - 1, -1):
                self.rec.inject(lam, grad_traces[n])
                self._adjoint_step(lam, self._qs[n - seg_start])
        return lam


class EulerMisfitFunction(torch.autograd.Function):
    """``traces = F(q0)`` for an :class:`EulerAdjointSolver`, with the
    hand-written adjoint as its backward."""

    @staticmethod
    def forward(ctx, q0, solver: EulerAdjointSolver):
        traces, ckpts = solver.forward(q0.detach().contiguous())
        ctx.solver = solver
        ctx.ckpts = ckpts
        return traces

    @staticmethod
    def backward(ctx, grad_traces):
        lam = ctx.solver.backward(grad_traces.contiguous(), ctx.ckpts)
        ctx.ckpts = None
        return lam, None

"""Binomial checkpointing for the reverse sweep of a time integrator.

The reverse of step ``n`` needs the forward state ``q_n``.  With ``s`` free
state slots, the states needed by a reverse sweep over ``l`` steps are
recomputed from a stored state at the start of the range by the recursion of
Griewank's "Revolve" (A. Griewank, A. Walther, ACM TOMS 26(1), 2000):
advance ``j`` steps and store the state there, reverse the upper part with
``s - 1`` slots, free the slot, reverse the lower part with ``s`` slots.  The
split ``j`` minimising the number of recomputed steps is found here by
dynamic programming over

    C(1, s) = 1,   C(l, 0) = l (l + 1) / 2,
    C(l, s) = min_{0 < j < l} j + C(l - j, s - 1) + C(j, s),

whose minimum is the binomial bound of Revolve (l steps need about
t l recomputations when l <= binom(s + t, s)).  ``C`` counts every forward
step the reverse sweep runs, including the one step per reversed step that
records the stage values.

The schedule is independent of the integrator: :meth:`BinomialSchedule.reverse`
calls ``advance(state, a, b)`` (a new state advanced from index ``a`` to
``b``) and ``reverse_step(state_n, n)`` (reverse step ``n`` from its start
state), for ``n = l - 1, ..., 0`` in that order.
"""

from __future__ import annotations

import math

import numpy as np


class BinomialSchedule:
    """Optimal splits for reversing up to ``nsteps`` steps with ``slots`` slots."""

    def __init__(self, nsteps: int, slots: int):
        if nsteps < 1 or slots < 0:
            raise ValueError("need nsteps >= 1 and slots >= 0")
        self.nsteps = int(nsteps)
        self.slots = int(slots)
        n, s_max = self.nsteps, self.slots
        cost = np.zeros((n + 1, s_max + 1), dtype=np.int64)
        split = np.zeros((n + 1, s_max + 1), dtype=np.int64)
        ell = np.arange(n + 1, dtype=np.int64)
        cost[:, 0] = ell * (ell + 1) // 2
        for s in range(1, s_max + 1):
            cost[1, s] = 1
            for length in range(2, n + 1):
                js = np.arange(1, length)
                vals = js + cost[length - js, s - 1] + cost[js, s]
                k = int(np.argmin(vals))
                cost[length, s] = vals[k]
                split[length, s] = js[k]
        self.cost = cost
        self.split = split

    def first_descent(self) -> list[int]:
        """Indices the reverse sweep stores first (top of the recursion); a
        forward sweep that keeps these states saves their recomputation."""
        out, a, s = [], 0, self.slots
        while self.nsteps - a > 1 and s > 0:
            a += int(self.split[self.nsteps - a, s])
            out.append(a)
            s -= 1
        return out

    def recomputed_steps(self, stored: int = 0) -> int:
        """Forward steps the reverse sweep runs (``stored`` = steps of the
        first descent already covered by a forward sweep)."""
        return int(self.cost[self.nsteps, self.slots]) - stored

    def reverse(self, state0, advance, reverse_step, stored: dict | None = None,
                stats: dict | None = None) -> None:
        """Reverse steps ``nsteps - 1 .. 0`` starting from ``state0`` (the
        state at index 0, left untouched).  ``stored`` may hold states of the
        first descent by index; they are used instead of recomputed."""
        stored = dict(stored or {})
        st = stats if stats is not None else {}
        st.setdefault("advanced", 0)
        st.setdefault("peak_slots", 0)
        live = [0]

        def adv(q, a, b):
            st["advanced"] += b - a
            return advance(q, a, b)

        def rec(a, b, s, q_a):
            while b - a > 0:
                length = b - a
                if length == 1:
                    st["advanced"] += 1
                    reverse_step(q_a, a)
                    return
                if s == 0:
                    for n in range(b - 1, a - 1, -1):
                        q_n = q_a if n == a else adv(q_a, a, n)
                        st["advanced"] += 1
                        reverse_step(q_n, n)
                    return
                m = a + int(self.split[length, s])
                q_m = stored.pop(m, None)
                if q_m is None:
                    q_m = adv(q_a, a, m)
                live[0] += 1
                st["peak_slots"] = max(st["peak_slots"], live[0])
                rec(m, b, s - 1, q_m)
                del q_m
                live[0] -= 1
                b = m

        rec(0, self.nsteps, self.slots, state0)


def default_slots(nsteps: int) -> int:
    """sqrt(nsteps) state slots (the memory the benchmark's adjoint targets)."""
    return max(1, int(math.ceil(math.sqrt(nsteps))))

"""Low-storage RK(5,4) in NumPy (oracle; test infrastructure).

Carpenter & Kennedy (1994) five-stage fourth-order scheme:
res = a_s res + dt L(q); q = q + b_s res, s = 1..5.
"""

from __future__ import annotations

import numpy as np

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


def lsrk45_step(rhs, q: np.ndarray, dt: float, res: np.ndarray | None = None):
    """One step of ``dq/dt = rhs(q)``; returns the new state."""
    q = q.copy()
    res = np.zeros_like(q) if res is None else res
    for a, b in zip(RK4A, RK4B):
        res = a * res + dt * rhs(q)
        q = q + b * res
    return q

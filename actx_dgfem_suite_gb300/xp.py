"""Array-library helpers so that initial conditions evaluate on host NumPy
arrays and on device torch tensors with the same code."""

from __future__ import annotations

import numpy as np


def is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def array_module(x):
    if is_torch(x):
        import torch
        return torch
    return np


def zeros(like, shape):
    if is_torch(like):
        import torch
        return torch.zeros(shape, dtype=torch.float64, device=like.device)
    return np.zeros(shape)


def r2(nodes, center=(0.0, 0.0, 0.0)):
    """|x - center|^2 of (dim, ...) node coordinates (dim 2 or 3; the center's
    leading ``dim`` entries are used)."""
    return sum((nodes[x] - center[x]) ** 2 for x in range(len(nodes)))

"""Regenerate the golden RHS fixtures from the CPU oracle.

The reference ships no golden vectors for this path and cannot run here, so
these fixtures are the oracle's own FP64 outputs for the reference's problem
definitions (``actx_dgfem_suite/equations/{wave,euler,maxwell}.py``) on tiny
box meshes.  They pin the oracle against regressions and give the GPU tests
a fixed target; they are not evidence of agreement with the reference.

Usage: ``python tests/golden/make_golden.py`` from the repository root.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

#: (equation, order, elements per axis)
CASES = [(eq, p, 1) for eq in ("wave", "euler", "maxwell") for p in (1, 2, 3, 4)] \
    + [(eq, 2, 2) for eq in ("wave", "euler", "maxwell")]


def fixture_path(eq: str, order: int, n: int) -> Path:
    return HERE / f"rhs_{eq}_P{order}_n{n}.npz"


def compute(eq: str, order: int, n: int):
    from actx_dgfem_suite_gb300.rhs_builder import get_problem
    from tests._helpers import oracle_rhs
    prob = get_problem(eq, 3, order, definition="reference", nel_1d=n)
    rhs, scale = oracle_rhs(prob, parts=True)
    return prob, rhs, scale


def main():
    for eq, order, n in CASES:
        prob, rhs, scale = compute(eq, order, n)
        np.savez_compressed(fixture_path(eq, order, n), rhs=rhs,
                            scale=np.float64(scale),
                            input_l2=np.float64(np.linalg.norm(prob.fields)),
                            params=np.array(prob.params, dtype=np.float64))
        print(fixture_path(eq, order, n).name, rhs.shape)


if __name__ == "__main__":
    main()

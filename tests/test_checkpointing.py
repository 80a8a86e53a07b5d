"""Binomial checkpointing schedule (host logic, CPU)."""

import math

import pytest

from actx_dgfem_suite_gb300.checkpointing import BinomialSchedule, default_slots


def _toy(nsteps):
    states = [1.0]
    for n in range(nsteps):
        states.append(math.sin(states[-1] + 0.1 * n) + 1.5)
    return states


@pytest.mark.parametrize("nsteps,slots", [(1, 0), (1, 3), (7, 0), (7, 1), (12, 2),
                                          (50, 3), (300, 18)])
def test_reverse_visits_every_step_with_its_state(nsteps, slots):
    truth = _toy(nsteps)
    sched = BinomialSchedule(nsteps, slots)
    seen = []

    def advance(q, a, b):
        for n in range(a, b):
            q = math.sin(q + 0.1 * n) + 1.5
        return q

    def reverse_step(q, n):
        assert q == truth[n]
        seen.append(n)

    stats = {}
    sched.reverse(truth[0], advance, reverse_step, stats=stats)
    assert seen == list(range(nsteps - 1, -1, -1))
    assert stats["advanced"] == sched.recomputed_steps()
    assert stats["peak_slots"] <= slots


def test_first_descent_states_are_not_recomputed():
    nsteps, slots = 300, 18
    truth = _toy(nsteps)
    sched = BinomialSchedule(nsteps, slots)
    desc = sched.first_descent()
    assert desc == sorted(desc) and len(desc) <= slots
    stored = {m: truth[m] for m in desc}
    stats = {}

    def advance(q, a, b):
        for n in range(a, b):
            q = math.sin(q + 0.1 * n) + 1.5
        return q

    sched.reverse(truth[0], advance, lambda q, n: None, stored=stored, stats=stats)
    assert stats["advanced"] == sched.recomputed_steps(stored=desc[-1])


def test_binomial_cost_scaling():
    # 300 steps with sqrt(300) slots: about 3 forward steps per reversed step, far below
    # the quadratic cost of storing nothing and the N-state cost of storing all
    sched = BinomialSchedule(300, default_slots(300))
    assert default_slots(300) == 18
    assert sched.recomputed_steps() <= 3.5 * 300   # incl. one recording step each
    assert BinomialSchedule(300, 0).recomputed_steps() == 300 * 301 // 2
    # more slots never cost more
    costs = [BinomialSchedule(60, s).recomputed_steps() for s in range(0, 8)]
    assert all(x >= y for x, y in zip(costs, costs[1:]))

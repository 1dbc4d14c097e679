"""Lab-grid sampling along every path the engine takes.

Single launches, 6-step graph replays, plain steps in between, state reads (which
replay the last collision) and repeated reads must all give the sums of the plain
one-step-at-a-time definition: the same counts exactly, velocities up to the
rounding of the float atomics' order.  The sums are kept in storage order and
gathered into the reference order on the device at each read.
"""
from __future__ import annotations

import numpy as np
import pytest

from cudampcd_gb300 import capi

pytestmark = pytest.mark.gpu

BOX = dict(L=(12, 10, 14), periodic=(1, 1, 0), n=10, dt=0.02, drag=2e-3, seed=31)


def _run(plan, algorithm=0):
    h = capi.Handle(algorithm=algorithm, **BOX)
    try:
        reads = []
        for kind, n in plan:
            if kind == "s":
                h.step_and_sample(n)
            elif kind == "p":
                h.step(n)
            elif kind == "x":
                h.positions()   # replays the last collision; must not disturb the pending sample
            else:
                reads.append(h.sample_mean())
        return reads, h.positions()
    finally:
        h.close()


def _same(r0, r1):
    for (d0, v0), (d1, v1) in zip(r0, r1):
        assert np.array_equal(d0, d1)
        np.testing.assert_allclose(v0, v1, rtol=0, atol=1e-6)


@pytest.mark.parametrize("algorithm", [0, 1])
def test_single_launches_and_graph_replays_sample_alike(algorithm):
    singles = [("s", 1)] * 13 + [("p", 5)] + [("s", 1)] * 12 + [("r", 0)]
    graphs = [("s", 13), ("p", 5), ("s", 12), ("r", 0)]
    r0, x0 = _run(singles, algorithm)
    r1, x1 = _run(graphs, algorithm)
    assert np.array_equal(x0, x1)   # sampling never changes the dynamics
    _same(r0, r1)


def test_reads_restart_the_sample_and_state_reads_keep_it():
    a, _ = _run([("s", 7), ("x", 0), ("s", 11), ("r", 0), ("s", 12), ("r", 0)])
    b, _ = _run([("s", 18), ("r", 0), ("p", 0), ("s", 12), ("r", 0)])
    _same(a, b)
    c, _ = _run([("p", 18), ("s", 12), ("r", 0)])
    _same(a[1:], c)   # the second read holds only the last 12 steps


def test_first_sampled_step_replaces_old_sums():
    # a run sampled and read, then sampled again: the second read must not see the first
    a, _ = _run([("s", 6), ("r", 0), ("p", 3), ("s", 9), ("r", 0)])
    b, _ = _run([("p", 9), ("s", 9), ("r", 0)])
    _same(a[1:], b)

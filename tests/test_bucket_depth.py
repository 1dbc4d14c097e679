"""Buckets shallower than the reference's 4n-deep cell table.

A cell's bucket holds `depth` = min(4n, n + ceil(4 sqrt(n)) + 2) slots; the
particles a cell receives past that go to the overflow list, and the step's
prologue copies the cell's colliding set (all of them, or the 4n lowest ids) into
the extension area that both step kernels then read.  MPCD_GB_BUCKET_DEPTH, read
when a handle is created, forces a smaller depth, so that most cells of these
boxes spill.  Every result must be bit-identical to the default depth: SRD cell
sums are exact fixed-point sums, the extended collision walks a cell's particles
in id order, and the choice of colliding particles follows particle ids, so the
storage order of a cell's particles changes nothing (only the lab-grid sample,
FP32 atomic sums, is order-dependent to rounding).  The layout dump too must not
change (its slot numbers do: they name where a particle is stored).
"""
from __future__ import annotations

import contextlib
import os

import numpy as np
import pytest

from cudampcd_gb300 import capi

pytestmark = pytest.mark.gpu

# box keywords, forced depth
CASES = {
    # SRD between walls (the run kernel, the prologue's wall ghosts): depth 3 of 40
    "srd_walls_n10": (dict(L=(12, 10, 14), periodic=(1, 1, 0), n=10, drag=1e-3, seed=5), 3),
    "srd_periodic_n20": (dict(L=(10, 10, 10), periodic=(1, 1, 1), n=20, seed=6), 12),
    # the extended collision (the tile kernel and its staging copies)
    "ext_walls_n10": (dict(L=(10, 8, 12), periodic=(1, 1, 0), n=10, algorithm=1, drag=1e-3, seed=7), 4),
    # n = 1: depth 1 of 4, and cells past 4n whose 4 lowest ids collide
    "srd_sparse_n1": (dict(L=(12, 10, 9), periodic=(1, 1, 0), n=1, dt=0.05, seed=8), 1),
    "srd_n3": (dict(L=(10, 9, 8), periodic=(1, 1, 0), n=3, dt=0.05, seed=9), 2),
    # the densest the run kernel takes, and the densest accepted (the tile kernel)
    "srd_dense_n64": (dict(L=(4, 4, 6), periodic=(1, 1, 0), n=64, seed=10), 40),
    "srd_max_density": (dict(L=(3, 3, 4), periodic=(1, 1, 0), n=409, seed=11), 300),
}


@contextlib.contextmanager
def forced_depth(depth: int):
    old = os.environ.get("MPCD_GB_BUCKET_DEPTH")
    os.environ["MPCD_GB_BUCKET_DEPTH"] = str(depth)
    try:
        yield
    finally:
        if old is None:
            del os.environ["MPCD_GB_BUCKET_DEPTH"]
        else:
            os.environ["MPCD_GB_BUCKET_DEPTH"] = old


def _pair(depth: int, **kw):
    base = capi.Handle(**kw)
    with forced_depth(depth):
        shallow = capi.Handle(**kw)
    return base, shallow


def _same_state(a: capi.Handle, b: capi.Handle, what: str):
    assert np.array_equal(a.positions(), b.positions()), f"positions {what}"
    assert np.array_equal(a.velocities(), b.velocities()), f"velocities {what}"


def _same_layout(a: capi.Handle, b: capi.Handle):
    ca, _, ia, na = a.layout()
    cb, _, ib, nb = b.layout()
    assert np.array_equal(na, nb) and np.array_equal(ca, cb) and np.array_equal(ia, ib)


@pytest.mark.parametrize("name", list(CASES))
def test_shallow_buckets_change_nothing(name):
    kw, depth = CASES[name]
    a, b = _pair(depth, **kw)
    try:
        _same_layout(a, b)
        a.step(1)
        b.step(1)
        _same_state(a, b, "after one step")
        _same_layout(a, b)
        a.step_and_sample(13)   # graph replays of six steps and single steps
        b.step_and_sample(13)
        _same_state(a, b, "after sampled steps")
        # the lab-grid sample adds FP32 velocities atomically, in storage order:
        # counts exact, mean velocities to FP32 rounding
        da, va = a.sample_mean()
        db, vb = b.sample_mean()
        assert np.array_equal(da, db)
        assert np.abs(va - vb).max() <= 1e-5
        _same_layout(a, b)
        assert a.counters()[1] == 0 and b.counters()[1] == 0
        # the shallow handle did spill, far more than the default one
        assert b.counters()[0] > max(10 * a.counters()[0], 100)
    finally:
        a.close()
        b.close()


# boxes large enough that every warp of the run kernel and every CTA of the tile
# kernel sweeps many runs or tiles, with about one cell in six (n = 20, depth 24)
# spilled into the extension area each step
LARGE = {
    "srd_160x160x20": (dict(L=(160, 160, 22), periodic=(1, 1, 0), n=20, drag=1e-3, seed=31), 24),
    "ext_100x100x20": (dict(L=(100, 100, 22), periodic=(1, 1, 0), n=20, algorithm=1, drag=5e-4, seed=32), 24),
}


@pytest.mark.parametrize("name", list(LARGE))
def test_shallow_buckets_in_large_boxes(name):
    kw, depth = LARGE[name]
    a, b = _pair(depth, **kw)
    try:
        a.step(1)
        b.step(1)
        _same_state(a, b, "after one step")
        a.step(6)   # one graph replay
        b.step(6)
        _same_state(a, b, "after a graph replay")
        assert a.counters()[1] == 0 and b.counters()[1] == 0
        assert b.counters()[0] > 10 * max(a.counters()[0], 1000)
    finally:
        a.close()
        b.close()


def test_shallow_buckets_with_every_particle_in_one_cell():
    """All particles of a 10^3, n = 10 box in one cell: that cell's 40 lowest ids
    collide, the others skip the collision (the reference's index-order table)."""
    a, b = _pair(7, L=(10, 10, 10), periodic=(1, 1, 1), n=10, dt=1.0, seed=3)
    try:
        for h in (a, b):
            h.inject_shift(h.step_index, (0, 0, 0))
            h.set_particles(np.full((h.N, 3), -5.0, np.float32),
                            np.random.default_rng(1).normal(size=(h.N, 3)).astype(np.float32) * 1e-3)
        _same_layout(a, b)
        for _ in range(3):
            a.step(1)
            b.step(1)
            _same_state(a, b, "with one crowded cell")
        assert a.counters()[1] == 0 and b.counters()[1] == 0
    finally:
        a.close()
        b.close()


def test_shallow_buckets_in_an_ensemble():
    boxes = [
        dict(L=(8, 8, 22), periodic=(1, 1, 0), n=5, drag=1e-3, seed=11),
        dict(L=(16, 8, 30), periodic=(1, 1, 0), n=10, drag=1e-4, seed=12),
        dict(L=(8, 16, 20), periodic=(1, 1, 0), n=20, drag=1e-2, seed=13),
    ]
    a = capi.Handle(boxes=boxes)
    with forced_depth(4):
        b = capi.Handle(boxes=boxes)
    try:
        a.step(1)
        b.step(1)
        a.step(12)
        b.step(12)
        _same_state(a, b, "of the ensemble")
        assert a.counters()[1] == 0 and b.counters()[1] == 0
    finally:
        a.close()
        b.close()


def test_shallow_buckets_with_the_pressure_estimator_and_getters():
    """The tile kernel's steps (pressure estimator on) and replays read the extension."""
    kw, depth = CASES["srd_walls_n10"]
    a, b = _pair(depth, **kw)
    try:
        for h in (a, b):
            h.wall_pressure(restart=True)
        for _ in range(4):
            a.step(1)
            b.step(1)
            _same_state(a, b, "with the pressure estimator")
        # impulses are summed per thread in FP32 (storage order), then in FP64
        pa, pb = np.asarray(a.wall_pressure()), np.asarray(b.wall_pressure())
        assert np.allclose(pa, pb, rtol=1e-6, atol=0)
    finally:
        a.close()
        b.close()


def test_full_extension_is_an_error():
    """More spilled particles than the extension holds (2^22 slots for N > 2^22):
    the step reports it; the cells left without an extension collide their bucket
    only, and every particle is still stored."""
    with forced_depth(5):
        h = capi.Handle(L=(120, 100, 22), periodic=(1, 1, 0), n=20, seed=21)
    try:
        assert h.N > 1 << 22
        with pytest.raises(capi.GbError, match="extension"):
            h.step(1)
        assert h.counters()[1] & 8
    finally:
        h.close()

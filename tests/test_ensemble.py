"""Batched ensemble: independent boxes of uneven size, density and drag advanced
by one launch per step.  Every draw is keyed by (box seed, step, box-local cell or
particle), SRD cell sums are exact and the extended collision walks cells in
particle-id order, so each box of an ensemble must evolve bit-identically to a
single-box handle made from the same parameters -- including after the
autotuner has changed the tiling.  Boxes of different density take tiles of
different size within one launch (here 32 to 128 cells).
"""
from __future__ import annotations

import numpy as np
import pytest

from cudampcd_gb300 import capi

pytestmark = pytest.mark.gpu

BOXES = [
    dict(L=(8, 8, 22), periodic=(1, 1, 0), n=5, drag=1e-3, seed=11),
    dict(L=(16, 8, 30), periodic=(1, 1, 0), n=10, drag=1e-4, seed=12),
    dict(L=(8, 16, 20), periodic=(1, 1, 0), n=20, drag=1e-2, seed=13),
    dict(L=(6, 5, 7), periodic=(1, 1, 1), n=8, drag=0.0, seed=14),
    dict(L=(32, 8, 40), periodic=(1, 1, 0), n=5, drag=3e-3, dt=0.05, temperature=0.5, seed=15),
    dict(L=(8, 8, 12), periodic=(1, 1, 0), n=40, drag=2e-3, seed=16),
]


def _check_same(ens: capi.Handle, singles: list[capi.Handle]):
    pe, ve = ens.positions(), ens.velocities()
    for r, h in enumerate(singles):
        p0, n, _, _ = ens.box_range(r)
        assert np.array_equal(pe[p0:p0 + n], h.positions()), f"positions of box {r}"
        assert np.array_equal(ve[p0:p0 + n], h.velocities()), f"velocities of box {r}"


@pytest.mark.parametrize("alg", [0, 1])
def test_boxes_evolve_as_single_handles(alg):
    boxes = [dict(b, algorithm=alg) for b in BOXES]
    ens = capi.Handle(boxes=boxes)
    singles = [capi.Handle(**b) for b in boxes]
    try:
        assert ens.num_boxes == len(boxes)
        assert ens.N == sum(h.N for h in singles) and ens.C == sum(h.C for h in singles)
        for r, h in enumerate(singles):
            p0, n, c0, nc = ens.box_range(r)
            assert (n, nc) == (h.N, h.C)
            assert p0 == sum(s.N for s in singles[:r]) and c0 == sum(s.C for s in singles[:r])
        _check_same(ens, singles)   # initial states
        ens.step(7)
        for h in singles:
            h.step(7)
        _check_same(ens, singles)

        ens.step_and_sample(6)
        for h in singles:
            h.step_and_sample(6)
        d, v = ens.sample_mean()
        for r, h in enumerate(singles):
            _, _, c0, nc = ens.box_range(r)
            ds, vs = h.sample_mean()
            assert np.array_equal(d[c0:c0 + nc], ds)
            # sampled sums are float atomics: equal up to the rounding of their order
            np.testing.assert_allclose(v[c0:c0 + nc], vs, rtol=0, atol=1e-6)

        tile_cells, pbuf = ens.autotune(1)
        assert tile_cells in (8, 16, 32, 64, 128) and pbuf in (1024, 1280, 1344, 1408, 1536, 2048)
        for h in singles:
            h.step(ens.step_index - h.step_index)
        ens.step(3)
        for h in singles:
            h.step(3)
        _check_same(ens, singles)
        assert ens.counters()[1] == 0
    finally:
        ens.close()
        for h in singles:
            h.close()


@pytest.mark.parametrize("alg", [0, 1])
def test_dense_boxes_take_small_tiles_and_sub_tiles(alg):
    """Densities from 5 to 200 in one launch: 128- or 64-cell tiles down to 8-cell
    tiles with one warp per cell, and at n = 200 tiles whose particles exceed the
    buffer and run as several sub-tiles -- each box still as its single handle."""
    boxes = [dict(L=(10, 8, 14), periodic=(1, 1, 0), n=5, drag=1e-3, seed=21, algorithm=alg),
             dict(L=(6, 6, 12), periodic=(1, 1, 0), n=100, drag=2e-3, seed=22, algorithm=alg),
             dict(L=(5, 6, 10), periodic=(1, 1, 1), n=200, drag=0.0, seed=23, algorithm=alg),
             dict(L=(8, 8, 12), periodic=(1, 1, 0), n=20, drag=1e-3, seed=24, algorithm=alg)]
    ens = capi.Handle(boxes=boxes)
    singles = [capi.Handle(**b) for b in boxes]
    try:
        ens.step(5)
        for h in singles:
            h.step(5)
        _check_same(ens, singles)
        assert ens.counters() == (0, 0)
    finally:
        ens.close()
        for h in singles:
            h.close()


@pytest.mark.parametrize("alg", [0, 1])
def test_overflowing_boxes_evolve_as_single_handles(alg):
    """At n = 1 and 2 some cells receive more particles than their buckets hold;
    the lowest ids collide whatever order the claims arrived in, so an ensemble
    still reproduces its single handles bit for bit."""
    boxes = [dict(L=(12, 10, 12), periodic=(1, 1, 0), n=1, drag=1e-3, seed=31, algorithm=alg),
             dict(L=(10, 12, 10), periodic=(1, 1, 1), n=2, drag=0.0, seed=32, algorithm=alg)]
    ens = capi.Handle(boxes=boxes)
    singles = [capi.Handle(**b) for b in boxes]
    try:
        ens.step(8)
        for h in singles:
            h.step(8)
        _check_same(ens, singles)
        overflowed, flags = ens.counters()
        assert overflowed > 0 and flags == 0
    finally:
        ens.close()
        for h in singles:
            h.close()


def test_ensemble_rejects_mixed_algorithms_and_empty():
    with pytest.raises(capi.GbError, match="same algorithm"):
        capi.Handle(boxes=[dict(BOXES[0], algorithm=0), dict(BOXES[1], algorithm=1)])
    with pytest.raises(capi.GbError, match="at least one box"):
        capi.Handle(boxes=[])


def test_injected_draws_need_one_box():
    import oracle as O

    ens = capi.Handle(boxes=BOXES[:2])
    try:
        box = O.Box(L=BOXES[0]["L"], periodic=BOXES[0]["periodic"], n=BOXES[0]["n"])
        with pytest.raises(capi.GbError, match="single-box"):
            ens.inject_draws(O.Draws.empty(box))
    finally:
        ens.close()

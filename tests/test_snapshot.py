"""Snapshots: checkpoint and resume.

A trajectory interrupted by save -> new handle -> load continues bit for bit:
the snapshot holds the post-step state by particle id, and loading re-keys it
with the same streaming arithmetic as the step that produced the buckets.
"""
from __future__ import annotations

import numpy as np
import pytest

from cudampcd_gb300 import capi

pytestmark = pytest.mark.gpu

CASES = [
    [dict(L=(12, 10, 14), periodic=(1, 1, 0), n=10, drag=1e-3, algorithm=0, seed=41)],
    [dict(L=(8, 8, 12), periodic=(1, 1, 0), n=10, drag=5e-4, algorithm=1, seed=42)],
    [dict(L=(8, 8, 22), periodic=(1, 1, 0), n=5, drag=1e-3, seed=43),
     dict(L=(16, 8, 30), periodic=(1, 1, 0), n=10, drag=1e-2, seed=44)],
]


@pytest.mark.parametrize("boxes", CASES)
def test_resume_from_snapshot_is_bit_exact(tmp_path, boxes):
    path = tmp_path / "state.mpcd"
    a = capi.Handle(boxes=boxes)
    b = capi.Handle(boxes=boxes)
    try:
        a.step(9)
        a.save_snapshot(path)
        a.step(7)
        b.step(3)   # any state: the load replaces it
        b.load_snapshot(path)
        assert b.step_index == 9
        b.step(7)
        assert np.array_equal(a.positions(), b.positions())
        assert np.array_equal(a.velocities(), b.velocities())
    finally:
        a.close()
        b.close()


def test_snapshot_rejects_other_boxes_and_corruption(tmp_path):
    path = tmp_path / "state.mpcd"
    a = capi.Handle(**CASES[0][0])
    other = capi.Handle(**dict(CASES[0][0], seed=99))
    try:
        a.step(2)
        a.save_snapshot(path)
        with pytest.raises(capi.GbError, match="seed"):
            other.load_snapshot(path)
        raw = bytearray(path.read_bytes())
        raw[200] ^= 0xFF
        bad = tmp_path / "bad.mpcd"
        bad.write_bytes(bytes(raw))
        with pytest.raises(capi.GbError, match="checksum"):
            a.load_snapshot(bad)
        with pytest.raises(capi.GbError, match="cannot open"):
            a.load_snapshot(tmp_path / "missing.mpcd")
    finally:
        a.close()
        other.close()

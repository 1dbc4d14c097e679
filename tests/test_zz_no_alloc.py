"""Allocation-free cell offsets (mpcd_gb_cell_offsets_noalloc) against the layout dump.

The entry point writes, into a caller's device buffer, where each cell's run
starts in the mpcd_gb_dump_layout order; its scan scratch is a fixed array in
the library's device memory.  Every case calls it twice in a row and compares
both results with the offsets implied by mpcd_gb_dump_layout, so a scratch that
is not re-zeroed between calls shows up as a mismatch of the second call.  The
library's count of its device allocations (mpcd_gb_device_allocations: every device
buffer goes through one counting allocator) must not move across a call.
"""
from __future__ import annotations

import re

import numpy as np
import pytest

import oracle as O
from cudampcd_gb300 import capi

pytestmark = pytest.mark.gpu

SENTINEL = 0x7F7F7F7F


def _max_cells() -> int:
    text = open(capi.HEADER).read()
    return int(re.search(r"#define\s+MPCD_GB_NOALLOC_MAX_CELLS\s+(\d+)u", text).group(1))


def _device_buffer(entries: int):
    torch = pytest.importorskip("torch")
    return torch.full((entries,), SENTINEL, dtype=torch.int32, device="cuda")


def _read(h: capi.Handle, buf) -> np.ndarray:
    h.synchronize()
    return buf.cpu().numpy().view(np.uint32).astype(np.int64)


def _offsets_from_dump(h: capi.Handle, L, n) -> np.ndarray:
    """Offsets in storage order from mpcd_gb_dump_layout's counts, checked
    against the cells of its particle list."""
    cell, _, _, counts = h.layout()
    box = O.Box(L=L, n=n)
    bucketed = np.zeros(h.C, np.int64)
    bucketed[O.storage_index(box, np.arange(h.C))] = np.minimum(counts.astype(np.int64), 4 * n)
    offsets = np.concatenate([[0], np.cumsum(bucketed)])
    keys = O.storage_index(box, cell[: offsets[-1]]).astype(np.int64)
    assert np.all(np.diff(keys) >= 0)
    assert np.array_equal(np.bincount(keys, minlength=h.C), bucketed)
    return offsets


CASES = [
    # (L, periodic, n, algorithm): one scan tile, several tiles with walls, extended
    ((6, 5, 9), (1, 1, 0), 8, 0),
    ((40, 30, 22), (1, 1, 0), 10, 0),
    ((64, 48, 20), (1, 1, 1), 6, 1),
]


@pytest.mark.parametrize("L,periodic,n,alg", CASES)
def test_offsets_match_dump_on_consecutive_calls(L, periodic, n, alg):
    before_handle = capi.device_allocations()
    h = capi.Handle(L=L, periodic=periodic, n=n, algorithm=alg, drag=0.001 * (periodic[2] == 0), seed=11)
    assert capi.device_allocations() > before_handle   # the counter sees the handle's buffers
    try:
        first, second = _device_buffer(h.C + 1), _device_buffer(h.C + 1)
        for _ in range(2):
            h.step(3)
            h.cell_offsets_noalloc(first.data_ptr(), h.C + 1)
            h.synchronize()
            allocations = capi.device_allocations()
            h.cell_offsets_noalloc(second.data_ptr(), h.C + 1)
            h.synchronize()
            assert capi.device_allocations() == allocations   # every device buffer is counted
            expected = _offsets_from_dump(h, L, n)
            assert np.array_equal(_read(h, first), expected)
            assert np.array_equal(_read(h, second), expected)
            assert h.counters()[1] == 0
    finally:
        h.close()


def test_rejects_short_buffer_and_null():
    h = capi.Handle(L=(12, 10, 8), periodic=(1, 1, 1), n=5, seed=3)
    try:
        buf = _device_buffer(h.C + 1)
        with pytest.raises(capi.GbError, match="needed"):
            h.cell_offsets_noalloc(buf.data_ptr(), h.C)
        with pytest.raises(capi.GbError, match="null"):
            h.cell_offsets_noalloc(0, h.C + 1)
        assert np.all(_read(h, buf) == SENTINEL)
    finally:
        h.close()


def test_rejects_cells_beyond_limit():
    limit = _max_cells()
    L = (2049, 2049, 8)
    assert L[0] * L[1] * L[2] > limit
    h = capi.Handle(L=L, periodic=(1, 1, 1), n=1, seed=5)
    try:
        assert h.C > limit
        buf = _device_buffer(h.C + 1)
        with pytest.raises(capi.GbError, match="exceed the limit"):
            h.cell_offsets_noalloc(buf.data_ptr(), h.C + 1)
        assert np.all(_read(h, buf)[:4096] == SENTINEL)
    finally:
        h.close()

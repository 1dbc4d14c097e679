"""Shared helpers of the GPU parity tests."""
from __future__ import annotations

import numpy as np

import oracle as O
from cudampcd_gb300 import capi

# Tolerance of the floating-point parity checks: 1e-5 relative to
# max(|v|, thermal velocity) per component.
REL_TOL = 1e-5


def make(box: O.Box, seed: int = 7) -> capi.Handle:
    return capi.Handle(L=box.L, periodic=box.periodic, n=box.n, dt=box.dt, drag=box.drag,
                       temperature=box.thermal_velocity ** 2, algorithm=box.algorithm, experiment=box.experiment,
                       seed=seed)


def storage_keys(box: O.Box, ref_cells: np.ndarray) -> np.ndarray:
    return O.storage_index(box, ref_cells)


def set_state(h: capi.Handle, pos, vel, shift=None):
    """Load a dense state (particle id = row), optionally with the grid shift of
    the next step injected; returns the resulting layout (cell, slot, id, counts)."""
    if shift is not None:
        h.inject_shift(h.step_index, shift)
    h.set_particles(pos, vel)
    return h.layout()


def rel_err(a, b, scale=1.0):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), scale)

"""SRD shear viscosity from a Poiseuille channel against the analytic value.

Workload: fluid 10 x 10 x 100 cells between no-slip walls in z (container
10 x 10 x 102, periodic in x and y), n = 10, T = 1, body force g = 0.001 along
x, dt = 0.02, rotation angle 120 degrees.  The analytic collisional viscosity
of SRD is eta = (1 - cos a) / (18 dt) (n - 1 + e^-n) = 37.50 (the kinetic part,
about 0.085, is below 0.3 % and left out, as in the reference's own check,
README.md:94-102).

Estimator: the lab-grid sampled x-velocity averaged over x and y gives u(z);
the steady profile is u(z) = u0 - (n g / 2 eta) z^2, so a least-squares fit of
cell averages of a - b z^2 over the fluid layers gives eta = n g / (2 b).  The
curvature does not depend on where the walls sit or on slip at them.  The
slowest mode of the start-up flow decays with tau = L^2 / (pi^2 nu) = 270 time
units = 13,500 steps, so the warm-up is 5 tau before sampling.  Independent
replicas, run as one batched ensemble, give the error bar.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from cudampcd_gb300 import capi

pytestmark = pytest.mark.gpu

LX, LY, LZ_FLUID = 10, 10, 100
N_PER_CELL, DRAG, DT = 10, 0.001, 0.02
ALPHA = 2.0 * math.pi / 3.0
ETA_THEORY = (1.0 - math.cos(ALPHA)) / (18.0 * DT) * (N_PER_CELL - 1 + math.exp(-N_PER_CELL))
TAU_STEPS = 13_500


REPLICAS = 16


def profiles_from_sample(h: capi.Handle, steps: int) -> np.ndarray:
    """u_x(z) of every replica's container layers, averaged over x and y, for a
    sample of `steps` steps.  The sampled mean divides by steps - 1 (the
    reference's getSampleMean, cuda_backend_impl.cu:199-210); undo that here."""
    h.step_and_sample(steps)
    _, vel = h.sample_mean()
    vx = vel[:, 0].reshape(REPLICAS, LZ_FLUID + 2, LY, LX)   # per box: x + Lx (y + Ly z)
    return vx.mean(axis=(2, 3)).astype(np.float64) * (steps - 1) / steps


def fit_eta(u: np.ndarray) -> float:
    """eta from the curvature of u(z) over the fluid layers: cell averages of
    a - b z^2 over [zc - 1/2, zc + 1/2] are a - b (zc^2 + 1/12)."""
    zc = np.arange(LZ_FLUID + 2) + 0.5 - (LZ_FLUID + 2) / 2.0
    fluid = slice(1, LZ_FLUID + 1)
    A = np.stack([np.ones(LZ_FLUID), -(zc[fluid] ** 2 + 1.0 / 12.0)], axis=1)
    (a, b), *_ = np.linalg.lstsq(A, u[fluid], rcond=None)
    return N_PER_CELL * DRAG / (2.0 * b)


def test_srd_viscosity_within_two_percent_of_theory():
    """16 independent replicas of the 10 x 10 x 100 channel (seeds 2024 + r), advanced
    together as one batched ensemble; the slowest mode relaxes over 13,500 steps, so
    time blocks of one channel are correlated and the error bar comes from the
    spread over the independent replicas instead."""
    assert abs(ETA_THEORY - 37.50) < 0.01
    box = dict(L=(LX, LY, LZ_FLUID + 2), periodic=(1, 1, 0), n=N_PER_CELL, dt=DT, drag=DRAG)
    h = capi.Handle(boxes=[dict(box, seed=2024 + r) for r in range(REPLICAS)])
    try:
        h.step(5 * TAU_STEPS)
        u = np.mean([profiles_from_sample(h, 10_000) for _ in range(10)], axis=0)   # (replica, z)
        assert h.counters()[1] == 0
    finally:
        h.close()
    etas = np.array([fit_eta(ur) for ur in u])
    eta = fit_eta(u.mean(axis=0))
    err = etas.std(ddof=1) / math.sqrt(REPLICAS)
    print(f"eta = {eta:.3f} +- {err:.3f} over {REPLICAS} replicas (per replica {np.round(etas, 1)}), "
          f"theory {ETA_THEORY:.3f}, deviation {100 * (eta / ETA_THEORY - 1):+.2f} %")
    assert abs(eta / ETA_THEORY - 1.0) < 0.02
    assert err / ETA_THEORY < 0.01   # the estimate is precise enough for the 2 % bound to mean something

"""Wall pressure and density profile (equation of state) against theory and the reference.

The reference has no pressure measurement.  The estimator (mpcd_gb_wall_pressure)
is the momentum per unit area and time that the fluid gives the two z walls:
bounce-backs plus the momentum the wall ghosts take up in collisions.  It is
applied identically to the oracle's restatement of the reference CPU step
(orc_run_pressure_steps, reference Xoshiro draws).
- SRD is an ideal gas: its pressure must be n T.
- The extended MPC collision (stochastic gate, non-ideal equation of state) must
  give the reference's pressure, density profile and viscosity within statistical
  error.
"""
from __future__ import annotations

import math
import multiprocessing as mp

import numpy as np
import pytest

import oracle as O
from cudampcd_gb300 import capi

pytestmark = pytest.mark.gpu


def gpu_blocks(alg, L, n, steps, blocks, seed, T=1.0):
    h = capi.Handle(L=L, periodic=(1, 1, 0), n=n, dt=0.02, drag=0.0, temperature=T, algorithm=alg, seed=seed)
    try:
        h.step(300)
        P = []
        for _ in range(blocks):
            h.wall_pressure(restart=True)
            h.step(steps)
            p0, p1, k = h.wall_pressure()
            assert k == steps
            P.append((p0 + p1) / 2)
        h.step_and_sample(steps * blocks)
        density, _ = h.sample_mean()
        S = steps * blocks
        layers = density.reshape(L[2], L[1], L[0]).mean(axis=(1, 2)) * (S - 1) / S
        assert h.counters()[1] == 0
    finally:
        h.close()
    P = np.array(P)
    return P.mean(), P.std(ddof=1) / np.sqrt(len(P)), layers


def oracle_blocks(alg, L, n, steps, blocks, seed):
    box = O.Box(L=L, periodic=(1, 1, 0), n=n, dt=0.02, drag=0.0, algorithm=alg)
    r = O.Run(box, seed)
    try:
        imp = np.zeros(2)
        r.pressure_steps(300, imp)
        P, layers = [], np.zeros(L[2])
        for _ in range(blocks):
            imp[:] = 0.0
            r.pressure_steps(steps, imp, layers)
            P.append(imp.mean() / (L[0] * L[1] * steps * 0.02))
    finally:
        r.close()
    P = np.array(P)
    return P.mean(), P.std(ddof=1) / np.sqrt(len(P)), layers / (L[0] * L[1] * steps * blocks)


def test_srd_wall_pressure_is_the_ideal_gas_pressure():
    """Three independent runs; the error bar comes from their spread.  Consecutive
    blocks of one run are correlated (the pressure relaxes slowly), and their
    standard error understates the spread of independent runs by a factor of about
    three (eight seeds: block z-scores up to 4.6, seed means within 0.3 % of n T)."""
    n, T = 10, 1.3
    runs = [gpu_blocks(0, (16, 16, 22), n, 2000, 10, seed=seed, T=T) for seed in (4, 5, 6)]
    means = np.array([r[0] for r in runs])
    P = means.mean()
    err = max(means.std(ddof=1) / np.sqrt(len(means)), max(r[1] for r in runs))
    layers = np.mean([r[2] for r in runs], axis=0)
    print(f"SRD wall pressure {P:.4f} +- {err:.4f} (runs {means}), n T = {n * T}")
    assert abs(P - n * T) < max(4 * err, 1e-3 * n * T)
    assert abs(P / (n * T) - 1) < 0.01
    fluid = layers[1:-1]
    # the wall layers stay (nearly) empty: only lone particles, which keep their shifted
    # position (simulation_functions.cpp:169-191), are sampled there
    assert np.all(np.abs(fluid / n - 1) < 0.03) and layers[0] < 1e-3 and layers[-1] < 1e-3


def test_extended_pressure_and_density_match_the_reference_cpu_step():
    L, n = (8, 8, 12), 10
    Pg, eg, lg = gpu_blocks(1, L, n, 4000, 16, seed=6)
    Po, eo, lo = oracle_blocks(O.EXTENDED, L, n, 1000, 8, seed=6)
    sigma = np.hypot(eg, eo)
    print(f"extended MPC wall pressure: GPU {Pg:.4f} +- {eg:.4f}, reference CPU step {Po:.4f} +- {eo:.4f}, "
          f"n T = {n}; density layers GPU {np.round(lg[1:-1], 3)} reference {np.round(lo[1:-1], 3)}")
    assert abs(Pg - Po) < 4 * sigma
    assert np.all(np.abs(lg[1:-1] - lo[1:-1]) < 0.05 * n)


# ---------------------------------------------------------------- viscosity of the extended collision

VISC = dict(L=(8, 8, 12), n=10, drag=0.01, warm=6000, sample=20000)


def _fit_eta(u: np.ndarray, Lz: int, n: int, g: float) -> float:
    zc = np.arange(Lz) + 0.5 - Lz / 2.0
    A = np.stack([np.ones(Lz - 2), -(zc[1:-1] ** 2 + 1.0 / 12.0)], axis=1)
    (_, b), *_ = np.linalg.lstsq(A, u[1:-1], rcond=None)
    return n * g / (2.0 * b)


def _oracle_profile(seed: int) -> np.ndarray:
    """u_x(z) of one channel advanced by the restated reference CPU step (pool worker)."""
    L, n, g = VISC["L"], VISC["n"], VISC["drag"]
    box = O.Box(L=L, periodic=(1, 1, 0), n=n, dt=0.02, drag=g, algorithm=O.EXTENDED)
    pos, vel, _ = O.distribute(box, box.N_fluid, seed, seed + 1)
    rng = O.xoshiro(seed + 2, seed + 3)
    pos, vel = O.reference_steps(box, pos, vel, rng, VISC["warm"])[:2]
    sampler = O.Sampler(box)
    O.reference_steps(box, pos, vel, rng, VISC["sample"], sampler)
    _, v = sampler.mean()
    S = VISC["sample"]
    return v[:, 0].reshape(L[2], L[1], L[0]).mean(axis=(1, 2)).astype(np.float64) * (S - 1) / S


def test_extended_viscosity_matches_the_reference_cpu_step():
    """Poiseuille viscosity of the extended collision: 8 reference-step channels
    (spawned worker processes) against 32 GPU replicas of the same channel; each
    side's error bar is the spread over its independent replicas."""
    L, n, g = VISC["L"], VISC["n"], VISC["drag"]
    with mp.get_context("spawn").Pool(8) as pool:
        pending = pool.map_async(_oracle_profile, [100 + 7 * r for r in range(8)])
        R = 32
        h = capi.Handle(boxes=[dict(L=L, periodic=(1, 1, 0), n=n, dt=0.02, drag=g, algorithm=1, seed=500 + r)
                               for r in range(R)])
        try:
            h.step(VISC["warm"])
            h.step_and_sample(VISC["sample"])
            _, v = h.sample_mean()
            assert h.counters()[1] == 0
        finally:
            h.close()
        S = VISC["sample"]
        ug = v[:, 0].reshape(R, L[2], L[1], L[0]).mean(axis=(2, 3)).astype(np.float64) * (S - 1) / S
        uo = np.array(pending.get(timeout=1200))
    eg = np.array([_fit_eta(u, L[2], n, g) for u in ug])
    eo = np.array([_fit_eta(u, L[2], n, g) for u in uo])
    mg, sg = _fit_eta(ug.mean(axis=0), L[2], n, g), eg.std(ddof=1) / math.sqrt(len(eg))
    mo, so = _fit_eta(uo.mean(axis=0), L[2], n, g), eo.std(ddof=1) / math.sqrt(len(eo))
    print(f"extended MPC viscosity: GPU {mg:.3f} +- {sg:.3f}, reference CPU step {mo:.3f} +- {so:.3f}")
    assert abs(mg - mo) < 4 * math.hypot(sg, so)
    assert sg / mg < 0.03 and so / mo < 0.05

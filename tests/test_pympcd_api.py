"""The reference's Python API, run against this repository's module.

The first two tests restate the reference's own integration tests
(tests/python/test_integration.py: a basic run, and positions changing after a
step); the third follows the README example (README.md:47-100): Params as
documented, Simulation(params, "cuda"), step, step_and_sample and
get_mean_fields with the reference's array shapes, giving a Poiseuille profile.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import cudampcd_gb300 as pympcd

pytestmark = pytest.mark.gpu


def test_basic_simulation():
    params = pympcd.Params()
    params.volume_size = [10, 10, 10]
    params.n = 5
    sim = pympcd.Simulation(params)
    sim.step(10)
    positions = sim.get_particle_positions()
    assert len(positions) > 0 and positions.shape == (sim.num_particles, 3)


def test_memory_consistency():
    params = pympcd.Params()
    params.volume_size = [5, 5, 5]
    params.n = 2
    sim = pympcd.Simulation(params)
    pos1 = sim.get_particle_positions()
    sim.step(1)
    pos2 = sim.get_particle_positions()
    assert not np.allclose(pos1, pos2)


def test_readme_poiseuille_flow():
    params = pympcd.Params()
    params.n = 10
    params.temperature = 1.0
    params.volume_size = (10, 10, 40)
    params.periodicity = (1, 1, 0)
    params.drag = 0.005
    params.delta_t = 0.02
    params.experiment = "standard"
    params.algorithm = "srd"
    params.collision_kernel = "optimized"
    params.seed = 3
    assert tuple(params.volume_size) == (10, 10, 42)   # the wall layers are added
    sim = pympcd.Simulation(params, "cuda")
    sim.step(15000)   # about 7 relaxation times of a 40-layer channel
    sim.step_and_sample(5000)
    density, velocity = sim.get_mean_fields()
    assert density.shape == (10, 10, 42) and velocity.shape == (10, 10, 42, 3)
    assert abs(density[:, :, 1:-1].mean() - params.n) < 0.05 * params.n
    profile = velocity[:, :, :, 0].mean(axis=(0, 1))
    L = params.volume_size[2] - 2
    eta = L * L * params.n * params.drag / (8 * profile.max())   # the README's estimate
    eta_theo = (1 - math.cos(120 / 180 * math.pi)) / (6 * 3 * params.delta_t) * (params.n - 1 + math.exp(-params.n))
    assert profile[21] > profile[5] > profile[1] > 0
    assert abs(eta / eta_theo - 1) < 0.1


def test_unsupported_backend_is_an_error():
    params = pympcd.Params()
    params.volume_size = [4, 4, 4]
    with pytest.raises(Exception, match="Unsupported backend"):
        pympcd.Simulation(params, "cpu")

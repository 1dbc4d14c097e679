"""The reference's own Python binding, running the GB300 step.

baseline/build_ref.py compiles the reference's unchanged src/bindings/bindings.cpp,
SimulationHandle (src/libmpcd/api/simulator_handle.cpp) and CPU backend, with the
GbBackend class (baseline/dropin/gb300_backend.hpp) and the factory diff
(baseline/dropin/backend_factory.diff), against libmpcd_gb.so
(baseline/_ref/dropin/pympcd).  These tests import that module in a
child process (the reference's module is also named `pympcd`, and pybind11 keeps
one registration of its classes per process) and run the flows of the reference's
own integration tests (tests/python/test_integration.py: a basic run, positions
changing after a step) and of its README example (README.md:47-100: a Poiseuille
channel, step / step_and_sample / get_mean_fields), then check that the process
ran the GB300 library: libmpcd_gb.so is mapped, and the particle count is the
GB300 backend's.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from baseline import build_ref  # noqa: E402

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import json, math, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import pympcd

out = {}
# tests/python/test_integration.py: a basic run
params = pympcd.Params()
params.volume_size = (10, 10, 10)
params.n = 5
sim = pympcd.Simulation(params, "cuda")
sim.step(10)
pos = sim.get_particle_positions()
out["basic"] = [int(pos.shape[0]), int(pos.shape[1])]
# positions change after a step
params = pympcd.Params()
params.volume_size = (5, 5, 5)
params.n = 2
sim = pympcd.Simulation(params, "cuda")
p1 = sim.get_particle_positions()
sim.step(1)
p2 = sim.get_particle_positions()
out["moved"] = bool(not np.allclose(p1, p2))
del sim
# README example: Poiseuille channel
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
sim = pympcd.Simulation(params, "cuda")
sim.step(15000)
sim.step_and_sample(5000)
density, velocity = sim.get_mean_fields()
out["shapes"] = [list(density.shape), list(velocity.shape)]
out["density_fluid"] = float(density[:, :, 1:-1].mean())
profile = velocity[:, :, :, 0].mean(axis=(0, 1))
out["profile"] = [float(x) for x in profile]
v = sim.get_particle_velocities()
out["n_particles"] = int(v.shape[0])
# the reference's CPU backend is still there
params = pympcd.Params()
params.volume_size = (4, 4, 4)
params.n = 3
cpu = pympcd.Simulation(params, "cpu")
cpu.step(2)
out["cpu_particles"] = int(cpu.get_particle_positions().shape[0])
with open("/proc/self/maps") as f:
    maps = f.read()
out["libmpcd_gb_mapped"] = "libmpcd_gb.so" in maps
out["module"] = pympcd._pympcd.__file__
print("RESULT " + json.dumps(out))
"""


def test_reference_binding_runs_the_gb300_step():
    if not os.path.exists(build_ref.module_path("dropin")):
        pytest.skip("the reference's binding was not built (no reference sources staged in baseline/_ref)")
    proc = subprocess.run([sys.executable, "-c", SCRIPT, build_ref.module_dir("dropin")], capture_output=True,
                          text=True, timeout=900)
    assert proc.returncode == 0, proc.stderr[-3000:]
    line = [l for l in proc.stdout.splitlines() if l.startswith("RESULT ")][-1]
    r = json.loads(line[len("RESULT "):])
    assert r["libmpcd_gb_mapped"], "the reference module did not load libmpcd_gb.so"
    assert "baseline/_ref/dropin" in r["module"].replace(os.sep, "/")
    assert r["basic"] == [10 * 10 * 10 * 5, 3]
    assert r["moved"]
    assert r["shapes"] == [[10, 10, 42], [10, 10, 42, 3]]
    # sampled density: n, times S / (S - 1) from the reference's sample count quirk
    assert abs(r["density_fluid"] - 10 * 5000 / 4999) < 0.05 * 10
    # n x fluid cells: the GB300 backend's count (the reference's CUDA backend
    # allocates n x container cells, 10 x 10 x 42 x 10, backend_context.cu:19)
    assert r["n_particles"] == 10 * 10 * 10 * 40
    assert r["cpu_particles"] == 4 * 4 * 4 * 3
    prof = r["profile"]
    L, n, g, dt = 40, 10, 0.005, 0.02
    eta = L * L * n * g / (8 * max(prof))   # the README's estimate
    eta_theo = (1 - (-0.5)) / (18 * dt) * (n - 1 + 2.718281828459045 ** -n)
    assert prof[21] > prof[5] > prof[1] > 0
    assert abs(eta / eta_theo - 1) < 0.1


"""GPU parity of the MPCD step against the oracle (which is pinned to the reference).

All calls go through the C ABI of libmpcd_gb.so (cudampcd_gb300.capi).

* streaming + cell index + counts + sort permutation: bit-exact for an injected
  grid shift (reference: translate_particles, simulation_functions.cpp:38-103,
  and a stable sort by cell);
* collision fed the draws the reference CPU code consumed (recorded by the
  oracle's Xoshiro128+ replay): positions bit-exact, velocities within 1e-5;
* production (Philox) draws vs the oracle's restatement of the same draw model;
* momentum / energy conservation, determinism, sampling, getters and setters.
"""
import numpy as np
import pytest

import oracle as O
from _helpers import REL_TOL, make, rel_err, set_state

pytestmark = pytest.mark.gpu

BOXES = {
    "srd_periodic": O.Box(L=(6, 5, 7), periodic=(1, 1, 1), algorithm=O.SRD, n=8, dt=0.05, drag=0.01),
    "srd_walls": O.Box(L=(6, 5, 9), periodic=(1, 1, 0), algorithm=O.SRD, n=10, dt=0.05, drag=0.01),
    "srd_walls_dense": O.Box(L=(4, 4, 10), periodic=(1, 1, 0), algorithm=O.SRD, n=20, dt=0.02, drag=0.001),
    "ext_periodic": O.Box(L=(5, 5, 6), periodic=(1, 1, 1), algorithm=O.EXTENDED, n=20, dt=0.02, drag=0.0005),
    "ext_walls": O.Box(L=(4, 5, 8), periodic=(1, 1, 0), algorithm=O.EXTENDED, n=20, dt=0.02, drag=0.0005),
    # channel: Lx == Lz, because the reference's channel init takes the radius from
    # Lx (simulation_functions.cpp:11) and otherwise overfills the cells
    "channel": O.Box(L=(8, 8, 8), periodic=(1, 0, 0), experiment=O.CHANNEL, algorithm=O.SRD, n=6, dt=0.05,
                     drag=0.01),
}

SHIFTS = [(0.13, -0.31, -0.22), (0.21, 0.44, 0.37), (-0.5, 0.0, 0.4999)]


@pytest.mark.parametrize("name", list(BOXES))
@pytest.mark.parametrize("shift", SHIFTS)
def test_stream_keys_counts_permutation_bit_exact(name, shift):
    box = BOXES[name]
    h = make(box, seed=11)
    pos, vel, _ = O.distribute(box, h.N, 3, 4)
    cell, slot, pid, counts = set_state(h, pos, vel, shift)
    tp, tv, tc, counter, _ = O.translate(box, pos, vel, np.float32(shift))
    assert np.array_equal(counts, counter)
    # every particle of the layout sits in the reference's cell of its index
    assert np.array_equal(cell, tc[pid])
    # the layout is the stable sort of the (id-ordered) array by storage cell
    assert counts.max() <= 4 * box.n, "test configuration must not overflow a cell"
    perm = O.stable_perm(O.storage_index(box, tc), box.C)
    assert np.array_equal(pid, perm)
    # the clean state is stored unchanged and read back by particle id
    assert np.array_equal(h.positions(), pos) and np.array_equal(h.velocities(), vel)
    h.close()


def test_translate_known_answer():
    """test_simulation_functions.cpp:4-43 / test_simulation_kernels.cu:16-47 through the GPU path.

    Every particle starts at the origin, so most cells overflow their 4n slots:
    counts and the cell of every particle stay exact (which particles overflow
    follows arrival order on the GPU, index order in the reference)."""
    box = O.Box(L=(10, 10, 10), periodic=(1, 1, 1), n=10, dt=1.0)
    h = make(box)
    v = O.xoshiro_sequence(42, 43, 3, h.N)
    cell, _, pid, counts = set_state(h, np.zeros((h.N, 3), np.float32), v, (0, 0, 0))
    assert np.array_equal(cell, O.cell_index(box, v[pid]))   # after dt = 1 the position equals the velocity
    _, _, _, counter, _ = O.translate(box, np.zeros((h.N, 3), np.float32), v, (0, 0, 0))
    assert np.array_equal(counts, counter)
    # all particles at (-5, -5, -5) with zero velocity land in cell 0
    h.inject_shift(h.step_index, (0, 0, 0))
    h.set_particles(np.full((h.N, 3), -5.0, np.float32), np.zeros((h.N, 3), np.float32))
    counts = h.layout()[3]
    assert counts[0] == h.N and counts[1:].sum() == 0
    overflowed, flags = h.counters()
    assert overflowed >= h.N - 4 * box.n and flags == 0
    h.close()


def _collide_with_reference_draws(box, shift0, shift1, seed_a, seed_b):
    h = make(box, seed=99)
    pos, vel, _ = O.distribute(box, h.N, seed_a, seed_b)
    set_state(h, pos, vel, shift0)
    tp, tv, tc, counter, table = O.translate(box, pos, vel, np.float32(shift0))
    draws = O.Draws.empty(box)
    op, ov, oc = O.collide(box, tp, tv, tc, counter, table, np.float32(shift0), draws, O.DRAWS_XOSHIRO,
                           rng=O.xoshiro(seed_a, seed_b))
    h.inject_shift(h.step_index + 1, shift1)
    h.inject_draws(draws)
    h.step(1)
    gp, gv = h.positions(), h.velocities()
    cell_out, _, id_out, counts_out = h.layout()
    # the new layout is keyed by the cell after streaming the next step: the
    # stable sort of the id-ordered collided state by that cell
    _, _, nc, ncount, _ = O.translate(box, op, ov, np.float32(shift1))
    expect = O.stable_perm(O.storage_index(box, nc), box.C)
    h.close()
    return dict(pos=pos, vel=vel, gp=gp, gv=gv, op=op, ov=ov, draws=draws, tc=tc, tv=tv, nc=nc,
                ncount=ncount, counts_out=counts_out, id_out=id_out, expect=expect, cell_out=cell_out)


@pytest.mark.parametrize("name", list(BOXES))
@pytest.mark.parametrize("seeds", [(5, 7), (8, 1)])
def test_collision_matches_reference_draws(name, seeds):
    box = BOXES[name]
    r = _collide_with_reference_draws(box, SHIFTS[0], SHIFTS[1], *seeds)
    # positions after the collision: exact
    assert np.array_equal(r["gp"], r["op"])
    # velocities: within the tolerance (exact where no transcendental is involved)
    err = rel_err(r["gv"], r["ov"], box.thermal_velocity)
    if box.algorithm == O.EXTENDED:
        # a gate comparison u < 1 - exp(...) can flip at the last ulp of exp; allow
        # such cells only where |u - p| is below 1e-6 (none expected at these sizes)
        assert err.max() <= REL_TOL or (err > REL_TOL).any(axis=1).sum() <= 2
    else:
        assert err.max() <= REL_TOL
    # next layout = stable sort of the collided state by the next cell
    assert np.array_equal(r["counts_out"], r["ncount"])
    assert np.array_equal(r["id_out"], r["expect"])
    assert np.array_equal(r["cell_out"], r["nc"][r["id_out"]])


def test_srd_collision_at_fp32_rounding_of_reference_draws():
    """The SRD cell mean is an exact fixed-point sum rounded once; the reference
    sums in float in index order.  They differ by a few ulp at most."""
    box = BOXES["srd_walls_dense"]
    r = _collide_with_reference_draws(box, SHIFTS[2], SHIFTS[0], 21, 22)
    assert np.array_equal(r["gp"], r["op"])
    assert rel_err(r["gv"], r["ov"], box.thermal_velocity).max() <= 2e-6


@pytest.mark.parametrize("name", ["srd_periodic", "srd_walls", "ext_periodic", "ext_walls", "channel"])
def test_production_step_matches_oracle_draw_model(name):
    box = BOXES[name]
    seed = 2024
    h = make(box, seed=seed)
    pos, vel, _ = O.distribute(box, h.N, 31, 32)
    k = h.step_index
    set_state(h, pos, vel)
    s0 = h.shift(k)
    assert np.array_equal(s0, O.gb_shift(seed, k))
    h.step(1)
    gp, gv = h.positions(), h.velocities()
    tp, tv, tc, counter, table = O.translate(box, pos, vel, s0)
    op, ov, _ = O.collide(box, tp, tv, tc, counter, table, s0, O.Draws.empty(box), O.DRAWS_PHILOX, seed=seed,
                          step=k)
    assert rel_err(gp, op, 1.0).max() <= REL_TOL
    err = rel_err(gv, ov, box.thermal_velocity)
    assert err.max() <= REL_TOL or (box.algorithm == O.EXTENDED and (err > REL_TOL).any(axis=1).sum() <= 2)
    h.close()


def test_srd_conserves_cell_momentum_and_energy():
    box = O.Box(L=(8, 8, 8), periodic=(1, 1, 1), algorithm=O.SRD, n=12, dt=0.1, drag=0.0)
    r = _collide_with_reference_draws(box, (0.1, 0.2, 0.3), (0.0, 0.0, 0.0), 1, 2)
    tc = r["tc"]
    before = np.zeros((box.C, 3))
    after = np.zeros((box.C, 3))
    e_before = np.zeros(box.C)
    e_after = np.zeros(box.C)
    np.add.at(before, tc, r["tv"].astype(np.float64))
    np.add.at(after, tc, r["gv"].astype(np.float64))
    np.add.at(e_before, tc, (r["tv"].astype(np.float64) ** 2).sum(1))
    np.add.at(e_after, tc, (r["gv"].astype(np.float64) ** 2).sum(1))
    np.testing.assert_allclose(after, before, atol=2e-5 * box.n)
    np.testing.assert_allclose(e_after, e_before, rtol=2e-5)


def test_deterministic_and_getters_are_pure():
    box = BOXES["srd_walls"]
    a, b = make(box, seed=5), make(box, seed=5)
    a.step(3)
    _ = a.positions(), a.velocities(), a.layout()   # reading must not perturb the run
    a.step(4)
    b.step(7)
    assert np.array_equal(a.positions(), b.positions()) and np.array_equal(a.velocities(), b.velocities())
    a.close()
    b.close()


def test_set_get_roundtrip_and_momentum_drift():
    box = O.Box(L=(10, 10, 12), periodic=(1, 1, 1), algorithm=O.SRD, n=10, dt=0.02, drag=0.001)
    h = make(box, seed=3)
    v0 = h.velocities()
    assert np.abs(v0.astype(np.float64).mean(0)).max() < 1e-6   # zero net momentum at init
    h.step(20)
    x, v = h.positions(), h.velocities()
    h.set_particles(x, v)
    assert np.array_equal(h.positions(), x) and np.array_equal(h.velocities(), v)
    h.set_velocities(v * 0.5)
    assert np.array_equal(h.velocities(), v * 0.5) and np.array_equal(h.positions(), x)
    # periodic box: drag adds drag*dt to every collided particle per step, so the
    # total x momentum grows linearly; y and z are conserved
    p0 = h.velocities().astype(np.float64).sum(0)
    h.step(50)
    p1 = h.velocities().astype(np.float64).sum(0)
    assert abs((p1[0] - p0[0]) / (h.N * box.drag * box.dt * 50) - 1) < 1e-2
    assert np.abs(p1[1:] - p0[1:]).max() < 1e-3
    h.close()


def test_sampling_matches_oracle_on_the_same_states():
    box = BOXES["srd_walls"]
    h = make(box, seed=17)
    sampler = O.Sampler(box)
    for _ in range(5):
        h.step_and_sample(1)
        sampler.sample(h.positions(), h.velocities(), model="gb")
    d, v = h.sample_mean()
    od, ov = sampler.mean(model="gb")
    np.testing.assert_allclose(d, od, rtol=1e-6)
    np.testing.assert_allclose(v, ov, rtol=1e-5, atol=1e-5)
    h.close()


def test_invalid_parameters_raise():
    from cudampcd_gb300 import capi

    with pytest.raises(capi.GbError, match="volume_size"):
        capi.Handle(L=(10, 10, 0.5))
    with pytest.raises(capi.GbError, match="n must"):
        capi.Handle(n=0)


EXTREME = {
    # one particle per cell: most cells hold 0-2 particles (lone particles skip the
    # collision and keep their shifted position), 128-cell tiles
    "srd_sparse": O.Box(L=(12, 10, 9), periodic=(1, 1, 0), algorithm=O.SRD, n=1, dt=0.05, drag=0.01),
    "srd_n3": O.Box(L=(10, 9, 8), periodic=(1, 1, 0), algorithm=O.SRD, n=3, dt=0.05, drag=0.01),
    # dense cells: 16-cell tiles, up to 5n = 320 staged entries in one cell with its ghosts
    "srd_dense": O.Box(L=(4, 4, 6), periodic=(1, 1, 0), algorithm=O.SRD, n=64, dt=0.02, drag=0.001),
    "ext_dense": O.Box(L=(4, 3, 5), periodic=(1, 1, 0), algorithm=O.EXTENDED, n=64, dt=0.02, drag=0.001),
    # the densest accepted n: the particle buffer is 5n = 2045 entries (a full
    # bucket and its ghosts), and 8-cell tiles run as several sub-tiles
    "srd_max_density": O.Box(L=(3, 3, 4), periodic=(1, 1, 0), algorithm=O.SRD, n=409, dt=0.02, drag=0.001),
    # a single fluid layer between the walls
    "srd_one_layer": O.Box(L=(6, 6, 3), periodic=(1, 1, 0), algorithm=O.SRD, n=10, dt=0.05, drag=0.01),
}


@pytest.mark.parametrize("name", list(EXTREME))
def test_extreme_densities_and_thin_boxes_match_oracle(name):
    box = EXTREME[name]
    seed = 77
    h = make(box, seed=seed)
    pos, vel, _ = O.distribute(box, h.N, 3, 4)
    k = h.step_index
    set_state(h, pos, vel)
    s0 = h.shift(k)
    h.step(1)
    gp, gv = h.positions(), h.velocities()
    tp, tv, tc, counter, table = O.translate(box, pos, vel, s0)
    op, ov, _ = O.collide(box, tp, tv, tc, counter, table, s0, O.Draws.empty(box), O.DRAWS_PHILOX, seed=seed,
                          step=k)
    assert rel_err(gp, op, 1.0).max() <= REL_TOL
    # A cell that received more than 4n particles overflows: as in the reference, its
    # 4n lowest particle ids collide and the others skip the collision, whatever the
    # order in which the GPU's claims arrived.
    cap = 4 * box.n
    if name == "srd_sparse":
        assert (counter[tc] > cap).any()   # n = 1 does overflow some cells
    err = rel_err(gv, ov, box.thermal_velocity)
    assert err.max() <= REL_TOL or (box.algorithm == O.EXTENDED and (err > REL_TOL).any(axis=1).sum() <= 2)
    h.step(5)   # and keeps stepping without device errors
    assert h.counters()[1] == 0
    h.close()


def test_fast_particles_take_the_64_bit_sums():
    """Speeds of 32 and more (1 % of the particles at |vx| = 40): the run kernel's
    SRD cell sums leave their 32-bit fast path for 64-bit sums.  Two production
    steps; the getters replay a step with the tile kernel, so the second step (whose
    inputs are the run kernel's output of the first) is compared with the oracle's
    restatement of the reference step (Philox draw model) applied to the state read
    after the first."""
    box = O.Box(L=(8, 8, 8), periodic=(1, 1, 1), algorithm=O.SRD, n=10, dt=0.005, drag=0.0)
    seed = 91
    h = make(box, seed=seed)
    try:
        pos, vel, _ = O.distribute(box, h.N, 7, 8)
        fast = np.arange(0, h.N, 100)
        vel = vel.copy()
        vel[fast, 0] = np.where(fast % 200 == 0, 40.0, -40.0).astype(np.float32)
        set_state(h, pos, vel)
        h.step(1)
        pos, vel = h.positions(), h.velocities()
        assert (np.abs(vel) >= 32.0).sum() >= len(fast) // 2   # still fast after one collision
        k = h.step_index
        s0 = h.shift(k)
        h.step(1)
        gp, gv = h.positions(), h.velocities()
        tp, tv, tc, counter, table = O.translate(box, pos, vel, s0)
        op, ov, _ = O.collide(box, tp, tv, tc, counter, table, s0, O.Draws.empty(box), O.DRAWS_PHILOX, seed=seed,
                              step=k)
        assert rel_err(gp, op, 1.0).max() <= REL_TOL
        assert rel_err(gv, ov, box.thermal_velocity).max() <= REL_TOL
        assert h.counters()[1] == 0
    finally:
        h.close()


# Boxes large enough that every CTA of the persistent step kernel (4 per SM x 152
# SMs) sweeps many tiles: the next-tile locator, the one-tile-ahead count prefetch,
# the in-sweep clearing of the previous step's counts and the overflow chains all
# run as in production.  (box, production steps compared)
MULTI_TILE = {
    # 160 x 160 x 20 fluid layers + 2 walls, n = 20: 563,200 cells, 8,800 tiles of 64
    # cells, about 14 per CTA
    "srd_160x160x20": (O.Box(L=(160, 160, 22), periodic=(1, 1, 0), algorithm=O.SRD, n=20, dt=0.02, drag=0.001), 3),
    # extended, 100 x 100 x 20 + 2 walls: 220,000 cells in 64-cell tiles
    "ext_100x100x20": (O.Box(L=(100, 100, 22), periodic=(1, 1, 0), algorithm=O.EXTENDED, n=20, dt=0.02,
                             drag=0.0005), 2),
    # n = 1 over 200 x 200 x 10 + 2 walls: 480,000 cells in 128-cell tiles, and
    # cells that receive more than 4n particles in most tiles
    "srd_sparse_200x200x10": (O.Box(L=(200, 200, 12), periodic=(1, 1, 0), algorithm=O.SRD, n=1, dt=0.05,
                                    drag=0.01), 3),
}


@pytest.mark.parametrize("name", list(MULTI_TILE))
def test_multi_tile_production_steps_match_oracle(name):
    """Consecutive production steps of a large box, each compared with the oracle's
    restatement of the reference step (Philox draw model) applied to the GPU's own
    state before it: positions and velocities of every particle within 1e-5.  In
    the extended collision, a gate draw within FP32 rounding of its probability can
    flip between the GPU's fixed-tree sums and the oracle's sequential ones; the
    particles off by more than the tolerance must then all share one collision cell."""
    box, steps = MULTI_TILE[name]
    seed = 4242
    h = make(box, seed=seed)
    try:
        pos, vel, _ = O.distribute(box, h.N, 13, 14)
        set_state(h, pos, vel)
        overflowed = False
        for _ in range(steps):
            k = h.step_index
            s0 = h.shift(k)
            h.step(1)
            gp, gv = h.positions(), h.velocities()
            tp, tv, tc, counter, table = O.translate(box, pos, vel, s0)
            overflowed |= bool((counter > 4 * box.n).any())
            op, ov, _ = O.collide(box, tp, tv, tc, counter, table, s0, O.Draws.empty(box), O.DRAWS_PHILOX,
                                  seed=seed, step=k)
            assert rel_err(gp, op, 1.0).max() <= REL_TOL
            bad = (rel_err(gv, ov, box.thermal_velocity) > REL_TOL).any(axis=1)
            if box.algorithm == O.EXTENDED:
                assert len(np.unique(tc[bad])) <= 1, f"step {k}: {bad.sum()} particles in several cells differ"
            else:
                assert not bad.any(), f"step {k}: {bad.sum()} particles differ"
            pos, vel = gp, gv
        assert h.counters()[1] == 0
        if box.n == 1:
            assert overflowed and h.counters()[0] > 0
    finally:
        h.close()

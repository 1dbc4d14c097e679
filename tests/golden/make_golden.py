"""Generate golden vectors from the reference's own CPU code.

Runs oracle/_ref/libmpcd_ref.so (the reference's src/libmpcd/cpu_backend sources
compiled by oracle/build_oracle.py) on small seeded cases and stores inputs and
outputs in tests/golden/*.npz.  Run where the reference tree is present:

    python tests/golden/make_golden.py

The fixtures let the oracle be checked against the reference on machines where
the reference sources are absent.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402

# (name, L, periodic, algorithm, n, dt, drag, shift, collision seeds)
CASES = [
    ("srd_periodic", (6, 5, 7), (1, 1, 1), O.SRD, 8, 0.05, 0.01, (0.13, -0.31, -0.22), (5, 7)),
    ("srd_walls", (6, 5, 9), (1, 1, 0), O.SRD, 8, 0.05, 0.01, (0.21, 0.44, 0.37), (9, 4)),
    ("srd_walls_neg", (5, 6, 8), (1, 1, 0), O.SRD, 10, 0.02, 0.001, (-0.05, 0.12, -0.41), (3, 1)),
    ("ext_periodic", (5, 5, 6), (1, 1, 1), O.EXTENDED, 20, 0.02, 0.0005, (0.3, -0.1, 0.05), (8, 8)),
    ("ext_walls", (4, 5, 8), (1, 1, 0), O.EXTENDED, 20, 0.02, 0.0005, (-0.4, 0.25, -0.33), (6, 2)),
    ("ext_walls_pos", (5, 4, 7), (1, 1, 0), O.EXTENDED, 20, 0.02, 0.0005, (0.1, -0.2, 0.29), (1, 77)),
]


def ref_case(R, name, L, periodic, algo, n, dt, drag, shift, seeds):
    box = O.Box(L=L, periodic=periodic, algorithm=algo, n=n, dt=dt, drag=drag)
    N = box.N_fluid
    Lr, Pr = np.array(L, np.int32), np.array(periodic, np.int32)
    pos = np.zeros((N, 3), np.float32)
    vel = np.zeros((N, 3), np.float32)
    cell0 = np.zeros(N, np.uint32)
    R.ref_distribute(Lr, Pr, 0, np.float32(1.0), N, 1000 + len(name), 2000 + n, pos.reshape(-1),
                     vel.reshape(-1), cell0)
    shift = np.array(shift, np.float32)
    cap = 4 * n
    tp, tv = pos.copy(), vel.copy()
    counter = np.zeros(box.C, np.uint32)
    table = np.zeros(box.C * cap, np.uint32)
    tcell = np.zeros(N, np.uint32)
    R.ref_translate(Lr, Pr, 0, np.float32(dt), shift, N, tp.reshape(-1), tv.reshape(-1), counter, table, cap, tcell)
    cp, cv, ccell = tp.copy(), tv.copy(), tcell.copy()
    R.ref_collision(algo, Lr, Pr, np.float32(dt), np.float32(drag), np.float32(1.0), n, shift, N, cp.reshape(-1),
                    cv.reshape(-1), counter, table, cap, seeds[0], seeds[1], ccell)
    # whole backend: 6 sampled steps from the distributed state
    h = R.ref_backend_create(Lr, Pr, 0, algo, np.float32(dt), np.float32(drag), np.float32(1.0), n, N)
    R.ref_backend_set(h, pos.reshape(-1), vel.reshape(-1))
    R.ref_backend_seed(h, seeds[1], seeds[0])
    R.ref_backend_step_and_sample(h, 6)
    bp = np.zeros((N, 3), np.float32)
    bv = np.zeros((N, 3), np.float32)
    R.ref_backend_get(h, bp.reshape(-1), bv.reshape(-1))
    md = np.zeros(box.C, np.float32)
    mv = np.zeros(3 * box.C, np.float32)
    R.ref_backend_sample_mean(h, md, mv)
    R.ref_backend_destroy(h)
    return dict(L=np.array(L), periodic=np.array(periodic), algorithm=algo, n=n, dt=np.float32(dt),
                drag=np.float32(drag), shift=shift, seeds=np.array(seeds, np.uint64),
                init_seeds=np.array([1000 + len(name), 2000 + n], np.uint64),
                pos0=pos, vel0=vel, cell0=cell0,
                pos_t=tp, vel_t=tv, cell_t=tcell, counter=counter, table=table,
                pos_c=cp, vel_c=cv, cell_c=ccell,
                pos_b=bp, vel_b=bv, mean_density=md, mean_velocity=mv.reshape(-1, 3))


def main():
    R = O.ref()
    if R is None:
        sys.exit("reference build unavailable: the reference tree is needed to make golden vectors")
    rng = {}
    for kind, label in ((0, "u32"), (1, "uniform"), (2, "gaussian"), (3, "unit_vector")):
        rng[label] = O.xoshiro_sequence(12345, 67890, kind, 2000, use_ref=True)
    np.savez_compressed(os.path.join(HERE, "xoshiro_12345_67890.npz"), **rng)
    for case in CASES:
        out = ref_case(R, *case)
        np.savez_compressed(os.path.join(HERE, f"ref_{case[0]}.npz"), **out)
        print(case[0], "N =", len(out["pos0"]))


if __name__ == "__main__":
    main()

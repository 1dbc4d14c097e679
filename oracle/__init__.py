"""ctypes front end of the MPCD oracle -- TEST INFRASTRUCTURE ONLY.

Loaded by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg to check (never to run) the CUDA path.  ``liboracle.so`` is the C
restatement of the reference CPU step (``oracle/oracle.c``); ``_ref/libmpcd_ref.so``
is the reference's own CPU code compiled by ``oracle/build_oracle.py`` where the
reference tree is present.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import build_oracle

_lib = None
_ref = None

u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

STANDARD, CHANNEL = 0, 1
SRD, EXTENDED = 0, 1
DRAWS_XOSHIRO, DRAWS_TABLE, DRAWS_PHILOX = 0, 1, 2


class OrcParams(C.Structure):
    _fields_ = [("L", C.c_int32 * 3), ("periodic", C.c_int32 * 3), ("experiment", C.c_int32),
                ("algorithm", C.c_int32), ("dt", C.c_float), ("drag", C.c_float),
                ("thermal_velocity", C.c_float), ("n_density", C.c_uint32), ("cap", C.c_uint32)]


class OrcXoshiro(C.Structure):
    _fields_ = [("s", C.c_uint32 * 4), ("generate_f", C.c_int32), ("z1_f", C.c_float)]


class OrcDraws(C.Structure):
    _fields_ = [("mode", C.c_int32), ("rng", C.POINTER(OrcXoshiro)), ("seed", C.c_uint64),
                ("step", C.c_uint64), ("gmax", C.c_uint32), ("pmax", C.c_uint32),
                ("ghost_count", C.c_void_p), ("ghost_pos", C.c_void_p), ("ghost_vel", C.c_void_p),
                ("axis", C.c_void_p), ("gate_u", C.c_void_p), ("gauss", C.c_void_p),
                ("collided", C.c_void_p)]


class OrcSampler(C.Structure):
    _fields_ = [("C", C.c_size_t), ("in_progress", C.c_int32), ("sample_counter", C.c_uint64),
                ("density", C.c_void_p), ("velocity", C.c_void_p), ("kahan_density", C.c_void_p),
                ("kahan_velocity", C.c_void_p), ("acc_density", C.c_void_p), ("acc_velocity", C.c_void_p),
                ("step_count", C.c_void_p), ("step_sum", C.c_void_p), ("step_mean", C.c_void_p)]


@dataclass
class Box:
    """Geometry and physics of one box; L is the container size incl. wall layers."""
    L: tuple = (10, 10, 10)
    periodic: tuple = (1, 1, 1)
    experiment: int = STANDARD
    algorithm: int = SRD
    dt: float = 0.02
    drag: float = 0.0
    thermal_velocity: float = 1.0
    n: int = 10
    cap: int | None = None

    @property
    def C(self) -> int:
        return int(self.L[0] * self.L[1] * self.L[2])

    @property
    def N_fluid(self) -> int:
        m = self.n
        for a in range(3):
            m *= self.L[a] - 2 * (1 - self.periodic[a])
        return int(m)

    def cstruct(self) -> OrcParams:
        p = OrcParams()
        p.L[:] = [int(v) for v in self.L]
        p.periodic[:] = [int(v) for v in self.periodic]
        p.experiment, p.algorithm = int(self.experiment), int(self.algorithm)
        p.dt, p.drag, p.thermal_velocity = self.dt, self.drag, self.thermal_velocity
        p.n_density = int(self.n)
        p.cap = int(self.cap if self.cap is not None else 4 * self.n)
        return p


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build_oracle()
        L = C.CDLL(path)
        L.orc_xoshiro_sequence.argtypes = [C.c_uint64, C.c_uint64, C.c_int32, C.c_size_t, C.c_void_p]
        L.orc_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.orc_gb_shift.argtypes = [C.c_uint64, C.c_uint64, f32p]
        L.orc_gb_ext_axis_table.argtypes = [f32p]
        L.orc_cell_index.argtypes = [C.POINTER(OrcParams), f32p]
        L.orc_cell_index.restype = C.c_uint32
        L.orc_storage_index.argtypes = [C.POINTER(OrcParams), C.c_uint32]
        L.orc_storage_index.restype = C.c_uint32
        L.orc_distribute.argtypes = [C.POINTER(OrcParams), f32p, f32p, u32p, C.c_size_t, C.POINTER(OrcXoshiro)]
        L.orc_translate.argtypes = [C.POINTER(OrcParams), f32p, f32p, u32p, C.c_size_t, f32p, u32p, u32p]
        for fn in (L.orc_srd_collision, L.orc_extended_collision):
            fn.argtypes = [C.POINTER(OrcParams), f32p, f32p, u32p, C.c_size_t, f32p, u32p, u32p,
                           C.POINTER(OrcDraws)]
            fn.restype = C.c_int
        L.orc_xoshiro_seed.argtypes = [C.POINTER(OrcXoshiro), C.c_uint64, C.c_uint64]
        for fn in (L.orc_sample_reference, L.orc_sample_gb):
            fn.argtypes = [C.POINTER(OrcParams), C.POINTER(OrcSampler), f32p, f32p, C.c_size_t]
        for fn in (L.orc_sample_mean_reference, L.orc_sample_mean_gb):
            fn.argtypes = [C.POINTER(OrcSampler), f32p, f32p]
        L.orc_reference_steps.argtypes = [C.POINTER(OrcParams), f32p, f32p, u32p, C.c_size_t,
                                          C.POINTER(OrcXoshiro), C.c_int32, u32p, u32p, C.c_void_p]
        L.orc_reference_steps.restype = C.c_int
        L.orc_stable_perm.argtypes = [u32p, C.c_size_t, C.c_uint32, u32p]
        L.orc_time_reference_steps.argtypes = [C.POINTER(OrcParams), C.c_uint64, C.c_int32]
        L.orc_time_reference_steps.restype = C.c_double
        L.orc_run_create.argtypes = [C.POINTER(OrcParams), C.c_uint64]
        L.orc_run_create.restype = C.c_void_p
        L.orc_run_steps.argtypes = [C.c_void_p, C.c_int32]
        L.orc_run_steps.restype = C.c_int
        L.orc_run_pressure_steps.argtypes = [C.c_void_p, C.c_int32, f64p, C.c_void_p]
        L.orc_run_pressure_steps.restype = C.c_int
        L.orc_run_particles.argtypes = [C.c_void_p]
        L.orc_run_particles.restype = C.c_size_t
        L.orc_run_destroy.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def ref():
    """The reference's own CPU code (oracle/_ref), or None where it was not built."""
    global _ref
    if _ref is None:
        path = build_oracle.build_ref() if build_oracle.reference_available() else None
        if path is None:
            path = build_oracle.REF_SO if os.path.exists(build_oracle.REF_SO) else None
        if path is None:
            return None
        R = C.CDLL(path)
        R.ref_xoshiro_sequence.argtypes = [C.c_uint64, C.c_uint64, C.c_int32, C.c_size_t, C.c_void_p]
        R.ref_distribute.argtypes = [i32p, i32p, C.c_int32, C.c_float, C.c_uint32, C.c_uint64, C.c_uint64,
                                     f32p, f32p, u32p]
        R.ref_translate.argtypes = [i32p, i32p, C.c_int32, C.c_float, f32p, C.c_uint32, f32p, f32p, u32p,
                                    u32p, C.c_uint32, u32p]
        R.ref_collision.argtypes = [C.c_int32, i32p, i32p, C.c_float, C.c_float, C.c_float, C.c_uint32, f32p,
                                    C.c_uint32, f32p, f32p, u32p, u32p, C.c_uint32, C.c_uint64, C.c_uint64,
                                    u32p]
        R.ref_backend_create.argtypes = [i32p, i32p, C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_float,
                                         C.c_uint32, C.c_uint32]
        R.ref_backend_create.restype = C.c_void_p
        R.ref_backend_destroy.argtypes = [C.c_void_p]
        R.ref_backend_seed.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64]
        R.ref_backend_set.argtypes = [C.c_void_p, f32p, f32p]
        R.ref_backend_get.argtypes = [C.c_void_p, f32p, f32p]
        R.ref_backend_step.argtypes = [C.c_void_p, C.c_int32]
        R.ref_backend_step_and_sample.argtypes = [C.c_void_p, C.c_int32]
        R.ref_backend_sample_mean.argtypes = [C.c_void_p, f32p, f32p]
        _ref = R
    return _ref


# ---------------------------------------------------------------- RNG helpers

def xoshiro_sequence(a: int, b: int, kind: int, n: int, use_ref: bool = False) -> np.ndarray:
    out = np.zeros(n * (3 if kind == 3 else 1), dtype=np.uint32 if kind == 0 else np.float32)
    L = ref() if use_ref else lib()
    fn = L.ref_xoshiro_sequence if use_ref else L.orc_xoshiro_sequence
    fn(a, b, kind, n, out.ctypes.data)
    return out.reshape(n, 3) if kind == 3 else out


def philox(ctr, key) -> np.ndarray:
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(np.asarray(ctr, dtype=np.uint32), np.asarray(key, dtype=np.uint32), out)
    return out


def gb_shift(seed: int, step: int) -> np.ndarray:
    out = np.zeros(3, dtype=np.float32)
    lib().orc_gb_shift(seed, step, out)
    return out


def ext_axis_table() -> np.ndarray:
    out = np.zeros((13, 3), dtype=np.float32)
    lib().orc_gb_ext_axis_table(out)
    return out


def xoshiro(a: int, b: int) -> OrcXoshiro:
    r = OrcXoshiro()
    lib().orc_xoshiro_seed(C.byref(r), a, b)
    return r


# ---------------------------------------------------------------- geometry

def cell_index(box: Box, pos: np.ndarray) -> np.ndarray:
    p = box.cstruct()
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    return np.array([lib().orc_cell_index(C.byref(p), pos[i].copy()) for i in range(len(pos))], dtype=np.uint32)


def storage_index(box: Box, ref_index: np.ndarray) -> np.ndarray:
    Lx, Ly, Lz = (int(v) for v in box.L)
    r = np.asarray(ref_index, dtype=np.int64)
    x, y, z = r % Lx, (r // Lx) % Ly, r // (Lx * Ly)
    return (z + Lz * (x + Lx * y)).astype(np.uint32)


def stable_perm(keys: np.ndarray, nkeys: int) -> np.ndarray:
    keys = np.ascontiguousarray(keys, dtype=np.uint32)
    perm = np.zeros(len(keys), dtype=np.uint32)
    lib().orc_stable_perm(keys, len(keys), nkeys, perm)
    return perm


# ---------------------------------------------------------------- draws tables

@dataclass
class Draws:
    """Per-cell random draws of one collision step (indexed by reference cell index)."""
    C: int
    gmax: int
    pmax: int
    ghost_count: np.ndarray = field(default=None)
    ghost_pos: np.ndarray = field(default=None)
    ghost_vel: np.ndarray = field(default=None)
    axis: np.ndarray = field(default=None)
    gate_u: np.ndarray = field(default=None)
    gauss: np.ndarray = field(default=None)
    collided: np.ndarray = field(default=None)

    @classmethod
    def empty(cls, box: Box) -> "Draws":
        cap = box.cap if box.cap is not None else 4 * box.n
        d = cls(C=box.C, gmax=box.n, pmax=cap + box.n)
        d.ghost_count = np.zeros(box.C, dtype=np.uint32)
        d.ghost_pos = np.zeros((box.C, d.gmax, 3), dtype=np.float32)
        d.ghost_vel = np.zeros((box.C, d.gmax, 3), dtype=np.float32)
        d.axis = np.zeros((box.C, 3), dtype=np.float32)
        d.gate_u = np.zeros(box.C, dtype=np.float32)
        d.gauss = np.zeros((box.C, d.pmax), dtype=np.float32)
        d.collided = np.zeros(box.C, dtype=np.uint8)
        return d

    def cstruct(self, mode: int, rng: OrcXoshiro | None = None, seed: int = 0, step: int = 0) -> OrcDraws:
        s = OrcDraws()
        s.mode = mode
        s.rng = C.pointer(rng) if rng is not None else C.POINTER(OrcXoshiro)()
        s.seed, s.step, s.gmax, s.pmax = seed, step, self.gmax, self.pmax
        for name in ("ghost_count", "ghost_pos", "ghost_vel", "axis", "gate_u", "gauss", "collided"):
            arr = getattr(self, name)
            setattr(s, name, arr.ctypes.data if arr is not None else None)
        return s


# ---------------------------------------------------------------- steps

def distribute(box: Box, N: int, a: int, b: int):
    pos = np.zeros((N, 3), dtype=np.float32)
    vel = np.zeros((N, 3), dtype=np.float32)
    cell = np.zeros(N, dtype=np.uint32)
    r = xoshiro(a, b)
    p = box.cstruct()
    lib().orc_distribute(C.byref(p), pos.reshape(-1), vel.reshape(-1), cell, N, C.byref(r))
    return pos, vel, cell


def translate(box: Box, pos: np.ndarray, vel: np.ndarray, shift):
    """Streaming + shift + cell table, in place on copies; returns (pos, vel, cell, counter, table)."""
    p = box.cstruct()
    pos = np.ascontiguousarray(pos, dtype=np.float32).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float32).copy()
    N = len(pos)
    cell = np.zeros(N, dtype=np.uint32)
    counter = np.zeros(box.C, dtype=np.uint32)
    table = np.zeros(box.C * p.cap, dtype=np.uint32)
    lib().orc_translate(C.byref(p), pos.reshape(-1), vel.reshape(-1), cell, N,
                        np.asarray(shift, dtype=np.float32), counter, table)
    return pos, vel, cell, counter, table


def collide(box: Box, pos, vel, cell, counter, table, shift, draws: Draws, mode: int,
            rng: OrcXoshiro | None = None, seed: int = 0, step: int = 0):
    p = box.cstruct()
    pos = np.ascontiguousarray(pos, dtype=np.float32).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float32).copy()
    cell = np.ascontiguousarray(cell, dtype=np.uint32).copy()
    ds = draws.cstruct(mode, rng, seed, step)
    fn = lib().orc_srd_collision if box.algorithm == SRD else lib().orc_extended_collision
    rc = fn(C.byref(p), pos.reshape(-1), vel.reshape(-1), cell, len(pos),
            np.asarray(shift, dtype=np.float32), counter, table, C.byref(ds))
    if rc:
        raise RuntimeError("oracle collision failed")
    return pos, vel, cell


class Sampler:
    def __init__(self, box: Box):
        self.box = box
        n = box.C
        self.arrays = dict(
            density=np.zeros(n, np.float32), velocity=np.zeros(3 * n, np.float32),
            kahan_density=np.zeros(n, np.float32), kahan_velocity=np.zeros(3 * n, np.float32),
            acc_density=np.zeros(n, np.float64), acc_velocity=np.zeros(3 * n, np.float64),
            step_count=np.zeros(n, np.uint32), step_sum=np.zeros(3 * n, np.int64),
            step_mean=np.zeros(3 * n, np.float32))
        self.s = OrcSampler()
        self.s.C = n
        for k, v in self.arrays.items():
            setattr(self.s, k, v.ctypes.data)

    def sample(self, pos, vel, model: str = "reference"):
        p = self.box.cstruct()
        fn = lib().orc_sample_reference if model == "reference" else lib().orc_sample_gb
        fn(C.byref(p), C.byref(self.s), np.ascontiguousarray(pos, np.float32).reshape(-1),
           np.ascontiguousarray(vel, np.float32).reshape(-1), len(pos))

    def mean(self, model: str = "reference"):
        d = np.zeros(self.box.C, np.float32)
        v = np.zeros(3 * self.box.C, np.float32)
        fn = lib().orc_sample_mean_reference if model == "reference" else lib().orc_sample_mean_gb
        fn(C.byref(self.s), d, v)
        return d, v.reshape(-1, 3)


def reference_steps(box: Box, pos, vel, rng: OrcXoshiro, nsteps: int, sampler: Sampler | None = None):
    """Restated CPUBackend::step(nsteps) on copies of (pos, vel)."""
    p = box.cstruct()
    pos = np.ascontiguousarray(pos, dtype=np.float32).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float32).copy()
    N = len(pos)
    cell = np.zeros(N, dtype=np.uint32)
    counter = np.zeros(box.C, dtype=np.uint32)
    table = np.zeros(box.C * p.cap, dtype=np.uint32)
    rc = lib().orc_reference_steps(C.byref(p), pos.reshape(-1), vel.reshape(-1), cell, N, C.byref(rng),
                                   nsteps, counter, table, C.byref(sampler.s) if sampler else None)
    if rc:
        raise RuntimeError("oracle step failed")
    return pos, vel


def time_reference_steps(box: Box, seed: int, steps: int) -> float:
    p = box.cstruct()
    return float(lib().orc_time_reference_steps(C.byref(p), seed, steps))


class Run:
    """A box advanced by the restated reference CPU step (used for the CPU baseline)."""

    def __init__(self, box: Box, seed: int):
        self._p = box.cstruct()
        self._h = lib().orc_run_create(C.byref(self._p), seed)
        if not self._h:
            raise MemoryError("oracle run allocation failed")
        self.N = int(lib().orc_run_particles(self._h))

    def steps(self, n: int) -> None:
        if lib().orc_run_steps(self._h, n):
            raise RuntimeError("oracle step failed")

    def pressure_steps(self, n: int, impulse: np.ndarray, layer_count: np.ndarray | None = None) -> None:
        """n steps, adding the outward wall impulses {bottom, top} to `impulse` and the
        particles per lab z layer to `layer_count` (float64 arrays)."""
        if lib().orc_run_pressure_steps(self._h, n, impulse,
                                        None if layer_count is None else layer_count.ctypes.data):
            raise RuntimeError("oracle step failed")

    def close(self) -> None:
        if self._h:
            lib().orc_run_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

"""ctypes front end of the C ABI in include/mpcd_gb.h (libmpcd_gb.so).

Used by the parity tests and the benchmark to call the library the way a
foreign-language binding of the reference would.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmpcd_gb.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "mpcd_gb.h")

f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")


class Params(C.Structure):
    _fields_ = [("experiment", C.c_int32), ("algorithm", C.c_int32), ("collision_kernel", C.c_int32),
                ("periodicity", C.c_int32 * 3), ("volume_size", C.c_float * 3), ("N", C.c_uint32),
                ("n", C.c_uint32), ("device_id", C.c_uint32), ("delta_t", C.c_float), ("temperature", C.c_float),
                ("thermal_velocity", C.c_float), ("drag", C.c_float), ("seed", C.c_uint64)]


_lib = None


def declared_symbols() -> list[str]:
    """Function names declared in include/mpcd_gb.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(mpcd_gb_[a-z_0-9]+)\s*\(", text)))


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not built")
        L = C.CDLL(LIB_PATH)
        H = C.c_void_p
        L.mpcd_gb_abi_version.restype = C.c_int32
        L.mpcd_gb_create.argtypes = [C.POINTER(Params), C.POINTER(H)]
        L.mpcd_gb_destroy.argtypes = [H]
        L.mpcd_gb_destroy.restype = None
        L.mpcd_gb_last_error.argtypes = [H]
        L.mpcd_gb_last_error.restype = C.c_char_p
        for name in ("mpcd_gb_step", "mpcd_gb_step_and_sample"):
            getattr(L, name).argtypes = [H, C.c_int32]
        L.mpcd_gb_get_sample_mean.argtypes = [H, f32p, f32p]
        L.mpcd_gb_num_particles.argtypes = [H]
        L.mpcd_gb_num_particles.restype = C.c_size_t
        L.mpcd_gb_num_cells.argtypes = [H]
        L.mpcd_gb_num_cells.restype = C.c_size_t
        for name in ("mpcd_gb_get_positions", "mpcd_gb_get_velocities", "mpcd_gb_set_positions",
                     "mpcd_gb_set_velocities"):
            getattr(L, name).argtypes = [H, f32p]
        L.mpcd_gb_set_particles.argtypes = [H, f32p, f32p]
        L.mpcd_gb_set_stream.argtypes = [H, C.c_void_p]
        L.mpcd_gb_synchronize.argtypes = [H]
        L.mpcd_gb_time_steps.argtypes = [H, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.mpcd_gb_step_index.argtypes = [H]
        L.mpcd_gb_step_index.restype = C.c_uint64
        L.mpcd_gb_inject_shift.argtypes = [H, C.c_uint64, f32p]
        L.mpcd_gb_get_shift.argtypes = [H, C.c_uint64, f32p]
        L.mpcd_gb_dump_layout.argtypes = [H, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.mpcd_gb_inject_draws.argtypes = [H, C.c_uint32, C.c_uint32] + [C.c_void_p] * 6
        L.mpcd_gb_counters.argtypes = [H, u64p]
        L.mpcd_gb_cell_offsets_noalloc.argtypes = [H, C.c_void_p, C.c_uint64]
        L.mpcd_gb_device_allocations.argtypes = []
        L.mpcd_gb_device_allocations.restype = C.c_uint64
        L.mpcd_gb_ensemble_create.argtypes = [C.c_void_p, C.c_int32, C.POINTER(H)]
        L.mpcd_gb_num_boxes.argtypes = [H]
        L.mpcd_gb_box_range.argtypes = [H, C.c_int32, u64p]
        L.mpcd_gb_set_particles_device.argtypes = [H, C.c_void_p, C.c_void_p]
        L.mpcd_gb_get_particles_device.argtypes = [H, C.c_void_p, C.c_void_p]
        L.mpcd_gb_set_drag.argtypes = [H, C.c_float]
        L.mpcd_gb_set_step.argtypes = [H, C.c_uint64]
        L.mpcd_gb_save_snapshot.argtypes = [H, C.c_char_p]
        L.mpcd_gb_load_snapshot.argtypes = [H, C.c_char_p]
        L.mpcd_gb_wall_pressure.argtypes = [H, C.c_int32, np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")]
        L.mpcd_gb_profile_forward.argtypes = [H, C.c_int32, C.c_int32, C.c_void_p]
        L.mpcd_gb_profile_backward.argtypes = [H, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
        L.mpcd_gb_profile_tape.argtypes = [H] + [C.c_void_p] * 5
        L.mpcd_gb_autotune.argtypes = [H, C.c_int32, np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")]
        _lib = L
    return _lib


class GbError(RuntimeError):
    pass


def device_allocations() -> int:
    """Device allocations the library has made in this process (all handles)."""
    return int(lib().mpcd_gb_device_allocations())


def make_params(L=(10, 10, 10), periodic=(1, 1, 1), n=10, dt=0.02, drag=0.0, temperature=1.0, algorithm=0,
                experiment=0, seed=0, device_id=0) -> Params:
    p = Params()
    p.experiment, p.algorithm, p.collision_kernel = experiment, algorithm, 2
    p.periodicity[:] = [int(v) for v in periodic]
    p.volume_size[:] = [float(v) for v in L]
    p.n, p.device_id = n, device_id
    p.delta_t, p.temperature, p.thermal_velocity, p.drag = dt, temperature, float(np.sqrt(temperature)), drag
    p.seed = seed
    return p


class Handle:
    """One simulation behind the C ABI."""

    def __init__(self, L=(10, 10, 10), periodic=(1, 1, 1), n=10, dt=0.02, drag=0.0, temperature=1.0,
                 algorithm=0, experiment=0, seed=0, device_id=0, boxes=None):
        """One box from the keyword arguments, or a batched ensemble from
        `boxes`, a list of dicts with the same keywords (one per box)."""
        self._lib = lib()
        if boxes is None:
            boxes = [dict(L=L, periodic=periodic, n=n, dt=dt, drag=drag, temperature=temperature,
                          algorithm=algorithm, experiment=experiment, seed=seed, device_id=device_id)]
        plist = [make_params(**b) for b in boxes]
        arr = (Params * max(1, len(plist)))(*plist)
        self.params = plist[0] if plist else None
        self.h = C.c_void_p()
        rc = self._lib.mpcd_gb_ensemble_create(C.cast(arr, C.c_void_p), len(plist), C.byref(self.h))
        if rc != 0:
            raise GbError(f"mpcd_gb_create failed ({rc}): {self._lib.mpcd_gb_last_error(None).decode()}")
        self.N = int(self._lib.mpcd_gb_num_particles(self.h))
        self.C = int(self._lib.mpcd_gb_num_cells(self.h))

    @property
    def num_boxes(self):
        return int(self._lib.mpcd_gb_num_boxes(self.h))

    def box_range(self, r):
        """(first_particle, num_particles, first_cell, num_cells) of box r."""
        out = np.zeros(4, np.uint64)
        self._check(self._lib.mpcd_gb_box_range(self.h, r, out))
        return tuple(int(v) for v in out)

    def autotune(self, steps_per_candidate=3):
        out = np.zeros(2, np.uint32)
        self._check(self._lib.mpcd_gb_autotune(self.h, steps_per_candidate, out))
        return int(out[0]), int(out[1])

    def _check(self, rc):
        if rc != 0:
            raise GbError(f"({rc}) {self._lib.mpcd_gb_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            self._lib.mpcd_gb_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1):
        self._check(self._lib.mpcd_gb_step(self.h, n))

    def step_and_sample(self, n=1):
        self._check(self._lib.mpcd_gb_step_and_sample(self.h, n))

    def sample_mean(self):
        d = np.zeros(self.C, np.float32)
        v = np.zeros(3 * self.C, np.float32)
        self._check(self._lib.mpcd_gb_get_sample_mean(self.h, d, v))
        return d, v.reshape(-1, 3)

    def positions(self):
        out = np.zeros((self.N, 3), np.float32)
        self._check(self._lib.mpcd_gb_get_positions(self.h, out.reshape(-1)))
        return out

    def velocities(self):
        out = np.zeros((self.N, 3), np.float32)
        self._check(self._lib.mpcd_gb_get_velocities(self.h, out.reshape(-1)))
        return out

    def set_particles(self, pos, vel):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
        vel = np.ascontiguousarray(vel, np.float32).reshape(-1)
        self._check(self._lib.mpcd_gb_set_particles(self.h, pos, vel))

    def set_positions(self, pos):
        self._check(self._lib.mpcd_gb_set_positions(self.h, np.ascontiguousarray(pos, np.float32).reshape(-1)))

    def set_velocities(self, vel):
        self._check(self._lib.mpcd_gb_set_velocities(self.h, np.ascontiguousarray(vel, np.float32).reshape(-1)))

    @property
    def step_index(self):
        return int(self._lib.mpcd_gb_step_index(self.h))

    def inject_shift(self, step, shift):
        self._check(self._lib.mpcd_gb_inject_shift(self.h, step, np.asarray(shift, np.float32)))

    def shift(self, step):
        out = np.zeros(3, np.float32)
        self._check(self._lib.mpcd_gb_get_shift(self.h, step, out))
        return out

    def layout(self):
        """(cell, slot, id, counts) of the current bucket layout (see mpcd_gb_dump_layout)."""
        cell = np.zeros(self.N, np.uint32)
        slot = np.zeros(self.N, np.uint32)
        pid = np.zeros(self.N, np.uint32)
        counts = np.zeros(self.C, np.uint32)
        self._check(self._lib.mpcd_gb_dump_layout(self.h, cell.ctypes.data, slot.ctypes.data, pid.ctypes.data,
                                                  counts.ctypes.data))
        return cell, slot, pid, counts

    def inject_draws(self, draws):
        """draws: oracle.Draws tables (reference cell order); None returns to Philox draws."""
        if draws is None:
            self._check(self._lib.mpcd_gb_inject_draws(self.h, 0, 0, None, None, None, None, None, None))
            return
        self._keep = [np.ascontiguousarray(getattr(draws, k)) for k in
                      ("ghost_count", "ghost_pos", "ghost_vel", "axis", "gate_u", "gauss")]
        self._check(self._lib.mpcd_gb_inject_draws(self.h, draws.gmax, draws.pmax,
                                                   *[a.ctypes.data for a in self._keep]))

    def counters(self):
        out = np.zeros(2, np.uint64)
        self._check(self._lib.mpcd_gb_counters(self.h, out))
        return int(out[0]), int(out[1])

    def cell_offsets_noalloc(self, d_offsets: int, n_offsets: int):
        """Queue the cell offsets of the current layout into the device buffer at
        address d_offsets (n_offsets uint32 entries) on the handle's stream."""
        self._check(self._lib.mpcd_gb_cell_offsets_noalloc(self.h, C.c_void_p(d_offsets), n_offsets))

    # device-pointer I/O and the differentiable profile (addresses of device buffers)
    def set_particles_device(self, d_pos, d_vel):
        self._check(self._lib.mpcd_gb_set_particles_device(self.h, C.c_void_p(d_pos or None),
                                                           C.c_void_p(d_vel or None)))

    def get_particles_device(self, d_pos, d_vel):
        self._check(self._lib.mpcd_gb_get_particles_device(self.h, C.c_void_p(d_pos or None),
                                                           C.c_void_p(d_vel or None)))

    def save_snapshot(self, path):
        self._check(self._lib.mpcd_gb_save_snapshot(self.h, str(path).encode()))

    def load_snapshot(self, path):
        self._check(self._lib.mpcd_gb_load_snapshot(self.h, str(path).encode()))

    def set_step(self, step):
        self._check(self._lib.mpcd_gb_set_step(self.h, int(step)))

    def wall_pressure(self, restart=False):
        """(bottom, top) wall pressure over the steps since the last restart, and that step count."""
        out = np.zeros(3, np.float64)
        self._check(self._lib.mpcd_gb_wall_pressure(self.h, 1 if restart else 0, out))
        return float(out[0]), float(out[1]), int(out[2])

    def set_drag(self, drag):
        self._check(self._lib.mpcd_gb_set_drag(self.h, float(drag)))

    def profile_forward(self, steps, every, d_profile):
        self._check(self._lib.mpcd_gb_profile_forward(self.h, steps, every, C.c_void_p(d_profile)))

    def profile_backward(self, d_grad_profile, d_grad_vel):
        g = C.c_double()
        self._check(self._lib.mpcd_gb_profile_backward(self.h, C.c_void_p(d_grad_profile), C.c_void_p(d_grad_vel),
                                                       C.byref(g)))
        return g.value

    def profile_tape(self, steps):
        """Fixed events of the last profile forward: (key, lab, ncell, lab_count, bounce0)."""
        key = np.zeros((steps, self.N), np.uint32)
        lab = np.zeros((steps, self.N), np.uint32)
        ncell = np.zeros((steps, self.C), np.uint32)
        cnt = np.zeros((steps, self.C), np.uint32)
        b0 = np.zeros(self.N, np.uint32)
        self._check(self._lib.mpcd_gb_profile_tape(self.h, key.ctypes.data, lab.ctypes.data, ncell.ctypes.data,
                                                   cnt.ctypes.data, b0.ctypes.data))
        return key, lab, ncell, cnt, b0

    def set_stream(self, stream_ptr):
        self._check(self._lib.mpcd_gb_set_stream(self.h, C.c_void_p(stream_ptr)))

    def synchronize(self):
        self._check(self._lib.mpcd_gb_synchronize(self.h))

    def time_steps(self, n):
        t, k = C.c_float(), C.c_float()
        self._check(self._lib.mpcd_gb_time_steps(self.h, n, C.byref(t), C.byref(k)))
        return t.value, k.value

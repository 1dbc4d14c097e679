"""Host-side logic of the C ABI, on CPU: argument checks and parameter validation
run before any CUDA call, so they are testable without a GPU.

Every entry point that takes a handle rejects a NULL one with MPCD_GB_EINVAL;
mpcd_gb_create / mpcd_gb_ensemble_create reject invalid parameters and sizes
beyond the engine's index spaces with MPCD_GB_EINVAL and a message.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

from cudampcd_gb300 import capi

EINVAL = -1

if not os.path.exists(capi.LIB_PATH):
    pytest.skip("libmpcd_gb.so not built", allow_module_level=True)


def _create(**kw):
    L = capi.lib()
    p = capi.make_params(**kw)
    h = C.c_void_p()
    rc = L.mpcd_gb_create(C.byref(p), C.byref(h))
    return rc, L.mpcd_gb_last_error(None).decode(), h


def test_abi_version_matches_header():
    text = open(capi.HEADER).read()
    version = int(re.search(r"#define\s+MPCD_GB_ABI_VERSION\s+(\d+)", text).group(1))
    assert capi.lib().mpcd_gb_abi_version() == version


@pytest.mark.parametrize("kw,message", [
    (dict(L=(10, 10, 0.5)), "volume_size"),
    (dict(L=(10.5, 10, 10)), "volume_size"),
    (dict(periodic=(1, 2, 1)), "periodicity"),
    (dict(L=(10, 10, 2), periodic=(1, 1, 0)), "walled axis"),
    (dict(n=0), "n must"),
    (dict(algorithm=3), "algorithm"),
    (dict(experiment=2), "experiment"),
    (dict(dt=0.0), "delta_t"),
    (dict(dt=float("nan")), "delta_t"),
    (dict(drag=float("inf")), "drag"),
    (dict(n=500), "n above 409"),
    (dict(L=(2048, 2048, 512), n=1), "too many cells"),
    (dict(L=(1024, 1024, 200), n=10), "slot space"),
])
def test_create_rejects_invalid_parameters_before_touching_the_device(kw, message):
    rc, err, h = _create(**kw)
    assert rc == EINVAL and message in err and not h.value


def test_ensemble_checks():
    L = capi.lib()
    h = C.c_void_p()
    arr = (capi.Params * 2)(capi.make_params(algorithm=0), capi.make_params(algorithm=1))
    assert L.mpcd_gb_ensemble_create(C.cast(arr, C.c_void_p), 2, C.byref(h)) == EINVAL
    assert "same algorithm" in L.mpcd_gb_last_error(None).decode()
    assert L.mpcd_gb_ensemble_create(C.cast(arr, C.c_void_p), 0, C.byref(h)) == EINVAL
    assert L.mpcd_gb_ensemble_create(None, 1, C.byref(h)) == EINVAL


def test_null_handle_is_rejected_everywhere():
    L = capi.lib()
    f = np.zeros(64, np.float32)
    u32 = np.zeros(64, np.uint32)
    u64 = np.zeros(4, np.uint64)
    f64 = np.zeros(3, np.float64)
    fp, up = f.ctypes.data, u32.ctypes.data
    calls = {
        "mpcd_gb_step": (1,), "mpcd_gb_step_and_sample": (1,),
        "mpcd_gb_get_sample_mean": (f, f), "mpcd_gb_get_positions": (f,), "mpcd_gb_get_velocities": (f,),
        "mpcd_gb_set_positions": (f,), "mpcd_gb_set_velocities": (f,), "mpcd_gb_set_particles": (f, f),
        "mpcd_gb_set_stream": (None,), "mpcd_gb_synchronize": (),
        "mpcd_gb_time_steps": (1, C.byref(C.c_float()), C.byref(C.c_float())),
        "mpcd_gb_inject_shift": (0, f), "mpcd_gb_get_shift": (0, f),
        "mpcd_gb_dump_layout": (up, up, up, up), "mpcd_gb_counters": (u64,),
        "mpcd_gb_save_snapshot": (b"/nonexistent",), "mpcd_gb_load_snapshot": (b"/nonexistent",),
        "mpcd_gb_box_range": (0, u64), "mpcd_gb_autotune": (1, u32),
        "mpcd_gb_set_particles_device": (fp, fp), "mpcd_gb_get_particles_device": (fp, fp),
        "mpcd_gb_set_step": (0,), "mpcd_gb_wall_pressure": (0, f64), "mpcd_gb_set_drag": (0.0,),
        "mpcd_gb_profile_forward": (1, 1, fp), "mpcd_gb_profile_backward": (fp, fp, C.byref(C.c_double())),
        "mpcd_gb_profile_tape": (up, up, up, up, up), "mpcd_gb_cell_offsets_noalloc": (up, 1),
        "mpcd_gb_inject_draws": (0, 0, None, None, None, None, None, None),
    }
    for name, args in calls.items():
        assert getattr(L, name)(None, *args) == EINVAL, name
    assert L.mpcd_gb_num_particles(None) == 0 and L.mpcd_gb_num_cells(None) == 0
    assert L.mpcd_gb_num_boxes(None) == 0 and L.mpcd_gb_step_index(None) == 0
    L.mpcd_gb_destroy(None)
    declared = set(capi.declared_symbols())
    covered = set(calls) | {"mpcd_gb_num_particles", "mpcd_gb_num_cells", "mpcd_gb_num_boxes",
                            "mpcd_gb_step_index", "mpcd_gb_destroy", "mpcd_gb_abi_version", "mpcd_gb_create",
                            "mpcd_gb_ensemble_create", "mpcd_gb_last_error", "mpcd_gb_device_allocations"}
    assert declared == covered, declared ^ covered

"""cudampcd_gb300 -- the MPCD time step of azantop/cudaMPCD, rebuilt for one GB300.

Drop-in for the reference's Python API::

    import cudampcd_gb300 as pympcd
    params = pympcd.Params()
    params.volume_size = (10, 10, 100); params.periodicity = (1, 1, 0)
    sim = pympcd.Simulation(params, "cuda")
    sim.step_and_sample(1000)
    density, velocity = sim.get_mean_fields()

``Params`` and ``Simulation`` come from the native module ``_pympcd`` (C++),
which drives the CUDA kernels of ``libmpcd_gb.so`` through the C ABI declared
in ``include/mpcd_gb.h``.  There is no CPU fallback: importing fails when the
native library has not been built (``python -c "import __graft_entry__ as g; g.build()"``).
"""
from __future__ import annotations

import os

_HERE = os.path.dirname(os.path.abspath(__file__))

try:
    from ._pympcd import Params, Simulation, __version__  # noqa: F401
except ImportError as exc:  # pragma: no cover - exercised only without a build
    raise ImportError(
        "cudampcd_gb300: native extension not built (run cudampcd_gb300/build.py or __graft_entry__.build()): "
        f"{exc}") from exc

from . import capi  # noqa: E402,F401

__all__ = ["Params", "Simulation", "capi", "__version__"]

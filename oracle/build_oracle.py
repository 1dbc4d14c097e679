"""Build recipe for the test oracle (TEST INFRASTRUCTURE ONLY).

* ``oracle/liboracle.so`` -- the C restatement in ``oracle/oracle.c``; builds on
  any machine with gcc.
* ``oracle/_ref/libmpcd_ref.so`` -- ``oracle/ref_harness.cpp`` compiled with the
  reference's own CPU sources, read where they lie in the reference tree.  Built
  only where that tree exists: ``MPCD_REFERENCE_ROOT``, else a checkout named
  ``reference`` beside this repository, else the copy that
  ``baseline/build_ref.py`` staged in ``baseline/_ref/tree``; the output stays
  out of version control.

Flags: the reference's Release build (``-O3 -DNDEBUG``, C++17) for the harness;
``-ffp-contract=off`` everywhere so that no multiply-add is fused (GCC fuses by
default on aarch64).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
_CPU_SRC = os.path.join("src", "libmpcd", "cpu_backend", "simulation_functions.cpp")


def _find_ref_root() -> str:
    env = os.environ.get("MPCD_REFERENCE_ROOT")
    if env:
        return env
    repo = os.path.dirname(HERE)
    for cand in (os.path.join(os.path.dirname(repo), "reference"), os.path.join(repo, "baseline", "_ref", "tree")):
        if os.path.isfile(os.path.join(cand, _CPU_SRC)):
            return cand
    return os.path.join(os.path.dirname(repo), "reference")


REF_ROOT = _find_ref_root()

ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmpcd_ref.so")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "oracle.h")]
    if force or _stale(ORACLE_SO, srcs):
        tmp = ORACLE_SO + ".tmp"
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
              "-Wall", "-Wextra", srcs[0], "-o", tmp, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REF_ROOT, _CPU_SRC))


def build_ref(force: bool = False) -> str | None:
    """Compile the reference CPU path with the harness; None where the tree is absent."""
    if not reference_available():
        return None
    lib = os.path.join(REF_ROOT, "src", "libmpcd")
    srcs = [os.path.join(HERE, "ref_harness.cpp"),
            os.path.join(lib, "cpu_backend", "simulation_functions.cpp"),
            os.path.join(lib, "cpu_backend", "cpu_backend.cpp")]
    if force or _stale(REF_SO, srcs):
        os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
        tmp = REF_SO + ".tmp"
        _run(["g++", "-std=c++17", "-O3", "-DNDEBUG", "-fPIC", "-shared", "-ffp-contract=off",
              "-w", "-I", lib, "-I", os.path.join(REF_ROOT, "include"), *srcs, "-o", tmp])
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))

"""Build recipe of the native parts of cudampcd_gb300 (in-tree, no cmake).

Outputs, next to this file:
  libmpcd_gb.so        CUDA kernels + host engine + the C ABI of include/mpcd_gb.h
                       (nvcc, sm_103a only; the kernels' translation unit is
                       compiled with --fmad=false so float expressions are
                       evaluated exactly as written, like the reference CPU code)
  _pympcd*.so          the Python binding (Params, Simulation) over that ABI,
                       pybind11 headers taken from the installed torch
"""
from __future__ import annotations

import os
import subprocess
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

LIB = os.path.join(PKG, "libmpcd_gb.so")
EXT_SUFFIX = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
PYMOD = os.path.join(PKG, "_pympcd" + EXT_SUFFIX)

KERNEL_SRCS = ["mpcd_kernels.cu"]
ENGINE_SRCS = ["mpcd_engine.cu"]
HEADERS = ["mpcd_types.h", "mpcd_device.cuh", "mpcd_kernels.h"]
BINDING_SRCS = ["pympcd/bindings.cpp", "pympcd/simulation_handle.cpp", "pympcd/gb_backend.cpp"]
BINDING_HDRS = ["pympcd/simulation_parameters.hpp", "pympcd/backend.hpp", "pympcd/simulation_handle.hpp",
                "pympcd/gb_backend.hpp"]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _wait(procs):
    failed = []
    for cmd, p in procs:
        out, err = p.communicate()
        if p.returncode != 0:
            failed.append(f"$ {' '.join(cmd)}\n{out}\n{err}")
    if failed:
        raise RuntimeError("build failed:\n" + "\n".join(failed))


def _start(cmd):
    return cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    include = os.path.join(ROOT, "include")
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(include, "mpcd_gb.h")]
    objs, procs = [], []
    for src, extra in [(s, ["--fmad=false"]) for s in KERNEL_SRCS] + [(s, []) for s in ENGINE_SRCS]:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + hdrs):
            cmd = [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", *extra, "-Xcompiler", "-fPIC,-O2",
                   "-I", include, "-c", path, "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            procs.append(_start(cmd))
    _wait(procs)
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _wait([_start([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"])])
        os.replace(tmp, LIB)
    return LIB


def _torch_include() -> str:
    import importlib.util

    spec = importlib.util.find_spec("torch")
    if spec is None or not spec.submodule_search_locations:
        raise RuntimeError("torch is needed for its bundled pybind11 headers")
    inc = os.path.join(list(spec.submodule_search_locations)[0], "include")
    if not os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
        raise RuntimeError(f"pybind11 headers not found under {inc}")
    return inc


def build_binding(force: bool = False) -> str:
    srcs = [os.path.join(CSRC, s) for s in BINDING_SRCS]
    deps = srcs + [os.path.join(CSRC, h) for h in BINDING_HDRS] + [LIB, os.path.join(ROOT, "include", "mpcd_gb.h")]
    if force or _stale(PYMOD, deps):
        tmp = PYMOD + ".tmp"
        cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
               "-I", _torch_include(), "-I", sysconfig.get_paths()["include"], "-I", os.path.join(ROOT, "include"),
               "-I", CSRC, *srcs, "-o", tmp, "-L", PKG, "-lmpcd_gb", "-Wl,-rpath,$ORIGIN"]
        _wait([_start(cmd)])
        os.replace(tmp, PYMOD)
    return PYMOD


def build(force: bool = False, verbose: bool = False) -> None:
    build_library(force=force, verbose=verbose)
    build_binding(force=force)


if __name__ == "__main__":
    import sys

    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
    print(PYMOD)

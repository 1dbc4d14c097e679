"""Builds of the unmodified reference (azantop/cudaMPCD) used as baselines.

Nothing here is part of the GB300 step: this recipe compiles the reference's
own sources so that the benchmark can time the reference's CUDA and CPU
backends on the same machine, and so that a test can run the reference's own
Python binding over libmpcd_gb.so.  Everything it writes goes to
``baseline/_ref/``, which version control ignores.

Steps
  stage()        copy the reference sources the builds need (include/,
                 src/libmpcd/, src/bindings/, src/pympcd/) from the reference
                 checkout -- ``MPCD_REFERENCE_ROOT``, else a checkout named
                 ``reference`` beside this repository -- into
                 ``baseline/_ref/tree``, and a second copy into
                 ``baseline/_ref/tree_dropin`` with the two changes a maintainer
                 makes to the reference: the GbBackend class
                 (``baseline/dropin/gb300_backend.hpp``, written to
                 src/libmpcd/gb300_backend/gb300_backend.hpp) and the factory
                 diff (``baseline/dropin/backend_factory.diff``, applied to
                 src/libmpcd/common/backend_factory.hpp).  Machines without the
                 checkout build from the staged copies.
  build_stock()  ``baseline/_ref/stock/pympcd``: the reference's binding,
                 SimulationHandle, CPU backend and CUDA backend, unchanged, as
                 its CMake files list them (src/libmpcd/cuda_backend/CMakeLists.txt:
                 relocatable device code, USE_CUDA, Release -O3), compiled for
                 sm_103a.  ``Simulation(params, "cuda")`` runs the reference's
                 own kernels; ``"cpu"`` its CPU backend.
  build_dropin() ``baseline/_ref/dropin/pympcd``: the reference's binding,
                 SimulationHandle and CPU backend with -DUSE_GB300=1, linked
                 against cudampcd_gb300/libmpcd_gb.so; ``Simulation(params,
                 "cuda")`` runs the GB300 step.

No CMake: the reference's CMake files name the sources and flags, and this
recipe passes the same ones to nvcc and g++ directly (pybind11 headers come
from the installed torch, as for this repository's own binding).
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
TREE = os.path.join(OUT, "tree")
TREE_DROPIN = os.path.join(OUT, "tree_dropin")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
EXT_SUFFIX = sysconfig.get_config_var("EXT_SUFFIX") or ".so"

# what the builds read from the reference checkout
STAGED = ["include", os.path.join("src", "libmpcd"), os.path.join("src", "bindings"), os.path.join("src", "pympcd")]
# src/libmpcd/cuda_backend/CMakeLists.txt (add_library(cuda_backend ...))
CUDA_SRCS = ["backend_context.cu", "collision_strategy.cu", "cuda_allocator.cu", "cuda_backend.cu",
             "cuda_backend_impl.cu", "extended_collision_strategy.cu", "gpu_arrays.cu", "simulation_kernels.cu",
             "sort_particles.cu", "srd_collision_strategy.cu"]
# src/libmpcd/cpu_backend/CMakeLists.txt, src/libmpcd/CMakeLists.txt (mpcd_backend), src/bindings/CMakeLists.txt
CPU_SRCS = [os.path.join("cpu_backend", "cpu_backend.cpp"), os.path.join("cpu_backend", "simulation_functions.cpp")]
HANDLE_SRCS = [os.path.join("api", "simulator_handle.cpp")]


def reference_root() -> str:
    return os.environ.get("MPCD_REFERENCE_ROOT") or os.path.join(os.path.dirname(ROOT), "reference")


def _checkout_present(root: str) -> bool:
    return os.path.isfile(os.path.join(root, "src", "libmpcd", "cuda_backend", "srd_collision_strategy.cu"))


def staged() -> bool:
    return _checkout_present(TREE) and _checkout_present(TREE_DROPIN)


def module_dir(kind: str) -> str:
    """Directory to put on sys.path to import that build as `pympcd`."""
    return os.path.join(OUT, kind)


def module_path(kind: str) -> str:
    return os.path.join(OUT, kind, "pympcd", "_pympcd" + EXT_SUFFIX)


# ---------------------------------------------------------------- staging

DROPIN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dropin")


def dropin_sources() -> tuple[str, str]:
    """The GbBackend class and the factory diff that turn the reference into a
    client of libmpcd_gb.so (baseline/dropin/)."""
    with open(os.path.join(DROPIN, "gb300_backend.hpp")) as f:
        cls = f.read()
    with open(os.path.join(DROPIN, "backend_factory.diff")) as f:
        diff = f.read()
    return cls, diff


def apply_unified_diff(original: str, diff: str) -> str:
    """Apply a one-file unified diff (context, '-' and '+' lines); every context
    and removed line must match, or the diff does not apply."""
    src = original.splitlines(keepends=True)
    out, pos = [], 0
    hunks = re.split(r"^@@ [^\n]*@@\n", diff, flags=re.M)[1:]
    heads = re.findall(r"^@@ -(\d+)(?:,\d+)? \+\d+(?:,\d+)? @@", diff, flags=re.M)
    if not hunks or len(hunks) != len(heads):
        raise RuntimeError("malformed diff")
    for head, body in zip(heads, hunks):
        start = int(head) - 1
        if start < pos:
            raise RuntimeError("overlapping hunks")
        out.extend(src[pos:start])
        pos = start
        for line in body.splitlines(keepends=True):
            tag, rest = (line[0], line[1:]) if line.strip("\n") else (" ", "\n")
            if tag == "+":
                out.append(rest)
            elif tag in (" ", "-"):
                if pos >= len(src) or src[pos].rstrip("\n") != rest.rstrip("\n"):
                    raise RuntimeError(f"diff does not apply at line {pos + 1}: {rest!r}")
                if tag == " ":
                    out.append(src[pos])
                pos += 1
            else:
                raise RuntimeError(f"unexpected diff line {line!r}")
    out.extend(src[pos:])
    return "".join(out)


def stage(force: bool = False) -> bool:
    """Copy the reference sources into baseline/_ref (both trees); False where
    no checkout is present (the staged copies, if any, are kept)."""
    root = reference_root()
    if not _checkout_present(root):
        return False
    cls, diff = dropin_sources()
    for tree in (TREE, TREE_DROPIN):
        if force and os.path.isdir(tree):
            shutil.rmtree(tree)
        for rel in STAGED:
            src, dst = os.path.join(root, rel), os.path.join(tree, rel)
            if os.path.isdir(src):
                shutil.copytree(src, dst, dirs_exist_ok=True)
    # the drop-in tree: the GbBackend class and the factory diff, nothing else
    lib = os.path.join(TREE_DROPIN, "src", "libmpcd")
    os.makedirs(os.path.join(lib, "gb300_backend"), exist_ok=True)
    _write_if_changed(os.path.join(lib, "gb300_backend", "gb300_backend.hpp"), cls)
    with open(os.path.join(root, "src", "libmpcd", "common", "backend_factory.hpp")) as f:
        factory = apply_unified_diff(f.read(), diff)
    _write_if_changed(os.path.join(lib, "common", "backend_factory.hpp"), factory)
    return True


def _write_if_changed(path: str, text: str) -> None:
    if os.path.exists(path):
        with open(path) as f:
            if f.read() == text:
                return
    with open(path, "w") as f:
        f.write(text)


# ---------------------------------------------------------------- builds

def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{proc.stdout[-4000:]}\n{proc.stderr[-4000:]}")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers(tree: str) -> list[str]:
    hs = []
    for base in (os.path.join(tree, "src", "libmpcd"), os.path.join(tree, "include")):
        for dp, _, fs in os.walk(base):
            hs += [os.path.join(dp, f) for f in fs if f.endswith((".hpp", ".h"))]
    return hs


def _torch_include() -> str:
    import importlib.util

    spec = importlib.util.find_spec("torch")
    if spec is None or not spec.submodule_search_locations:
        raise RuntimeError("torch is needed for its bundled pybind11 headers")
    return os.path.join(list(spec.submodule_search_locations)[0], "include")


def _compile_all(jobs: list[tuple[str, list[str], list[str]]]) -> None:
    """jobs: (object, deps, command); compiled in parallel where stale."""
    todo = [cmd for obj, deps, cmd in jobs if _stale(obj, deps)]
    with ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, c) for c in todo]:
            f.result()


def _package(kind: str, tree: str, objs: list[str], link: list[str], linker: list[str]) -> str:
    target = module_path(kind)
    os.makedirs(os.path.dirname(target), exist_ok=True)
    shutil.copyfile(os.path.join(tree, "src", "pympcd", "__init__.py"),
                    os.path.join(os.path.dirname(target), "__init__.py"))
    if _stale(target, objs):
        tmp = target + ".tmp"
        _run([*linker, "-o", tmp, *objs, *link])
        os.replace(tmp, target)
    return target


def _cxx_flags(tree: str) -> list[str]:
    return ["-std=c++17", "-O3", "-DNDEBUG", "-fPIC", "-w", "-I", os.path.join(tree, "src", "libmpcd"),
            "-I", os.path.join(tree, "include")]


def _binding_jobs(tree: str, obj_dir: str, defines: list[str], extra_inc: list[str]) -> list:
    py_inc = ["-I", _torch_include(), "-I", sysconfig.get_paths()["include"]]
    hdrs = _headers(tree)
    jobs = []
    lib = os.path.join(tree, "src", "libmpcd")
    for rel in [os.path.join("..", "bindings", "bindings.cpp")] + HANDLE_SRCS + CPU_SRCS:
        src = os.path.normpath(os.path.join(lib, rel))
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        jobs.append((obj, [src] + hdrs,
                     ["g++", *_cxx_flags(tree), *defines, *extra_inc, *py_inc, "-fvisibility=hidden", "-c", src,
                      "-o", obj]))
    return jobs


def build_stock() -> str:
    """The reference unchanged, with its CUDA backend, as a `pympcd` module."""
    if not staged():
        raise RuntimeError("reference sources are not staged (baseline/_ref/tree)")
    obj_dir = os.path.join(OUT, "obj_stock")
    os.makedirs(obj_dir, exist_ok=True)
    defines = ["-DUSE_CUDA=1"]
    jobs = _binding_jobs(TREE, obj_dir, defines, [])
    hdrs = _headers(TREE)
    cuda_dir = os.path.join(TREE, "src", "libmpcd", "cuda_backend")
    for s in CUDA_SRCS:
        src = os.path.join(cuda_dir, s)
        obj = os.path.join(obj_dir, s + ".o")
        jobs.append((obj, [src] + hdrs,
                     [NVCC, *ARCH, "-rdc=true", "-O3", "-DNDEBUG", "-std=c++17", *defines, "-w",
                      "-Xcompiler", "-fPIC", "-I", os.path.join(TREE, "src", "libmpcd"),
                      "-I", os.path.join(TREE, "include"), "-c", src, "-o", obj]))
    _compile_all(jobs)
    objs = [j[0] for j in jobs]
    return _package("stock", TREE, objs, ["-Xcompiler", "-fPIC"], [NVCC, *ARCH, "-shared", "-rdc=true"])


def build_dropin() -> str:
    """The reference's binding and SimulationHandle over libmpcd_gb.so (baseline/dropin/)."""
    if not staged():
        raise RuntimeError("reference sources are not staged (baseline/_ref/tree_dropin)")
    gb_lib = os.path.join(ROOT, "cudampcd_gb300", "libmpcd_gb.so")
    if not os.path.exists(gb_lib):
        raise RuntimeError("libmpcd_gb.so is not built")
    obj_dir = os.path.join(OUT, "obj_dropin")
    os.makedirs(obj_dir, exist_ok=True)
    jobs = _binding_jobs(TREE_DROPIN, obj_dir, ["-DUSE_GB300=1"], ["-I", os.path.join(ROOT, "include")])
    for j in jobs:
        j[1].append(os.path.join(ROOT, "include", "mpcd_gb.h"))
    _compile_all(jobs)
    objs = [j[0] for j in jobs]
    target = module_path("dropin")
    rpath = os.path.relpath(os.path.dirname(gb_lib), os.path.dirname(target))
    return _package("dropin", TREE_DROPIN, objs + [gb_lib],
                    ["-L", os.path.dirname(gb_lib), "-lmpcd_gb", f"-Wl,-rpath,$ORIGIN/{rpath}"],
                    ["g++", "-shared", "-fPIC"])


def build(force: bool = False) -> dict:
    """Stage (where the checkout is) and build both modules (where the sources
    are staged).  Returns the built module paths by kind."""
    stage(force=force)
    if not staged():
        return {}
    if force:
        for d in ("obj_stock", "obj_dropin", "stock", "dropin"):
            p = os.path.join(OUT, d)
            if os.path.isdir(p):
                shutil.rmtree(p)
    with ThreadPoolExecutor(max_workers=2) as ex:
        fs = {"stock": ex.submit(build_stock), "dropin": ex.submit(build_dropin)}
        return {k: f.result() for k, f in fs.items()}


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

"""Benchmark of the MPCD step on GB300: particle-steps/s and the HBM roofline.

Workload (default, one GPU): SRD Poiseuille channel, 1000 x 1000 x 20 fluid cells
plus two wall layers in z, n = 20 particles per cell (N = 4.0e8), T = 1,
g = 0.001, dt = 0.02, alpha = 120 deg, Philox seed 0; W warm-up steps, then K
timed steps.  Synthetic data (random initial state), as in the reference's own
benchmark (benchmark.py:36-47).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Batched ensemble: --ensemble R runs R independent channel replicas drawn from a
seeded generator (Lx, Ly in {8, 16, 32, 64}, Lz uniform in [20, 200] incl. walls,
n in {5, 10, 20}, drag log-uniform in [1e-4, 1e-2], T = 1, dt = 0.02, seed
base + r) in one handle -- one step-kernel launch per step, CUDA-graph replays,
autotuned tiles -- and the same replicas stepped one handle at a time, and
prints one line with both rates.

Physics: --physics extended runs the extended-MPC channel with the non-ideal
equation of state (256 x 256 x 64 cells + 2 walls, n = 20, T = 1, dt = 0.02,
g = 0.0005): warm-up, then the wall pressure, the density profile and the
viscosity from the curvature of the sampled velocity profile.  --physics srd
runs the same measurement with the SRD collision.  --eta-guess E starts the
flow from the steady Poiseuille profile of viscosity E (the warm-up then only
has to relax the guess's error).  --physics viscosity runs the SRD viscosity
channel of the reference's own check (10 x 10 x 100 cells + 2 walls, n = 10,
g = 0.001, dt = 0.02) as 16 replicas in one handle, with the reference's protocol
(1000 warm-up steps, 100000 sampled) and with a warm-up of five relaxation times
(67500 steps), each read with the reference's estimator (README.md:94-96:
L^2 n g / (8 max u)) and with the curvature fit.

Profiling options (the default run uses none of them): --size LX LY LZ replaces
the fluid cells of the workload (walls are added in z), --algorithm extended
switches the collision, --no-e2e, --no-cpu and --no-adjoint skip those parts.

Adjoint: --adjoint times the differentiable channel (64 x 64 x 32 cells + 2 walls,
n = 10, 200 steps, checkpoints every 20): a plain step, the sampled forward with
checkpoints, and the adjoint (backward) per step, and their ratios.  The default
line carries the same figures in its `adjoint` block.

One JSON line on rank 0.  `value` is device-timed particle-steps/s with the
state resident in HBM; `e2e` is the same metric through the Python API the
reference exposes (Simulation.step_and_sample + get_mean_fields, host wall
clock, results read back to the host).  The default line also carries
`reference_gpu`: the reference's own CUDA backend ("optimized" kernel, built
unchanged by baseline/build_ref.py) timed on the same GPU in a child process
before this repository's arm runs.

Reference arms:
  --impl reference       the reference's own CPU backend (pympcd.Simulation(params,
                         "cpu") of the unchanged build), one process per host core,
                         each on a bounded slab of the workload; where that build is
                         absent, the oracle's restatement of the same step.
  --impl reference-cuda  the reference's own CUDA backend through
                         pympcd.Simulation(params, "cuda"): --kernel optimized |
                         sorting | trivial, --algorithm, --size as for this arm.
Several GPUs run independent replicas (the step has no exchange).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MPCD particle-steps/sec on 1 GB300, % HBM peak; batched & adjoint vs plain"
UNIT = "particle-steps/s"
WORKLOAD = dict(L=(1000, 1000, 22), periodic=(1, 1, 0), n=20, dt=0.02, drag=0.001, temperature=1.0, seed=0)
WORKLOAD_NAME = ("SRD Poiseuille channel 1000x1000x20 cells (+2 wall layers in z), n=20, N=4.0e8, T=1, "
                 "g=0.001, dt=0.02, alpha=120deg, Philox seed 0")
# Published reference number for this workload: 94 ms/step on an Ampere GPU
# ("optimized" kernel, README.md:41) = 4.0e8 / 0.094 s.
REFERENCE_PUBLISHED = 4.0e8 / 0.094
ALGO_BYTES_PER_PARTICLE = 48.0   # read + write FP32 position and velocity once per step
CPU_SLAB = dict(L=(1000, 2, 22), periodic=(1, 1, 0), n=20, dt=0.02, drag=0.001)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def ncu_traffic_per_particle():
    """DRAM bytes per particle of the step kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "srd_run_kernel_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_particle"]), d.get("source", path)
    except Exception:
        return None, None


# ---------------------------------------------------------------- ranks

def reduce_max(x: float, dist=None, device: str = "cuda") -> float:
    """x maximised over the ranks of the process group (the slowest rank's time);
    x itself without a process group."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, particles_per_rank: int, steps: int, elapsed_s: float) -> float:
    """Particle-steps/s of the whole job: every rank advances its own replica."""
    return world * particles_per_rank * steps / elapsed_s


# ---------------------------------------------------------------- CPU (oracle) timing

def cpu_rate(threads: int, warmup: int, steps: int):
    """Aggregate particle-steps/s of `threads` independent slabs advanced by the
    restated reference step; returns (rate, particles per thread, kind)."""
    import oracle as O

    box = O.Box(L=CPU_SLAB["L"], periodic=CPU_SLAB["periodic"], n=CPU_SLAB["n"], dt=CPU_SLAB["dt"],
                drag=CPU_SLAB["drag"])
    runs = [O.Run(box, 1000 + t) for t in range(threads)]
    barrier = threading.Barrier(threads + 1)
    times = [0.0] * threads

    def work(t):
        runs[t].steps(warmup)
        barrier.wait()
        t0 = time.perf_counter()
        runs[t].steps(steps)
        times[t] = time.perf_counter() - t0
        barrier.wait()

    ths = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    for th in ths:
        th.start()
    barrier.wait()
    barrier.wait()
    for th in ths:
        th.join()
    n = runs[0].N
    for r in runs:
        r.close()
    return threads * n * steps / max(times), n


def _ref_module_dir(kind: str):
    """sys.path entry of the reference build `kind` ("stock" or "dropin"), or None."""
    from baseline import build_ref

    return build_ref.module_dir(kind) if os.path.exists(build_ref.module_path(kind)) else None


def _ref_cpu_worker(mod_dir, slab, warmup, steps, barrier, out, i):
    """One host core: the reference's CPU backend on one slab (spawned process)."""
    sys.path.insert(0, mod_dir)
    import pympcd

    p = pympcd.Params()
    p.n = slab["n"]
    p.periodicity = slab["periodic"]
    p.volume_size = (slab["L"][0], slab["L"][1], slab["L"][2] - 2)
    p.drag = slab["drag"]
    p.delta_t = slab["dt"]
    p.temperature = 1.0
    sim = pympcd.Simulation(p, "cpu")
    sim.step(warmup)
    barrier.wait()
    t0 = time.perf_counter()
    sim.step(steps)
    out[i] = time.perf_counter() - t0
    out[len(out) // 2 + i] = len(sim.get_particle_positions())
    barrier.wait()


def reference_cpu_rate(procs: int, warmup: int, steps: int):
    """Aggregate particle-steps/s of the reference's own CPU backend: `procs`
    processes (the backend is single-threaded), each advancing one slab of the
    workload; None where the reference build is absent."""
    mod_dir = _ref_module_dir("stock")
    if mod_dir is None:
        return None
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(procs + 1)
    out = ctx.Array("d", 2 * procs)
    ps = [ctx.Process(target=_ref_cpu_worker, args=(mod_dir, CPU_SLAB, warmup, steps, barrier, out, i))
          for i in range(procs)]
    for p in ps:
        p.start()
    barrier.wait(timeout=600)
    barrier.wait(timeout=1800)
    for p in ps:
        p.join()
    if any(p.exitcode != 0 for p in ps):
        raise RuntimeError("a reference CPU worker failed")
    times, counts = list(out[:procs]), list(out[procs:])
    return sum(counts) * steps / max(times), int(counts[0])


def cpu_model() -> str:
    try:
        import platform

        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return f"{platform.machine()} {line.split(':', 1)[1].strip()}"
        return platform.machine()
    except Exception:
        return "unknown"


def cpu_baseline_block(warmup: int, steps: int):
    """cpu_baseline of a line: the reference's CPU backend on every host core,
    else the oracle's restatement on host threads."""
    cores = os.cpu_count() or 1
    slab = (f"{CPU_SLAB['L'][0]}x{CPU_SLAB['L'][1]}x{CPU_SLAB['L'][2] - 2} cells + walls, "
            f"n={CPU_SLAB['n']}")
    r = reference_cpu_rate(cores, warmup, steps)
    if r is not None:
        rate, n = r
        single = reference_cpu_rate(1, warmup, steps)   # the same slab in one process, alone on the host
        return {"value": rate, "unit": UNIT, "cores": cores, "kind": "reference", "cpu": cpu_model(),
                "sample": f"{cores} processes (one per core; the reference CPU backend is single-threaded), "
                          f"each one slab of the workload, {slab} ({n} particles), pympcd.Simulation(params, "
                          f"'cpu') of the unchanged reference build; {warmup} warm-up + {steps} timed steps",
                "single_core": {"value": single[0] if single else None, "unit": UNIT, "cores": 1}}
    threads = min(cores, 16)
    rate, n = cpu_rate(threads, warmup, steps)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "cpu": cpu_model(),
            "sample": f"{threads} threads x one slab, {slab} ({n} particles), the oracle's restatement of "
                      f"the reference CPU step (reference build absent); {warmup} warm-up + {steps} timed steps"}


def run_reference_arm(args, rank):
    if rank != 0:
        return
    cb = cpu_baseline_block(min(args.warmup, 3), min(args.steps, 20))
    rate = cb["value"]
    out = {"metric": METRIC, "value": rate, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": min(args.steps, 20), "warmup": min(args.warmup, 3),
           "ms_per_step": 4.0e8 / rate * 1e3,   # the whole workload's step at this aggregate rate
           "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": WORKLOAD_NAME, "sample": "one slab of the same workload per host core"},
           "cpu_baseline": cb,
           "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def reference_cuda_workload(args):
    algorithm = args.algorithm
    L = tuple(args.size) if args.size else (1000, 1000, 20)
    if algorithm == "extended" and not args.size:
        L = (256, 256, 64)
    n = 20
    drag = 0.0005 if algorithm == "extended" else 0.001
    return dict(L=L, n=n, drag=drag, dt=0.02, algorithm=algorithm)


def run_reference_cuda(args, rank, local_rank):
    """The reference's own CUDA backend on this GPU, through its unchanged Python
    API; host wall clock around step(K) + device synchronisation, as the
    reference's benchmark.py:53-66 times it, and CUDA events on the default stream
    the reference launches on."""
    if rank != 0:
        return
    mod_dir = _ref_module_dir("stock")
    wl = reference_cuda_workload(args)
    name = (f"reference {args.kernel} {wl['algorithm'].upper()} channel {wl['L'][0]}x{wl['L'][1]}x{wl['L'][2]} "
            f"cells (+2 wall layers in z), n={wl['n']}, T=1, g={wl['drag']}, dt={wl['dt']}")
    if mod_dir is None:
        print(json.dumps({"impl": "reference-cuda", "unavailable": "the reference build (baseline/_ref) is absent"}))
        return
    import torch

    sys.path.insert(0, mod_dir)
    import pympcd

    torch.cuda.set_device(local_rank)
    p = pympcd.Params()
    p.n = wl["n"]
    p.temperature = 1.0
    p.periodicity = (1, 1, 0)
    p.volume_size = wl["L"]
    p.drag = wl["drag"]
    p.delta_t = wl["dt"]
    p.algorithm = wl["algorithm"]
    p.collision_kernel = args.kernel
    p.device_id = local_rank
    if args.physics in ("srd", "extended"):
        run_reference_physics(args, p, pympcd, torch)
        return
    t0 = time.perf_counter()
    sim = pympcd.Simulation(p, "cuda")
    torch.cuda.synchronize()
    t_init = time.perf_counter() - t0
    N = len(sim.get_particle_positions())
    sim.step(args.warmup)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        t0 = time.perf_counter()
        start.record()
        sim.step(args.steps)
        stop.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    ev_ms = start.elapsed_time(stop)
    del sim
    out = {"metric": METRIC, "value": N * args.steps / wall, "unit": UNIT, "impl": "reference-cuda",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
           "event_ms_per_step": ev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": name, "kernel": args.kernel, "particles": N,
                      "particles_note": "the reference allocates n x container cells (wall layers included) "
                                        "and places them all in the fluid (backend_context.cu:19)",
                      "build": "unchanged reference sources, nvcc sm_103a, -O3 (baseline/build_ref.py)",
                      "init_s": t_init,
                      "timing": "host wall clock around step(K) + synchronize (benchmark.py:53-66)"},
           "clocks": clocks.summary()}
    print(json.dumps(out), flush=True)


def run_reference_physics(args, p, pympcd, torch):
    """The reference's own CUDA backend on the physics workload: warm-up, then 8
    blocks of step_and_sample + get_mean_fields (the reference divides the sums by
    S - 1, corrected here); viscosity from the curvature of each block's profile
    and the density profile, the estimators run_physics applies to this backend.
    The reference fills the fluid at n (Lz + 2) / Lz particles per cell
    (backend_context.cu:19): with n = 16 and Lz = 32 that is 17, the density of this
    backend's n = 17 run."""
    import numpy as np

    Lx, Ly, Lz = args.size or (256, 256, 32)
    n, g, dt = args.n or 16, 0.0005, 0.02
    p.n = n
    p.volume_size = (Lx, Ly, Lz)
    p.drag = g
    p.algorithm = args.physics
    sim = pympcd.Simulation(p, "cuda")
    N = len(sim.get_particle_positions())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.step(args.warmup)
    torch.cuda.synchronize()
    t_warm = time.perf_counter() - t0
    blocks, per = 8, max(2, args.steps // 8)
    zc = np.arange(Lz + 2) + 0.5 - (Lz + 2) / 2.0
    fluid = slice(1, Lz + 1)
    A = np.stack([np.ones(Lz), -(zc[fluid] ** 2 + 1.0 / 12.0)], axis=1)
    rho = N / (Lx * Ly * Lz)
    etas, dens = [], np.zeros(Lz + 2)
    for _ in range(blocks):
        sim.step_and_sample(per)
        d, v = sim.get_mean_fields()   # (x, y, z) and (x, y, z, 3)
        u = np.asarray(v)[:, :, :, 0].mean(axis=(0, 1)) * (per - 1) / per
        dens += np.asarray(d).mean(axis=(0, 1)) * (per - 1) / per / blocks
        (a0, b0), *_ = np.linalg.lstsq(A, u[fluid], rcond=None)
        etas.append(rho * g / (2.0 * b0))
    etas = np.array(etas)
    out = {"physics": args.physics, "impl": "reference-cuda", "kernel": args.kernel,
           "workload": f"reference {args.physics} channel {Lx}x{Ly}x{Lz} cells + 2 walls, params.n={n} "
                       f"(fluid density {rho:g}), T=1, dt={dt}, g={g}, N={N}",
           "fluid_density": rho, "warmup_steps": args.warmup, "sampled_steps": blocks * per, "warmup_s": t_warm,
           "ms_per_step_warmup": 1e3 * t_warm / max(1, args.warmup),
           "viscosity": {"mean": float(etas.mean()), "stderr": float(etas.std(ddof=1) / np.sqrt(blocks)),
                         "blocks": [float(e) for e in etas]},
           "density_profile_fluid": {"mean": float(dens[fluid].mean()), "min": float(dens[fluid].min()),
                                     "max": float(dens[fluid].max()), "first_layers": [float(x) for x in dens[1:5]],
                                     "layers": [float(x) for x in dens]},
           "velocity_profile": [float(x) for x in u],
           "wall_pressure": None,
           "wall_pressure_note": "the reference has no pressure measurement and its state between steps does not "
                                 "carry the bounce-back and collision momentum the estimator sums"}
    print(json.dumps(out), flush=True)


def reference_gpu_block(args, local_rank):
    """The reference's optimized CUDA kernel on the same workload, run in a child
    process (its memory is released, and a failure there cannot take this
    process's context with it); None when unavailable."""
    if _ref_module_dir("stock") is None:
        return {"unavailable": "the reference build (baseline/_ref) is absent"}
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference-cuda", "--kernel", "optimized",
           "--steps", str(args.steps), "--warmup", str(args.warmup)]
    if args.size:
        cmd += ["--size", *map(str, args.size)]
    env = dict(os.environ, LOCAL_RANK=str(local_rank), RANK="0", WORLD_SIZE="1")
    try:
        proc = subprocess.run(cmd, capture_output=True, text=True, timeout=1200, env=env)
    except subprocess.TimeoutExpired:
        return {"unavailable": "the reference arm did not finish within 1200 s"}
    lines = [l for l in proc.stdout.splitlines() if l.startswith("{")]
    if proc.returncode != 0 or not lines:
        return {"unavailable": f"the reference arm failed (rc {proc.returncode}): {proc.stderr.strip()[-300:]}"}
    r = json.loads(lines[-1])
    if "unavailable" in r:
        return r
    return {"kernel": "optimized", "value": r["value"], "unit": UNIT, "ms_per_step": r["ms_per_step"],
            "event_ms_per_step": r["event_ms_per_step"], "particles": r["config"]["particles"],
            "steps": r["steps"], "warmup": r["warmup"], "clocks": r["clocks"],
            "how": "pympcd.Simulation(params, 'cuda') of the unchanged reference build, same GPU, child process"}


# ---------------------------------------------------------------- GPU arm

def run_e2e(args, wl, algorithm, rank, local_rank, dist, world, N):
    """Same metric through the Python API the reference exposes: a fresh
    Simulation, step_and_sample over the timed steps and get_mean_fields (the
    device-to-host read of the result), host wall clock."""
    import cudampcd_gb300 as pympcd

    params = pympcd.Params()
    params.n = wl["n"]
    params.temperature = wl["temperature"]
    params.volume_size = (wl["L"][0], wl["L"][1], wl["L"][2] - 2)
    params.periodicity = wl["periodic"]
    params.drag = wl["drag"]
    params.delta_t = wl["dt"]
    params.algorithm = "extended" if algorithm else "srd"
    params.device_id = local_rank
    params.seed = wl["seed"] + rank
    sim = pympcd.Simulation(params, "cuda")
    sim.step_and_sample(min(args.warmup, 5))
    sim.get_mean_fields()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    sim.step_and_sample(args.steps)
    density, velocity = sim.get_mean_fields()
    e2e_s = reduce_max(time.perf_counter() - t0, dist)
    del sim
    e2e_value = whole_job_rate(world, N, args.steps, e2e_s)
    d2h = (density.nbytes + velocity.nbytes) / args.steps
    return {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": d2h,
            "api": "cudampcd_gb300.Simulation.step_and_sample + get_mean_fields (host wall clock)"}


def device_memory(handle_bytes: int, n: int, cells: int, particles: int) -> dict:
    """Device memory of one handle: measured (free memory before creation minus
    after the warm-up steps) and the two bucket sets' share: cells x depth slots of
    32 B, depth = min(4n, n + ceil(4 sqrt(n)) + 2), plus the extension area
    (min(N, 2^22) slots, at least 4n)."""
    depth = min(4 * n, n + math.ceil(4 * math.sqrt(n)) + 2)
    ext = max(4 * n, min(particles, 1 << 22))
    return {"handle_gb": handle_bytes / 1e9, "bucket_depth": depth, "bucket_depth_reference": 4 * n,
            "buckets_gb": 2 * 32 * (cells * depth + ext) / 1e9,
            "buckets_gb_at_reference_depth": 2 * 32 * cells * 4 * n / 1e9}


def run_gpu_arm(args, rank, world, local_rank):
    import torch

    from cudampcd_gb300 import capi

    # the reference's own CUDA kernel on the same GPU, first, in a child process
    ref_gpu = None
    if world == 1 and not args.no_reference_gpu:
        ref_gpu = reference_gpu_block(args, local_rank)

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    wl = dict(WORKLOAD)
    workload_name = WORKLOAD_NAME
    algorithm = 1 if args.algorithm == "extended" else 0
    if args.size or algorithm:
        if args.size:
            wl["L"] = (args.size[0], args.size[1], args.size[2] + 2)
        workload_name = (f"{args.algorithm.upper()} Poiseuille channel {wl['L'][0]}x{wl['L'][1]}x{wl['L'][2] - 2} "
                         f"cells (+2 wall layers in z), n={wl['n']}, T=1, g=0.001, dt=0.02, Philox seed 0")
    free_before = torch.cuda.mem_get_info(local_rank)[0]
    h = capi.Handle(L=wl["L"], periodic=wl["periodic"], n=wl["n"], dt=wl["dt"], drag=wl["drag"],
                    temperature=wl["temperature"], algorithm=algorithm, seed=wl["seed"] + rank,
                    device_id=local_rank)
    N, C = h.N, h.C
    h.step(args.warmup)
    h.synchronize()
    memory = device_memory(free_before - torch.cuda.mem_get_info(local_rank)[0], wl["n"], C, N)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        total_ms, kernel_ms = h.time_steps(args.steps)
    torch.cuda.synchronize()
    overflowed, flags = h.counters()
    h.close()
    elapsed = reduce_max(total_ms, dist)
    value = whole_job_rate(world, N, args.steps, elapsed * 1e-3)

    # end to end through the Python API: step_and_sample + get_mean_fields
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, wl, algorithm, rank, local_rank, dist, world, N)

    if rank == 0:
        peak, peak_kind = peaks()
        per_launch_ms = kernel_ms / args.steps
        achieved = ALGO_BYTES_PER_PARTICLE * N / (per_launch_ms * 1e-3) / 1e9
        bpp, src = ncu_traffic_per_particle() if algorithm == 0 else (None, None)
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": value / (world * REFERENCE_PUBLISHED), "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": workload_name, "particles_per_gpu": N, "cells_per_gpu": C,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": f"inputs larger than L2: {64 * N / 1e9:.1f} GB of particle state read and written per step",
                       "vs_baseline_ref": "reference README.md:41, 94 ms/step on an Ampere GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": bpp * N if bpp else None, "traffic_source": src,
                         "algorithmic_bytes_per_particle": ALGO_BYTES_PER_PARTICLE,
                         "kernel": "srd_run_kernel" if algorithm == 0 else "step_kernel<EXTENDED, Philox>",
                         "kernel_ms": per_launch_ms},
            "e2e": e2e,
            "clocks": clocks.summary(),
            "gpu_launches": 2 * args.steps,   # per step: overflow selection, step kernel
            "device_counters": {"bucket_overflows": overflowed, "error_flags": flags},
            "device_memory": memory,
        }
        if ref_gpu is not None:
            if "value" in ref_gpu:
                ref_gpu["speedup_ms_per_step"] = ref_gpu["ms_per_step"] / out["ms_per_step"]
                ref_gpu["speedup_particle_steps"] = value / ref_gpu["value"]
            out["reference_gpu"] = ref_gpu
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline_block(1, args.steps_cpu)
        if world == 1 and not args.no_adjoint:
            out["adjoint"] = adjoint_block(5)   # the adjoint's cost against a plain step (config 5)
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def ensemble_boxes(R: int, seed: int = 0, small: bool = False):
    """The replicas of the batched workload (numpy default_rng(seed)); `small`:
    Lx, Ly in {8, 16}, Lz in [20, 60], n in {5, 10} instead."""
    import numpy as np

    rng = np.random.default_rng(seed)
    boxes = []
    for r in range(R):
        lx, ly = (int(v) for v in rng.choice([8, 16] if small else [8, 16, 32, 64], size=2))
        lz = int(rng.integers(20, 61 if small else 201))
        n = int(rng.choice([5, 10] if small else [5, 10, 20]))
        drag = float(10 ** rng.uniform(-4, -2))
        boxes.append(dict(L=(lx, ly, lz), periodic=(1, 1, 0), n=n, dt=0.02, drag=drag, temperature=1.0,
                          seed=1000 + r))
    return boxes


def run_ensemble(args):
    import torch

    from cudampcd_gb300 import capi

    boxes = ensemble_boxes(args.ensemble, small=args.small_replicas)
    K = args.steps
    h = capi.Handle(boxes=boxes)
    N = h.N
    tile_cells, pbuf = h.autotune(2)
    h.step(max(args.warmup, 6))
    h.synchronize()
    with ClockSampler(0) as clocks:
        t0 = time.perf_counter()
        h.step(K)
        h.synchronize()
        t_batched = time.perf_counter() - t0
    flags = h.counters()[1]
    h.close()
    torch.cuda.synchronize()
    t_seq = 0.0
    for b in boxes:   # the same replicas through the plain single-box path, one after the other
        s = capi.Handle(**b)
        s.step(6)
        s.synchronize()
        t0 = time.perf_counter()
        s.step(K)
        s.synchronize()
        t_seq += time.perf_counter() - t0
        s.close()
    batched, sequential = N * K / t_batched, N * K / t_seq
    out = {"metric": METRIC, "value": batched, "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": args.warmup,
           "ms_per_step": 1e3 * t_batched / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"batched SRD ensemble: {len(boxes)} channel replicas, N = {N}, " +
                                  ("Lx,Ly in {8,16}, Lz in [20,60], n in {5,10}" if args.small_replicas else
                                   "Lx,Ly in {8,16,32,64}, Lz in [20,200], n in {5,10,20}") +
                                  ", drag log-uniform [1e-4,1e-2], T=1, dt=0.02, seeds 1000+r (numpy default_rng(0))",
                      "tiles": {"cells_per_tile": tile_cells, "particle_buffer": pbuf},
                      "timing": "host wall clock around step(K) + synchronize, both arms"},
           "batched_vs_sequential": {"batched": batched, "sequential": sequential, "speedup": batched / sequential},
           "clocks": clocks.summary(), "device_counters": {"error_flags": flags}}
    print(json.dumps(out), flush=True)


def run_ensemble_viscosity(args):
    """Per-replica SRD viscosity of the batched workload's replicas, as one batched
    handle.  The replicas are those of ensemble_boxes(R) whose fluid height is at most
    --max-height (the slowest mode of a taller channel relaxes over more steps than a
    bounded run takes).  Each starts from the Poiseuille profile of 0.9 x the analytic
    viscosity, so that a measurement pulled towards its start would read low; after
    the warm-up, 4 sampled blocks give each replica's viscosity from the curvature of
    its profile, with the spread of the blocks as its error.  A replica counts as
    relaxed when the warm-up is at least 3 of its slowest relaxation times
    L^2 n / (pi^2 eta dt) steps (the start's 10 % error is then below 0.5 %)."""
    import math

    import numpy as np

    from cudampcd_gb300 import capi

    boxes = [b for b in ensemble_boxes(args.ensemble) if b["L"][2] - 2 <= args.max_height]
    h = capi.Handle(boxes=boxes)
    alpha = 2 * math.pi / 3
    theory = [(1 - math.cos(alpha)) / (18 * b["dt"]) * (b["n"] - 1 + math.exp(-b["n"])) for b in boxes]
    pos, vel = h.positions(), h.velocities()
    ranges = [h.box_range(r) for r in range(len(boxes))]
    for b, eta, (p0, nr, _, _) in zip(boxes, theory, ranges):
        hz = (b["L"][2] - 2) / 2.0
        z = pos[p0:p0 + nr, 2].astype(np.float64)
        vel[p0:p0 + nr, 0] += (b["n"] * b["drag"] * (hz * hz - z * z) / (2.0 * 0.9 * eta)).astype(np.float32)
    h.set_velocities(vel)
    del pos, vel
    t0 = time.perf_counter()
    h.step(args.warmup)
    blocks, per = 4, max(2, args.steps // 4)
    etas = np.zeros((blocks, len(boxes)))
    for k in range(blocks):
        h.step_and_sample(per)
        _, v = h.sample_mean()
        for r, (b, (_, _, c0, cr)) in enumerate(zip(boxes, ranges)):
            Lx, Ly, Lz = b["L"]
            u = v[c0:c0 + cr, 0].reshape(Lz, Ly, Lx).mean(axis=(1, 2)).astype(np.float64) * (per - 1) / per
            zc = np.arange(Lz) + 0.5 - Lz / 2.0
            A = np.stack([np.ones(Lz - 2), -(zc[1:-1] ** 2 + 1.0 / 12.0)], axis=1)
            (_, curv), *_ = np.linalg.lstsq(A, u[1:-1], rcond=None)
            etas[k, r] = b["n"] * b["drag"] / (2.0 * curv)
    elapsed = time.perf_counter() - t0
    flags = h.counters()[1]
    h.close()
    eta, err = etas.mean(axis=0), etas.std(axis=0, ddof=1) / np.sqrt(blocks)
    rows, pulls, relaxed_dev = [], [], []
    for r, b in enumerate(boxes):
        Lf = b["L"][2] - 2
        tau = Lf * Lf * b["n"] / (math.pi ** 2 * theory[r] * b["dt"])
        relaxed = args.warmup >= 3 * tau
        dev = eta[r] / theory[r] - 1
        rows.append({"L": list(b["L"]), "n": b["n"], "drag": b["drag"], "eta": float(eta[r]), "stderr": float(err[r]),
                     "theory": theory[r], "deviation": float(dev), "tau_steps": tau, "relaxed": bool(relaxed)})
        if relaxed:
            pulls.append((eta[r] - theory[r]) / err[r])
            relaxed_dev.append(dev)
    pulls, relaxed_dev = np.array(pulls), np.array(relaxed_dev)
    precise = [row for row in rows if row["relaxed"] and row["stderr"] < 0.01 * row["theory"]]
    out = {"physics": "ensemble viscosity",
           "workload": f"{len(boxes)} of the {args.ensemble} batched-workload replicas (fluid height <= "
                       f"{args.max_height}), one batched handle, start at 0.9 x the analytic profile",
           "warmup_steps": args.warmup, "sampled_steps": blocks * per, "seconds": elapsed, "error_flags": flags,
           "relaxed_replicas": int(len(pulls)),
           "relaxed": {"mean_deviation": float(relaxed_dev.mean()) if len(pulls) else None,
                       "pull_mean": float(pulls.mean()) if len(pulls) else None,
                       "pull_std": float(pulls.std(ddof=1)) if len(pulls) > 1 else None},
           "precise_replicas": len(precise),
           "precise_within_2pct": sum(abs(row["deviation"]) < 0.02 for row in precise),
           "replicas": rows}
    print(json.dumps(out), flush=True)


def run_physics(args):
    import numpy as np

    from cudampcd_gb300 import capi

    alg = 1 if args.physics == "extended" else 0
    Lx, Ly, Lz = (args.size or (256, 256, 64))
    n, g, dt = args.n or 20, 0.0005, 0.02
    h = capi.Handle(L=(Lx, Ly, Lz + 2), periodic=(1, 1, 0), n=n, dt=dt, drag=g, algorithm=alg, seed=0)
    if args.eta_guess:   # start from the steady profile of a guessed viscosity: a shorter warm-up
        vel = h.velocities()
        z = h.positions()[:, 2].astype(np.float64)
        hz = Lz / 2.0
        vel[:, 0] += (n * g * (hz * hz - z * z) / (2.0 * args.eta_guess)).astype(np.float32)
        h.set_velocities(vel)
        del vel, z
    t0 = time.perf_counter()
    h.step(args.warmup)
    h.synchronize()
    t_warm = time.perf_counter() - t0
    blocks, per = 8, max(1, args.steps // 8)
    etas, P = [], []
    zc = np.arange(Lz + 2) + 0.5 - (Lz + 2) / 2.0
    fluid = slice(1, Lz + 1)
    A = np.stack([np.ones(Lz), -(zc[fluid] ** 2 + 1.0 / 12.0)], axis=1)
    dens = np.zeros(Lz + 2)
    for _ in range(blocks):
        h.wall_pressure(restart=True)
        h.step_and_sample(per)
        p0, p1, _ = h.wall_pressure()
        P.append((p0 + p1) / 2)
        d, v = h.sample_mean()
        u = v[:, 0].reshape(Lz + 2, Ly, Lx).mean(axis=(1, 2)) * (per - 1) / per
        dens += d.reshape(Lz + 2, Ly, Lx).mean(axis=(1, 2)) * (per - 1) / per / blocks
        (a, b), *_ = np.linalg.lstsq(A, u[fluid], rcond=None)
        etas.append(n * g / (2.0 * b))
    etas, P = np.array(etas), np.array(P)
    srd_theory = (1 - np.cos(2 * np.pi / 3)) / (18 * dt) * (n - 1 + np.exp(-n))
    out = {"physics": args.physics, "impl": "gb300",
           "workload": f"{args.physics} channel {Lx}x{Ly}x{Lz} cells + 2 walls, n={n}, T=1, dt={dt}, g={g}, N={h.N}",
           "fluid_density": n, "ms_per_step_warmup": 1e3 * t_warm / max(1, args.warmup),
           "warmup_steps": args.warmup, "sampled_steps": blocks * per, "warmup_s": t_warm,
           "initial_profile_eta": args.eta_guess,
           "wall_pressure": {"mean": float(P.mean()), "stderr": float(P.std(ddof=1) / np.sqrt(blocks)),
                             "ideal_gas_nT": float(n)},
           "viscosity": {"mean": float(etas.mean()), "stderr": float(etas.std(ddof=1) / np.sqrt(blocks)),
                         "srd_theory": float(srd_theory), "blocks": [float(e) for e in etas]},
           "density_profile_fluid": {"mean": float(dens[fluid].mean()), "min": float(dens[fluid].min()),
                                     "max": float(dens[fluid].max()), "first_layers": [float(x) for x in dens[1:5]],
                                     "layers": [float(x) for x in dens]},
           "velocity_profile": [float(x) for x in u],
           "device_counters": {"bucket_overflows": h.counters()[0], "error_flags": h.counters()[1]}}
    h.close()
    print(json.dumps(out), flush=True)


def run_viscosity(args):
    """SRD viscosity of the 10 x 10 x 100 channel, R replicas advanced as one
    batched handle (per-replica Philox seeds 2024 + r): eta per replica from the
    reference's estimator and from the curvature fit; mean and standard error
    over the replicas.  Analytic value (1 - cos a) / (18 dt) (n - 1 + e^-n)."""
    import numpy as np

    from cudampcd_gb300 import capi

    R, Lx, Ly, Lz, n, g, dt = 16, 10, 10, 100, 10, 0.001, 0.02
    theory = (1 - np.cos(2 * np.pi / 3)) / (18 * dt) * (n - 1 + np.exp(-n))
    zc = np.arange(Lz + 2) + 0.5 - (Lz + 2) / 2.0
    fluid = slice(1, Lz + 1)
    A = np.stack([np.ones(Lz), -(zc[fluid] ** 2 + 1.0 / 12.0)], axis=1)
    out = {"physics": "viscosity", "workload": f"SRD channel {Lx}x{Ly}x{Lz} cells + 2 walls, n={n}, T=1, dt={dt}, "
                                               f"g={g}, {R} replicas in one handle, seeds 2024+r",
           "srd_theory": float(theory), "protocols": {}}
    for name, warm, sampled in (("reference: 1000 warm-up, 100000 sampled", 1000, 100000),
                                ("5 relaxation times warm-up, 100000 sampled", 67500, 100000)):
        h = capi.Handle(boxes=[dict(L=(Lx, Ly, Lz + 2), periodic=(1, 1, 0), n=n, dt=dt, drag=g, seed=2024 + r)
                               for r in range(R)])
        t0 = time.perf_counter()
        h.step(warm)
        h.step_and_sample(sampled)
        _, v = h.sample_mean()
        elapsed = time.perf_counter() - t0
        flags = h.counters()[1]
        h.close()
        u = v[:, 0].reshape(R, Lz + 2, Ly, Lx).mean(axis=(2, 3)).astype(np.float64)   # as get_mean_fields gives it
        eta_max = Lz * Lz * n * g / (8.0 * u.max(axis=1))
        eta_fit = np.array([n * g / (2.0 * np.linalg.lstsq(A, ur[fluid] * (sampled - 1) / sampled, rcond=None)[0][1])
                            for ur in u])
        out["protocols"][name] = {
            "reference_estimator": {"mean": float(eta_max.mean()), "stderr": float(eta_max.std(ddof=1) / np.sqrt(R))},
            "curvature_fit": {"mean": float(eta_fit.mean()), "stderr": float(eta_fit.std(ddof=1) / np.sqrt(R))},
            "seconds": elapsed, "error_flags": flags}
    print(json.dumps(out), flush=True)


ADJOINT_WORKLOAD = dict(L=(64, 64, 34), n=10, drag=1e-3, dt=0.02, seed=5, steps=200, every=20)


def adjoint_block(warmup: int) -> dict:
    """The differentiable channel (64 x 64 x 32 cells + 2 walls, n = 10, dt = 0.02,
    200 sampled steps, checkpoints every 20): CUDA-event times of a plain step,
    of the sampled forward with checkpoints, and of the adjoint; the adjoint's
    cost relative to a plain step and to the forward."""
    import math

    import torch

    from cudampcd_gb300 import capi
    from cudampcd_gb300.adjoint import channel_profile

    w = ADJOINT_WORKLOAD
    L, n, drag0, dt, seed, S, K = w["L"], w["n"], w["drag"], w["dt"], w["seed"], w["steps"], w["every"]
    h = capi.Handle(L=L, periodic=(1, 1, 0), n=n, dt=dt, drag=drag0, seed=seed)
    N = h.N
    pos = torch.from_numpy(h.positions()).cuda()
    v_init = torch.from_numpy(h.velocities()).cuda()
    eta = (1.0 - math.cos(2 * math.pi / 3)) / (18.0 * dt) * (n - 1 + math.exp(-n))
    hz = L[2] / 2.0 - 1.0
    z = torch.arange(L[2], dtype=torch.float64, device="cuda") + 0.5 - L[2] / 2.0
    target = 1.1 * n * drag0 * (hz * hz - z * z) / (2.0 * eta)
    # plain steps (two launches each), timed on the handle's stream
    h.step(max(warmup, 6))
    total_ms, _ = h.time_steps(S)
    plain = total_ms / S
    fw, bw = [], []
    for rep in range(1 + 3):   # the first pass pays the one-time setup (tape allocation)
        v0 = v_init.clone().requires_grad_(True)
        g = torch.tensor(drag0, dtype=torch.float64, device="cuda", requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        U = channel_profile(h, pos, v0, g, S, K)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        loss = ((U[1:-1].double() - target[1:-1]) ** 2).mean()
        loss.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if rep:
            fw.append((t1 - t0) * 1e3 / S)
            bw.append((t2 - t1) * 1e3 / S)
        assert torch.isfinite(v0.grad).all()
    h.close()
    fwd, bwd = statistics.median(fw), statistics.median(bw)
    return {"workload": f"differentiable SRD channel {L[0]}x{L[1]}x{L[2] - 2} cells + 2 walls, n={n}, N={N}, "
                        f"dt={dt}, g={drag0}, {S} sampled steps, checkpoints every {K}; loss = MSE of U(z) against "
                        f"1.1 x the analytic parabola; gradients w.r.t. g and all V0",
            "timing": "plain steps: CUDA events on the handle's stream; forward and backward: host wall clock "
                      "around each call (both synchronise), median of 3 after one untimed pass",
            "particles": N, "plain_ms_per_step": plain, "forward_ms_per_step": fwd, "backward_ms_per_step": bwd,
            "backward_over_plain": bwd / plain, "backward_over_forward": bwd / fwd,
            "forward_plus_backward_over_plain": (fwd + bwd) / plain}


def run_adjoint(args):
    """The adjoint line: value = particle-steps/s of the adjoint (backward) sweep."""
    a = adjoint_block(args.warmup)
    bwd = a["backward_ms_per_step"]
    out = {"metric": METRIC, "value": a["particles"] / (bwd * 1e-3), "unit": UNIT, "n_gpus": 1,
           "steps": ADJOINT_WORKLOAD["steps"], "warmup": args.warmup, "ms_per_step": bwd, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": a["workload"], "timing": a["timing"]},
           "adjoint": {k: v for k, v in a.items() if k not in ("workload", "timing")}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=100)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference", "reference-cuda"])
    ap.add_argument("--kernel", default="optimized", choices=["optimized", "sorting", "trivial"])
    ap.add_argument("--no-reference-gpu", dest="no_reference_gpu", action="store_true")
    ap.add_argument("--adjoint", action="store_true")
    ap.add_argument("--steps-cpu", dest="steps_cpu", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", dest="no_adjoint", action="store_true")
    ap.add_argument("--size", type=int, nargs=3, metavar=("LX", "LY", "LZ"))
    ap.add_argument("--algorithm", default="srd", choices=["srd", "extended"])
    ap.add_argument("--ensemble", type=int, default=0, metavar="R")
    ap.add_argument("--small-replicas", dest="small_replicas", action="store_true")
    ap.add_argument("--physics", choices=["extended", "srd", "viscosity"])
    ap.add_argument("--eta-guess", dest="eta_guess", type=float, default=0.0)
    ap.add_argument("--n", type=int, default=0, help="particles per cell of the physics workloads")
    ap.add_argument("--viscosity", action="store_true", help="with --ensemble: per-replica viscosity")
    ap.add_argument("--max-height", dest="max_height", type=int, default=74)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("at least 3 warm-up steps")
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", args.gpus))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.adjoint:
        run_adjoint(args)
    elif args.ensemble and args.viscosity:
        run_ensemble_viscosity(args)
    elif args.ensemble:
        run_ensemble(args)
    elif args.physics == "viscosity":
        run_viscosity(args)
    elif args.physics and args.impl == "reference-cuda":
        run_reference_cuda(args, rank, local_rank)
    elif args.physics:
        run_physics(args)
    elif args.impl == "reference":
        run_reference_arm(args, rank)
    elif args.impl == "reference-cuda":
        run_reference_cuda(args, rank, local_rank)
    else:
        run_gpu_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    main()

"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1).

Each GPU rank runs an independent replica, so the only cross-rank steps are the
barrier and the max over ranks of the timed region; the whole-job value counts
every rank's particle-steps.  The reference arm prints on rank 0 alone.
"""
from __future__ import annotations

import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        dist.barrier()
        elapsed = bench.reduce_max(10.0 + 5.0 * rank, dist, device="cpu")   # rank 1 is the slow one
        out.put((rank, elapsed, bench.whole_job_rate(world, 1000, 20, elapsed)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_value_with_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp

    ctx = tmp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in results] == [0, 1]
    assert all(e == 15.0 for _, e, _ in results)                      # both ranks see the slowest time
    assert all(v == 2 * 1000 * 20 / 15.0 for _, _, v in results)       # all ranks' work over it
    assert torch is not None


def test_reference_arm_prints_on_rank_zero_only():
    import argparse

    import bench

    args = argparse.Namespace(gpus=2, steps=1, warmup=3)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference_arm(args, rank=1)
    assert buf.getvalue() == ""


def test_device_memory_block_at_config_2():
    """The bench line's bucket figures: depth min(4n, n + ceil(4 sqrt(n)) + 2) slots of
    32 B per cell and parity, plus the extension area; 56.6 GB at config 2 against
    112.6 GB at the reference's 4n."""
    import bench

    cells, n = 1000 * 1000 * 22, 20
    m = bench.device_memory(int(68.5e9), n, cells, 1000 * 1000 * 20 * n)
    assert m["bucket_depth"] == 40 and m["bucket_depth_reference"] == 80
    assert abs(m["buckets_gb"] - 56.59) < 0.01
    assert abs(m["buckets_gb_at_reference_depth"] - 112.64) < 0.01
    for k in (1, 2, 3, 5, 10, 64, 409):
        d = bench.device_memory(0, k, 1000, 1000 * k)["bucket_depth"]
        assert k < d <= 4 * k or k == 1 and d == 4

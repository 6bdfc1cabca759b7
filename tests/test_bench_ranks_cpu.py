"""Replica aggregation of bench.py across ranks, on CPU with the gloo backend.

Multi-GPU runs are replicas: each rank solves its own instance, the timed region
lasts as long as the slowest rank (max over ranks), and throughputs add up. Two
gloo processes check the helpers bench.py uses for exactly that.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        slowest = bench.reduce_over_ranks([1.0 + rank], dist, "max", device="cpu")[0]
        total = bench.reduce_over_ranks([10.0 * (rank + 1), 1.0], dist, "sum", device="cpu")
        value, secs = bench.job_throughput(5, 2.0 + rank, world, dist, device="cpu")
        q.put((rank, slowest, total, value, secs))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_and_sum_throughputs():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, total, value, secs in got:
        assert slowest == 2.0
        assert total == [30.0, 2.0]
        assert secs == 3.0 and value == pytest.approx(2 * 5 / 3.0)


def test_single_process_needs_no_group():
    import bench
    assert bench.reduce_over_ranks([4.0], None) == [4.0]
    assert bench.job_throughput(3, 1.5, 1, None) == (2.0, 1.5)


def test_reference_arm_prints_its_line():
    """`bench.py --impl reference` times the oracle's restatement of the reference
    build and serial matvec on the host cores and prints one JSON line with the
    contract's keys (the c0 workload and a one-second sample keep this short)."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--config", "c0",
                          "--steps", "1", "--warmup", "0", "--cpu-seconds", "1"],
                         capture_output=True, text=True, timeout=600, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([x for x in out.stdout.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["unit"] == "solves/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]

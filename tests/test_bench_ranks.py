"""The multi-rank reduction of bench.py (replicas: every rank steps its own
world, the job's time is the slowest rank's) on two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world_size, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        total_ms = bench.max_over_ranks(100.0 + 25.0 * rank, dist, "cpu")
        value = bench.job_throughput(1000, 10, world_size, total_ms)
        out.put((rank, total_ms, value))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total_ms, value in res:
        assert total_ms == 125.0                       # the slowest rank's time on every rank
        assert value == pytest.approx(2 * 1000 * 10 / 0.125)  # both ranks' bodies over that time


def test_single_process_paths():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(42.0, None, None) == 42.0
    assert bench.job_throughput(1_000_000, 20, 1, 2000.0) == pytest.approx(1e7)

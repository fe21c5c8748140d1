"""bench.py's multi-GPU reduction (replicas: max time over ranks, whole-job
throughput) on two gloo ranks on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [1000.0, 1500.0][rank]
    total_ms, value = bench.replica_throughput(local_ms, 1e6, world, device="cpu")
    q.put((rank, total_ms, value))
    dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total_ms, value in res:
        assert total_ms == 1500.0
        assert value == pytest.approx(2 * 1e6 / 1.5)

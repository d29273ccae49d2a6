"""The multi-GPU path of bench.py is replicas only (no data-path collective): each rank steps its own
copy of the scene and rank 0 reports the aggregate over the slowest rank's time.  The reduction and
the aggregate are exercised here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (r + 1) seconds: the job is as slow as rank 1
        t = bench.max_over_ranks(float(rank + 1), world, "cpu")
        out[rank] = (t, bench.replica_throughput(world, 1000, 50, t))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_slowest_rank():
    import torch.multiprocessing as mp
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        t, v = out[r]
        assert t == 2.0
        assert v == pytest.approx(2 * 1000 * 50 / 2.0)

"""Multi-rank bench logic on CPU (gloo, world_size 2): replicas are independent, and the
whole-job throughput is the units summed over ranks over the slowest rank's time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    d = bench.init_dist(world, "gloo")
    units = 1000.0 * (rank + 1)          # replicas of different sizes
    seconds = 0.5 + rank                 # rank 1 is the slowest
    value, tmax, total = bench.aggregate(d, units, seconds)
    bench.barrier(d)
    out[rank] = (value, tmax, total)
    dist.destroy_process_group()


def test_aggregate_two_ranks_gloo():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, join=True,
                       start_method="spawn")
    for r in range(world):
        value, tmax, total = out[r]
        assert tmax == 1.5 and total == 3000.0
        assert abs(value - 2000.0) < 1e-9


def test_single_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.init_dist(1, "gloo") is None
    assert bench.aggregate(None, 10.0, 2.0) == (5.0, 2.0, 10.0)

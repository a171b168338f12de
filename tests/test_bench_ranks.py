"""The multi-GPU path of bench.py is replicas: each rank runs the whole workload on its own GPU
with no exchange; the job's time is the slowest rank's (max over ranks) and `value` sums the work
of all ranks.  Checked here with 2 gloo ranks on CPU (no GPU needed)."""
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


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    mine = 1.0 + rank * 0.5                      # rank 1 is the slow one
    worst = bench.max_over_ranks(mine, dist, "cpu")
    units = 100.0                                # work per rank
    out[rank] = (worst, units * world / worst)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (1.5, 200.0 / 1.5)


def test_single_process_needs_no_collective():
    import bench
    assert bench.max_over_ranks(2.5) == 2.5

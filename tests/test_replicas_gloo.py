"""The N > 1 path of bench.py (independent replicas, one per rank) on CPU:
two gloo ranks exchange only the barrier and the max-over-ranks of the step
time; rank 0 reports the total throughput of all replicas."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, times, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(world)
    mx = bench.allreduce_max(times[rank], world)
    out[rank] = mx
    dist.destroy_process_group()


def test_two_rank_max_reduction():
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    times = [3.5, 7.25]
    mp.spawn(_worker, args=(world, port, times, out), nprocs=world, join=True)
    assert out[0] == out[1] == 7.25

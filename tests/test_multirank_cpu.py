"""The multi-rank path of bench.py on CPU: two gloo ranks (127.0.0.1).  Each
rank traces its own ray batch (distinct seeds, weak scaling) and the timed
region is the slowest rank's (max-reduce); no data-path collective."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.reduce_max(1.5 + rank, world)
    out[rank] = (t, bench.rank_ray_seed(rank))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_max_reduce_and_seeds():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    assert out[0][0] == out[1][0] == 2.5
    assert out[0][1] != out[1][1]
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.reduce_max(3.0, 1) == 3.0

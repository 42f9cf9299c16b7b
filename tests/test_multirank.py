"""CPU, world size 2 over gloo: the benchmark's multi-rank path -- each rank
owns a different shard of instances (no collective on the data path), the
ranks meet at a barrier, and the step time is the maximum over ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, float(rank + 1) * 0.5)
    seed = bench.SEED + 7919 * rank
    out[rank] = (t, seed)
    bench.barrier(dist)
    dist.destroy_process_group()


def test_two_ranks_gloo():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()      # no fork: the test process may run host worker threads
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    assert out[0][0] == out[1][0] == 1.0          # max over ranks
    assert out[0][1] != out[1][1]                  # disjoint instance shards

"""The N > 1 bench path on CPU: two gloo ranks (replicas) aggregate their
timings as the slowest rank and their SIP updates as the sum, and draw
disjoint seeds."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, ups = bench.aggregate_ranks(10.0 + rank, 1000.0 * (rank + 1), dist, "cpu")
    seeds = bench.rank_seeds(rank, 4)
    gathered = [None] * world
    dist.all_gather_object(gathered, seeds)
    out[rank] = (ms, ups, gathered)
    dist.destroy_process_group()


def test_two_rank_aggregation():
    world = 2
    port = _free_port()
    mgr = tmp.Manager()
    out = mgr.dict()
    tmp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        ms, ups, gathered = out[r]
        assert ms == 11.0                 # the slowest rank's time
        assert ups == 3000.0              # all ranks' SIP updates
        keys = [k for g in gathered for k in g[0]] + [k for g in gathered for k in g[1]]
        assert len(keys) == len(set(keys))   # disjoint Philox keys and state seeds

"""Host-side multi-rank logic on CPU with gloo, world size 2: shards cover
every item exactly once, and the benchmark's aggregation takes the slowest
rank's time and the total work."""
import os
import socket

import pytest

from einspline_gb300 import parallel


def test_shard_range_partitions():
    for n in (0, 1, 7, 1024, 1025):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = parallel.shard_range(n, r, world)
                seen.extend(range(lo, hi))
            assert seen == list(range(n))


def test_shard_splines_aligned():
    for N in (1, 100, 1024, 2048, 2050):
        for world in (1, 2, 4, 8):
            cols = []
            for r in range(world):
                f, c = parallel.shard_splines(N, r, world)
                assert f % 32 == 0
                cols.extend(range(f, f + c))
            assert cols == list(range(N))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lo, hi = parallel.shard_range(1000, rank, world)
    ms, work = parallel.aggregate(10.0 + rank, float(hi - lo))
    q.put((rank, ms, work))
    dist.destroy_process_group()


def test_aggregate_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, work in out:
        assert ms == 11.0 and work == 1000.0

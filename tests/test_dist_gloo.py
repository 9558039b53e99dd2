"""The replica path's host logic on two CPU ranks (gloo, world_size 2)."""
import os

import pytest


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from rpmplv2_gb300.dist import max_over_ranks, shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = max_over_ranks(1.0 + rank)          # the slowest rank defines the step time
    b, e = shard(1000, rank, world)
    dist.destroy_process_group()
    q.put((rank, t, b, e))


def test_two_rank_replicas():
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]
    assert res[0][2:] == (0, 500) and res[1][2:] == (500, 1000)


def test_shard_covers_everything():
    from rpmplv2_gb300.dist import shard
    for n in (0, 1, 7, 1000):
        for w in (1, 2, 3, 8):
            parts = [shard(n, r, w) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(w - 1))

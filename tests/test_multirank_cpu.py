"""Multi-GPU path on the CPU: world_size-2 gloo ranks shard the columns with
aeroapps_gb300.shard, check that the shards are disjoint, cover every column
and are balanced by cost, and reduce a per-rank time with MAX as bench.py
does.  No GPU and no data-path collective."""
import os
import socket

import numpy as np
import pytest

from aeroapps_gb300 import shard


def test_shard_bounds_cover_and_balance():
    rng = np.random.default_rng(0)
    ns = rng.choice([4, 6, 8, 12, 16], 5000)
    nl = rng.integers(20, 73, 5000)
    cost = shard.column_cost(ns, nl)
    for world in (1, 2, 3, 8):
        b = shard.shard_bounds(cost, world)
        assert b[0] == 0 and b[-1] == 5000 and np.all(np.diff(b) >= 0)
        per = np.array([cost[b[r]:b[r + 1]].sum() for r in range(world)])
        # each cut lands within one column of its cost target
        assert per.max() - per.min() <= 2 * cost.max() + 1e-9
    assert list(shard.shard_bounds([1.0, 1.0], 4)) == [0, 1, 1, 2, 2]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(1)
    ns = rng.choice([4, 6, 8, 12, 16], 777)
    nl = rng.integers(20, 73, 777)
    mine = shard.my_columns(ns, nl, rank, world)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([len(mine)], dtype=torch.int64))
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q.put((rank, mine.tolist(), [int(x.item()) for x in sizes], float(t.item())))
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_without_exchange():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    cols = res[0][1] + res[1][1]
    assert sorted(cols) == list(range(777)) and len(set(res[0][1]) & set(res[1][1])) == 0
    assert res[0][2] == res[1][2] == [len(res[0][1]), len(res[1][1])]
    assert res[0][3] == res[1][3] == 2.0

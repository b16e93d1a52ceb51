"""Multi-GPU path on the CPU: world_size-2 gloo ranks shard the columns with
aeroapps_gb300.shard, check that the shards are disjoint, cover every column
and are balanced by cost, and reduce a per-rank time with MAX as bench.py
does; each rank solves its shard (with the oracle, standing in for one GPU)
and shard.gather concatenates radiance(nobs, nch) on rank 0, bit-identical
to a one-rank solve.  No GPU and no data-path collective."""
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


def _solve(args):
    from oracle import oracle
    a = args
    rad, refl, rc, nf, st = oracle.scalar_lambert(
        a["km"], a["nch"], a["solar_zenith"].shape[0], a["channels"], 8, False, a["nMom"], 1, a["ROT"], a["depol"],
        a["tau"], a["ssa"], a["g"], a["pmom"], a["pe"], a["he"], a["te"], a["albedo"], a["solar_zenith"],
        a["relat_azymuth"], a["sensor_zenith"], -1.0e15)
    assert rc == 0
    return rad, refl


def _case():
    from rt_cases import random_aop_case
    c = random_aop_case(8, 24, nobs=37, nch=2, seed=4)
    return {"km": c["km"], "nch": c["nch"], "channels": c["channels"], "nMom": c["nmom"], "ROT": c["ROT"],
            "depol": c["depol"], "tau": c["tau"], "ssa": c["ssa"], "g": c["g"], "pmom": c["pmom"], "pe": c["pe"],
            "he": c["he"], "te": c["te"], "albedo": c["albedo"], "solar_zenith": c["sza"],
            "relat_azymuth": c["raa"], "sensor_zenith": c["vza"]}


def _gather_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    a = _case()
    nobs = a["solar_zenith"].shape[0]
    b = shard.shard_bounds(shard.column_cost(np.full(nobs, 8), np.full(nobs, a["km"])), world)
    mine = shard.slice_columns(a, b[rank], b[rank + 1])
    rad, refl = _solve(mine)
    full = shard.gather(rad, b, rank, world)
    full_refl = shard.gather(refl, b, rank, world)
    q.put((rank, None if full is None else (full, full_refl), [int(x) for x in b]))
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_radiances_identical_to_one_rank():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gather_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[1][1] is None
    b = res[0][2]
    assert b[0] == 0 < b[1] < b[2] == 37
    rad1, refl1 = _solve(_case())
    rad2, refl2 = res[0][1]
    assert rad2.shape == rad1.shape == (37, 2)
    assert np.array_equal(rad2, rad1) and np.array_equal(refl2, refl1)


def test_slice_columns_and_single_rank_gather():
    a = _case()
    s = shard.slice_columns(a, 5, 9)
    assert s["tau"].shape == (24, 2, 4) and s["ROT"].shape == (24, 4, 2) and s["pe"].shape == (25, 4)
    assert s["albedo"].shape == (4, 2) and s["solar_zenith"].shape == (4,) and s["pmom"].shape[2] == 4
    assert np.array_equal(s["tau"], a["tau"][:, :, 5:9]) and s["depol"] is a["depol"]
    x = np.arange(6.0).reshape(3, 2)
    assert shard.gather(x, [0, 3], 0, 1) is x
    with pytest.raises(ValueError):
        shard.gather(x, [0, 2], 0, 1)

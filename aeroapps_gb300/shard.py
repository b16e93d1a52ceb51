"""Column sharding across GPUs (one process per GPU).

Columns are independent: the reference distributes pixels over MPI ranks
(src/Components/rtms/geo_vlidort/geo_vlidort.F90:482-500) and nothing is
exchanged between them.  Here each rank takes one contiguous range of
columns, the ranges balanced by the estimated solve cost of each column
(layers x streams^3, the order of the per-layer eigen- and interface solves),
and results are concatenated on the host in rank order.  No collective is
needed on the data path; bench.py only reduces its timing with MAX.
"""
import numpy as np


def column_cost(nstreams, nlayers):
    """Relative cost of one column: L N^3 (plus a small per-column term)."""
    ns = np.asarray(nstreams, np.float64)
    nl = np.asarray(nlayers, np.float64)
    return nl * ns ** 3 + 64.0 * nl


def shard_bounds(cost, world):
    """Split columns 0..n-1 into `world` contiguous ranges of about equal total
    cost; returns bounds b (len world+1), rank r owns [b[r], b[r+1])."""
    cost = np.asarray(cost, np.float64)
    n = cost.size
    if world < 1:
        raise ValueError("world must be >= 1")
    c = np.concatenate([[0.0], np.cumsum(cost)])
    targets = c[-1] * np.arange(1, world) / world
    cuts = np.searchsorted(c, targets, side="left")
    b = np.concatenate([[0], np.clip(cuts, 0, n), [n]]).astype(np.int64)
    return np.maximum.accumulate(b)


def my_columns(nstreams, nlayers, rank, world):
    """Indices of the columns rank `rank` of `world` solves."""
    b = shard_bounds(column_cost(nstreams, nlayers), world)
    return np.arange(b[rank], b[rank + 1])

"""Column sharding across GPUs (one process per GPU).

Columns are independent: the reference distributes pixels over MPI ranks
(src/Components/rtms/geo_vlidort/geo_vlidort.F90:482-500) and nothing is
exchanged between them.  Here each rank takes one contiguous range of
columns, the ranges balanced by the estimated solve cost of each column
(layers x streams^3, the order of the per-layer eigen- and interface solves),
and results are concatenated on the host in rank order (the reference's
ranks write their pixels into one node-shared output array,
geo_vlidort.F90:482-500 with MAPL_AllocNodeArray).  No collective is needed
on the data path: `gather` moves each rank's finished rows once, at the end,
and bench.py only reduces its timing with MAX.
"""
import numpy as np

# Position of the column (pixel, nobs) axis in each argument of the
# reference routines, with their Fortran shapes
# (geo_vlidort/VLIDORT_LAMBERT.F90:34-168 and :172-342).
OBS_AXIS = {
    "ROT": 1, "alpha": 1,                                       # (km, nobs, nch)
    "tau": 2, "ssa": 2, "g": 2, "pmom": 2,                      # (km, nch, nobs[, nMom, nPol])
    "pe": 1, "he": 1, "te": 1,                                  # (km+1, nobs)
    "albedo": 0, "radiance_VL": 0, "reflectance_VL": 0, "Q": 0, "U": 0,  # (nobs, nch)
    "solar_zenith": 0, "relat_azymuth": 0, "sensor_zenith": 0,  # (nobs)
    "flux_factor": 1,                                           # (nch, nobs)
}


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


def slice_columns(args, lo, hi):
    """The arguments of the columns [lo, hi) of a reference call: every array
    named in OBS_AXIS is cut along its column axis (kept in Fortran order);
    the other entries (channels, depol, sizes) pass through."""
    out = {}
    for k, v in args.items():
        ax = OBS_AXIS.get(k)
        if ax is None or not isinstance(v, np.ndarray):
            out[k] = v
            continue
        idx = [slice(None)] * v.ndim
        idx[ax] = slice(lo, hi)
        out[k] = np.asfortranarray(v[tuple(idx)])
    return out


def gather(local, bounds, rank, world, dst=0, group=None):
    """Host-side concatenation of per-rank results along the column axis.

    `local` is this rank's (ncols_rank, ...) array for the columns
    [bounds[rank], bounds[rank+1]) -- radiance(nobs, nch) rows, say.  Rank
    `dst` returns the (bounds[-1], ...) array in column order, the others
    None.  One torch.distributed.gather on CPU tensors (gloo, or a CPU-capable
    backend), padded to the largest shard: a single exchange after the work,
    nothing on the data path.  world == 1 returns `local` unchanged."""
    local = np.asarray(local)
    b = np.asarray(bounds, np.int64)
    if b.size != world + 1 or local.shape[0] != b[rank + 1] - b[rank]:
        raise ValueError("local rows %d do not match shard [%d, %d)" % (local.shape[0], b[rank], b[rank + 1]))
    if world == 1:
        return local
    import torch
    import torch.distributed as dist
    width = int(np.max(np.diff(b)))
    tail = local.shape[1:]
    buf = torch.zeros((width,) + tail, dtype=torch.from_numpy(local[:0]).dtype)
    if local.shape[0]:
        buf[:local.shape[0]] = torch.from_numpy(np.ascontiguousarray(local))
    parts = [torch.empty_like(buf) for _ in range(world)] if rank == dst else None
    dist.gather(buf, parts, dst=dst, group=group)
    if rank != dst:
        return None
    return np.concatenate([parts[r][:b[r + 1] - b[r]].numpy() for r in range(world)], axis=0)

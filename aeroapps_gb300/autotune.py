"""Schedule autotuner for the RT solve, per (layers, streams, precision) bucket.

A launch solves columns of one stream count whose layer counts fall in one
bucket (upper bounds LAYER_BUCKETS).  For each bucket the tuner times a probe
batch of that bucket under each candidate schedule and keeps the fastest:

- the kernel: one thread per solve (thread kernel), or the two-pass team
  solve (set-up thread per solve, Fourier series on a whole warp per solve
  with the layer matrices in shared memory);
- threads per block of the thread kernel (32, 64 or 128), which sets how many
  solves share an SM's L1 for their per-solve working set;
- resident blocks per SM (0 = the occupancy limit), which caps the grid.

Timings use CUDA events on the launching stream.  The table measured on
GB300 ships with the package (schedules_gb300.json, applied by
apply_defaults); a re-tune writes the local cache (_build/schedules.json),
which overrides it.  Before each launch the caller applies the entry of the
launch's bucket (apply_for), which sets the library's schedule and kernel for
that stream count and precision (aerort_set_schedule, aerort_set_kernel).
Buckets without an entry run the library's automatic choice.
"""
import json
import os
import time

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULTS = os.path.join(HERE, "schedules_gb300.json")
CACHE = os.path.join(HERE, "_build", "schedules.json")
LAYER_BUCKETS = (36, 54, 72)

# (kernel, threads per block, blocks per SM); the team kernel has two-warp blocks
CANDIDATES = ((_lib.KERNEL_TEAM, 64, 0), (_lib.KERNEL_THREAD, 32, 0), (_lib.KERNEL_THREAD, 64, 0),
              (_lib.KERNEL_THREAD, 128, 0), (_lib.KERNEL_TEAM, 64, 4), (_lib.KERNEL_THREAD, 64, 2))

_active = {}  # (nstreams, layer bucket, precision) -> entry, for the current device


def layer_bucket(km):
    """Upper bound of the bucket holding a launch whose deepest column has km layers."""
    for b in LAYER_BUCKETS:
        if km <= b:
            return b
    raise ValueError("km > %d" % LAYER_BUCKETS[-1])


def _key(nstreams, km, precision):
    return "N%d|L%d|%s" % (nstreams, layer_bucket(km), "mixed" if precision == _lib.PREC_MIXED else "fp64")


def load_table(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_table(table, path=CACHE):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _set(nstreams, precision, kernel, threads_per_block, blocks_per_sm):
    L = _lib.lib()
    rc = L.aerort_set_schedule(nstreams, precision, threads_per_block, blocks_per_sm)
    if rc == 0:
        rc = L.aerort_set_kernel(nstreams, precision, kernel)
    if rc != 0:
        raise RuntimeError("aerort_set_schedule rc=%d: %s" % (rc, _lib.last_error()))


def apply_defaults(device_name, defaults=DEFAULTS, cache=CACHE):
    """Load the shipped table and the local cache (which wins) for this device
    name; returns a one-line description of where the entries came from."""
    _active.clear()
    src = []
    for path, label in ((defaults, "shipped GB300 table"), (cache, "local re-tune")):
        t = load_table(path).get(device_name, {})
        if t:
            _active.update({k: v for k, v in t.items()})
            src.append("%s (%d buckets)" % (label, len(t)))
    return ", ".join(src) if src else "none (library automatic choice)"


def table_summary(device_name=None):
    """{bucket: "kernel threads/blocks_per_sm"} of the active table."""
    name = {_lib.KERNEL_TEAM: "team", _lib.KERNEL_THREAD: "thread", _lib.KERNEL_AUTO: "auto"}
    return {k: "%s %d/%d" % (name.get(v["kernel"], "?"), v["threads"], v["blocks_per_sm"])
            for k, v in sorted(_active.items())}


def apply_for(nstreams, km, precision):
    """Install the schedule of the (layers, streams, precision) bucket of a
    launch (the library default when the table has no entry for it)."""
    v = _active.get(_key(nstreams, km, precision))
    if v is None:
        _set(nstreams, precision, _lib.KERNEL_AUTO, 32, 0)
    else:
        _set(nstreams, precision, v["kernel"], v["threads"], v["blocks_per_sm"])


def tune(run, nstreams, km, precision, device_name, candidates=CANDIDATES, reps=1, budget_s=60.0, path=CACHE):
    """Time `run()` (one launch of the bucket on the current CUDA stream, with
    device-resident inputs) under each candidate; keep, install and cache the
    fastest.  Returns {"best": (kernel, threads, bps, ms), "all": [...]}."""
    import torch
    results = []
    t0 = time.time()
    for kern, tpb, bps in candidates:
        if results and time.time() - t0 > budget_s:
            break
        _set(nstreams, precision, kern, tpb, bps)
        run()  # warm: scratch sized for this grid
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            run()
        e1.record()
        torch.cuda.synchronize()
        results.append((kern, tpb, bps, e0.elapsed_time(e1) / reps))
    kern, tpb, bps, ms = min(results, key=lambda r: r[3])
    entry = {"kernel": kern, "threads": tpb, "blocks_per_sm": bps, "ms": ms,
             "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    _active[_key(nstreams, km, precision)] = entry
    _set(nstreams, precision, kern, tpb, bps)
    table = load_table(path)
    table.setdefault(device_name, {})[_key(nstreams, km, precision)] = entry
    save_table(table, path)
    return {"best": (kern, tpb, bps, ms), "all": results}

"""Schedule autotuner for the RT kernel.

For each (stream count, precision) bucket the kernel runs as a persistent grid
of thread-per-solve blocks.  Two knobs decide how many solves are resident on
an SM, and with them how much of the per-solve working set (several KB of
matrices per thread) stays in L1/L2: threads per block and resident blocks per
SM.  The tuner times a short probe batch of the bucket under each candidate
schedule (CUDA events on the launching stream), keeps the fastest, and installs
it with aerort_set_schedule.  Results are cached per device name in a JSON
file so that later processes reuse them.
"""
import json
import os
import time


from . import _lib

# (kernel, threads per block, blocks per SM); the team kernel has 64-thread blocks
CANDIDATES = ((_lib.KERNEL_TEAM, 64, 0), (_lib.KERNEL_THREAD, 64, 0), (_lib.KERNEL_THREAD, 32, 0),
              (_lib.KERNEL_TEAM, 64, 2), (_lib.KERNEL_THREAD, 128, 0), (_lib.KERNEL_THREAD, 64, 2))
CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "schedules.json")


def _key(device_name, nstreams, precision):
    return "%s|N%d|%s" % (device_name, nstreams, "mixed" if precision == _lib.PREC_MIXED else "fp64")


def load_cache(path=CACHE):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(cache, path=CACHE):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply(nstreams, precision, threads_per_block, blocks_per_sm, kernel=None):
    L = _lib.lib()
    rc = L.aerort_set_schedule(nstreams, precision, threads_per_block, blocks_per_sm)
    if rc == 0 and kernel is not None:
        rc = L.aerort_set_kernel(nstreams, precision, kernel)
    if rc != 0:
        raise RuntimeError("aerort_set_schedule rc=%d: %s" % (rc, _lib.last_error()))


def apply_cached(device_name, path=CACHE):
    """Install every cached schedule of this device; returns how many."""
    n = 0
    for k, v in load_cache(path).items():
        dev, ns, prec = k.split("|")
        if dev != device_name:
            continue
        apply(int(ns[1:]), _lib.PREC_MIXED if prec == "mixed" else _lib.PREC_FP64, v["threads"], v["blocks_per_sm"],
              v.get("kernel"))
        n += 1
    return n


def tune(run, nstreams, precision, device_name, candidates=CANDIDATES, reps=1, budget_s=60.0, path=CACHE):
    """Time `run()` (one launch of the bucket on the current CUDA stream) under
    each candidate (kernel, schedule); install and cache the fastest.

    run: callable enqueuing the RT launch for this bucket (device-resident inputs).
    Returns {"kernel", "threads", "blocks_per_sm", "ms", "all": [(kernel, threads, bps, ms), ...]}.
    """
    import torch
    results = []
    t0 = time.time()
    for kern, tpb, bps in candidates:
        if results and time.time() - t0 > budget_s:
            break
        apply(nstreams, precision, tpb, bps, kern)
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
    apply(nstreams, precision, tpb, bps, kern)
    cache = load_cache(path)
    cache[_key(device_name, nstreams, precision)] = {"kernel": kern, "threads": tpb, "blocks_per_sm": bps, "ms": ms,
                                                    "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    save_cache(cache, path)
    return {"kernel": kern, "threads": tpb, "blocks_per_sm": bps, "ms": ms, "all": results}

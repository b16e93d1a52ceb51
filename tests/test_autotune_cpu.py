"""Host logic of the schedule autotuner (aeroapps_gb300/autotune.py): the
(layers, streams, precision) buckets, the shipped table and the local cache,
and their installation through aerort_set_schedule / aerort_set_kernel.  The
timing loop itself needs a GPU and runs in bench.py --tune."""
import ctypes
import json
import os

import pytest

from aeroapps_gb300 import _lib, autotune


@pytest.fixture
def restore_defaults():
    L = _lib.lib()
    saved = {}
    for ns in (4, 6, 8, 12, 16):
        for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
            t, b = ctypes.c_int(), ctypes.c_int()
            assert L.aerort_get_schedule(ns, prec, ctypes.byref(t), ctypes.byref(b)) == 0
            saved[(ns, prec)] = (t.value, b.value, L.aerort_get_kernel(ns, prec))
    yield
    for (ns, prec), (t, b, k) in saved.items():
        assert L.aerort_set_schedule(ns, prec, t, b) == 0
        assert L.aerort_set_kernel(ns, prec, k) == 0
    autotune._active.clear()


def _get(ns, prec):
    L = _lib.lib()
    t, b = ctypes.c_int(), ctypes.c_int()
    assert L.aerort_get_schedule(ns, prec, ctypes.byref(t), ctypes.byref(b)) == 0
    return L.aerort_get_kernel(ns, prec), t.value, b.value


def test_layer_buckets():
    assert [autotune.layer_bucket(k) for k in (1, 20, 36, 37, 54, 55, 72)] == [36, 36, 36, 54, 54, 72, 72]
    with pytest.raises(ValueError):
        autotune.layer_bucket(73)
    assert autotune._key(8, 40, _lib.PREC_MIXED) == "N8|L54|mixed"


def test_table_install_per_bucket(tmp_path, restore_defaults):
    shipped = os.path.join(tmp_path, "shipped.json")
    cache = os.path.join(tmp_path, "cache.json")
    T, H = _lib.KERNEL_TEAM, _lib.KERNEL_THREAD
    with open(shipped, "w") as f:
        json.dump({"GB300": {"N8|L36|mixed": {"kernel": H, "threads": 128, "blocks_per_sm": 0},
                             "N8|L72|mixed": {"kernel": T, "threads": 64, "blocks_per_sm": 4},
                             "N4|L72|fp64": {"kernel": H, "threads": 64, "blocks_per_sm": 2}},
                   "other GPU": {"N12|L72|fp64": {"kernel": H, "threads": 32, "blocks_per_sm": 1}}}, f)
    autotune.save_table({"GB300": {"N4|L72|fp64": {"kernel": T, "threads": 64, "blocks_per_sm": 0}}}, cache)
    src = autotune.apply_defaults("GB300", shipped, cache)
    assert "3 buckets" in src and "1 buckets" in src
    # the layer bucket of the launch picks the entry
    autotune.apply_for(8, 30, _lib.PREC_MIXED)
    assert _get(8, _lib.PREC_MIXED) == (H, 128, 0)
    autotune.apply_for(8, 72, _lib.PREC_MIXED)
    assert _get(8, _lib.PREC_MIXED) == (T, 64, 4)
    # the local re-tune overrides the shipped entry
    autotune.apply_for(4, 60, _lib.PREC_FP64)
    assert _get(4, _lib.PREC_FP64) == (T, 64, 0)
    # a bucket without an entry gets the library's automatic choice
    autotune.apply_for(8, 50, _lib.PREC_MIXED)
    assert _get(8, _lib.PREC_MIXED) == (_lib.KERNEL_AUTO, 32, 0)
    assert "N8|L36|mixed" in autotune.table_summary()


def test_shipped_table_is_valid():
    t = autotune.load_table(autotune.DEFAULTS)
    for dev, entries in t.items():
        for k, v in entries.items():
            n, lb, prec = k.split("|")
            assert int(n[1:]) in (4, 6, 8, 12, 16) and int(lb[1:]) in autotune.LAYER_BUCKETS
            assert prec in ("mixed", "fp64")
            assert v["kernel"] in (_lib.KERNEL_THREAD, _lib.KERNEL_TEAM) and v["threads"] in (32, 64, 96, 128)


def test_invalid_schedule_is_refused(restore_defaults):
    with pytest.raises(RuntimeError):
        autotune._set(8, _lib.PREC_FP64, _lib.KERNEL_THREAD, 48, 0)  # not a multiple of 32
    with pytest.raises(RuntimeError):
        autotune._set(10, _lib.PREC_FP64, _lib.KERNEL_THREAD, 64, 0)  # stream count not built


def test_corrupt_table_reads_as_empty(tmp_path):
    path = os.path.join(tmp_path, "schedules.json")
    with open(path, "w") as f:
        f.write("{not json")
    assert autotune.load_table(path) == {}

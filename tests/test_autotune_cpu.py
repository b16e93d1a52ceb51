"""Host logic of the schedule autotuner (aeroapps_gb300/autotune.py): the
per-device cache and its installation through aerort_set_schedule /
aerort_set_kernel.  The timing loop itself needs a GPU and runs in bench.py."""
import ctypes
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


def test_cache_round_trip_and_install(tmp_path, restore_defaults):
    path = os.path.join(tmp_path, "schedules.json")
    assert autotune.load_cache(path) == {}
    cache = {
        autotune._key("GB300", 8, _lib.PREC_MIXED): {"kernel": _lib.KERNEL_TEAM, "threads": 64, "blocks_per_sm": 2},
        autotune._key("GB300", 4, _lib.PREC_FP64): {"kernel": _lib.KERNEL_THREAD, "threads": 128,
                                                    "blocks_per_sm": 0},
        autotune._key("other GPU", 12, _lib.PREC_FP64): {"kernel": _lib.KERNEL_THREAD, "threads": 32,
                                                         "blocks_per_sm": 1},
    }
    autotune.save_cache(cache, path)
    assert autotune.load_cache(path) == cache
    assert autotune.apply_cached("GB300", path) == 2  # the other device's entry is not installed
    L = _lib.lib()
    t, b = ctypes.c_int(), ctypes.c_int()
    assert L.aerort_get_schedule(8, _lib.PREC_MIXED, ctypes.byref(t), ctypes.byref(b)) == 0
    assert (t.value, b.value) == (64, 2)
    assert L.aerort_get_kernel(8, _lib.PREC_MIXED) == _lib.KERNEL_TEAM
    assert L.aerort_get_schedule(4, _lib.PREC_FP64, ctypes.byref(t), ctypes.byref(b)) == 0
    assert (t.value, b.value) == (128, 0)
    assert L.aerort_get_kernel(4, _lib.PREC_FP64) == _lib.KERNEL_THREAD


def test_invalid_schedule_is_refused(restore_defaults):
    with pytest.raises(RuntimeError):
        autotune.apply(8, _lib.PREC_FP64, 48, 0)  # not a multiple of 32
    with pytest.raises(RuntimeError):
        autotune.apply(10, _lib.PREC_FP64, 64, 0)  # stream count not built


def test_corrupt_cache_reads_as_empty(tmp_path):
    path = os.path.join(tmp_path, "schedules.json")
    with open(path, "w") as f:
        f.write("{not json")
    assert autotune.load_cache(path) == {}

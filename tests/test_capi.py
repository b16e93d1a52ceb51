"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/aerort.h (no GPU needed: nothing is called that touches CUDA)."""
import ctypes
import os
import re

from aeroapps_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "aerort.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(aerort_\w+)\s*\(", src)))


def test_library_builds_and_exports_header_symbols():
    path = build.build()
    assert os.path.exists(path)
    h = ctypes.CDLL(path)
    names = _declared()
    assert "aerort_vlidort_scalar_lambert" in names and "aerort_get_aop_vector" in names
    missing = [n for n in names if not hasattr(h, n)]
    assert not missing, missing


def test_version_and_error_string_without_gpu():
    L = _lib.lib()
    assert L.aerort_version() >= 10
    assert isinstance(L.aerort_last_error(), bytes)


def test_argument_checks_return_reference_rc_codes():
    # VLIDORT_Init limits (VLIDORT_Mod.F90:365-374) are checked before any CUDA call
    L = _lib.lib()
    null = None
    rc = L.aerort_vlidort_scalar_lambert(80, 1, 1, null, 8, 0, 16, 1, *([null] * 13), -1e15, 0, null, null)
    assert rc == 3  # NLAYERS > MAXLAYERS
    rc = L.aerort_vlidort_scalar_lambert(72, 1, 1, null, 30, 0, 16, 1, *([null] * 13), -1e15, 0, null, null)
    assert rc == 2  # NSTREAMS > MAXSTREAMS
    rc = L.aerort_vlidort_scalar_lambert(72, 1, 1, null, 8, 0, 2000, 1, *([null] * 13), -1e15, 0, null, null)
    assert rc == 5  # nmom > MAXMOMENTS_INPUT


def test_solve_count_beyond_work_counter_range_is_rejected_on_the_host():
    # nobs * nch past the int work counter's headroom (2^30 x 4 would also wrap
    # the 32-bit product to 0): every RT entry point returns AERORT_RC_ARG
    # before any CUDA call (the dummy addresses are never dereferenced)
    L = _lib.lib()
    fake = ctypes.c_void_p(256)
    for nobs, nch in ((1 << 30, 4), (0x7f000000 // 2 + 1, 2)):
        rc = L.aerort_vlidort_scalar_lambert_batch_dev(72, nch, nobs, 8, 0, 16, None, fake, fake, fake, fake, fake,
                                                       None, None, None, fake, fake, fake, fake, fake, -1e15, fake,
                                                       fake, None, None, None)
        assert rc == 1002 and "too large" in _lib.last_error()
        rc = L.aerort_vlidort_scalar_lambert_mixed_batch_dev(72, nch, nobs, 8, 0, 16, None, fake, fake, fake, fake,
                                                             fake, None, None, None, fake, fake, fake, fake, fake,
                                                             -1e15, fake, fake, None, None, None)
        assert rc == 1002 and "too large" in _lib.last_error()
    # the largest accepted count still passes the check (then fails on the null outputs, not the size)
    rc = L.aerort_vlidort_scalar_lambert(72, 1, 1, None, 8, 0, 16, 1, *([None] * 13), -1e15, 0, None, None)
    assert rc == 1002 and "too large" not in _lib.last_error()


def test_ctypes_signatures_match_header_argument_counts():
    # every signature the Python package binds has the argument count of the
    # C prototype in include/aerort.h (a miscount shifts every later argument)
    src = open(os.path.join(ROOT, "include", "aerort.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = {}
    for name, args in re.findall(r"\b(aerort_\w+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        protos[name] = 0 if args.strip() in ("", "void") else args.count(",") + 1
    for name, (_, argtypes) in _lib._SIGNATURES.items():
        if name in protos:
            assert len(argtypes) == protos[name], (name, len(argtypes), protos[name])
    assert "aerort_vlidort_vector_lambert_ex" in protos

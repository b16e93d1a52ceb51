"""aerort_vlidort_scalar_lambert_batch_dev_noalloc: the allocation-free form
of the batched device entry point (static device arena instead of library-
allocated scratch) must give the results of aerort_vlidort_scalar_lambert_batch_dev
on the same inputs, on consecutive calls.  Collected last so it also runs
after every other test has used the allocating entry points."""
import ctypes

import numpy as np
import pytest

from aeroapps_gb300 import _lib

from rt_cases import MISSING, random_aop_case

RTOL = 1e-9


def test_rejects_oversized_batch_before_touching_the_device():
    # nobs * nch beyond the work-counter range: rejected on the host, before
    # any CUDA call (the dummy addresses are never dereferenced)
    L = _lib.lib()
    fake = ctypes.c_void_p(256)
    rc = L.aerort_vlidort_scalar_lambert_batch_dev_noalloc(72, 4, 1 << 30, 8, 0, 16, None, fake, fake, fake, fake,
                                                           fake, None, None, None, fake, fake, fake, fake, fake,
                                                           MISSING, fake, fake, None, None, None)
    assert rc == 1002
    assert "too large" in _lib.last_error()


def _device_case(c, nl, fp32_optics):
    import torch
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    keys = ("ROT", "depol", "he", "albedo", "sza", "raa", "vza")
    arrs = {k: d(c[k], np.float64) for k in keys}
    opt = np.float32 if fp32_optics else np.float64
    arrs["tau"], arrs["ssa"] = d(c["tau"], opt), d(c["ssa"], opt)
    arrs["pmom"] = d(c["pmom"][..., 0], opt)
    arrs["nlay"] = d(nl, np.int32)
    arrs["fp32"] = fp32_optics
    return arrs


def _run(fn, c, N, a, out, stream, plane_parallel):
    km, nch, nobs = c["km"], c["nch"], c["ncol"]
    rad, refl, nf, st = out
    opt = [a["tau"].data_ptr(), a["ssa"].data_ptr(), a["pmom"].data_ptr()]
    f64, f32 = (None, None, None), tuple(opt)
    if not a["fp32"]:
        f64, f32 = tuple(opt), (None, None, None)
    rc = fn(km, nch, nobs, N, plane_parallel, c["nmom"], a["nlay"].data_ptr(), a["ROT"].data_ptr(),
            a["depol"].data_ptr(), *f64, *f32, a["he"].data_ptr(), a["albedo"].data_ptr(), a["sza"].data_ptr(),
            a["raa"].data_ptr(), a["vza"].data_ptr(), MISSING, rad.data_ptr(), refl.data_ptr(), nf.data_ptr(),
            st.data_ptr(), stream)
    assert rc == 0, _lib.last_error()


# (8, 72, 700): two-pass team solve (the arena holds the slice); (16, 72, 300):
# FP64 team scratch at 16 streams is too large for a two-solve-per-warp slice,
# so the fused team kernel runs on a grid capped to the arena; (4, 30, 64):
# thread-per-solve kernel; (8, 40, 500) with FP32 optics straight from the AOP
# kernel and plane_parallel = 1
@pytest.mark.gpu
@pytest.mark.parametrize("N,km,nobs,fp32_optics,pp", [(8, 72, 700, False, 0), (16, 72, 300, False, 0),
                                                      (4, 30, 64, False, 0), (8, 40, 500, True, 1)])
def test_noalloc_matches_allocating_entry_point(N, km, nobs, fp32_optics, pp):
    import torch
    c = random_aop_case(N, km, nobs=nobs, nch=2, seed=4000 + N)
    nl = np.random.default_rng(N).integers(1, km + 1, nobs)
    nl[0] = km
    a = _device_case(c, nl, fp32_optics)
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    n = nobs * c["nch"]

    def outputs():
        return (torch.full((n,), float("nan"), dtype=torch.float64, device="cuda"),
                torch.full((n,), float("nan"), dtype=torch.float64, device="cuda"),
                torch.full((n,), -7, dtype=torch.int32, device="cuda"),
                torch.full((n,), -7, dtype=torch.int32, device="cuda"))

    ref = outputs()
    _run(L.aerort_vlidort_scalar_lambert_batch_dev, c, N, a, ref, stream, pp)
    got = []
    for _ in range(2):  # two calls in a row reuse the same static arena
        o = outputs()
        _run(L.aerort_vlidort_scalar_lambert_batch_dev_noalloc, c, N, a, o, stream, pp)
        got.append(o)
    torch.cuda.synchronize()
    rrad, rrefl, rnf, rst = [t.cpu().numpy() for t in ref]
    assert np.all(np.isfinite(rrad)) and np.all(rst == 0)
    for o in got:
        rad, refl, nf, st = [t.cpu().numpy() for t in o]
        assert np.array_equal(nf, rnf) and np.array_equal(st, rst)
        assert np.all(np.isfinite(rad)) and np.all(np.isfinite(refl))
        ok = rrad != MISSING
        assert np.array_equal(rad == MISSING, ~ok)
        assert np.max(np.abs(rad[ok] / rrad[ok] - 1.0)) <= RTOL
        assert np.max(np.abs(refl[ok] / rrefl[ok] - 1.0)) <= RTOL

"""Batched entry points on several CUDA streams at once (the library keeps one
scratch pad per caller stream, up to 8, and hands a pad to a new stream only
after the device has finished with it), the automatic kernel choice on a large
batch, a team-kernel batch larger than one set-up slice, and empty batches.
Bar: results bitwise identical to the same solves run alone on one stream;
the two kernels within 1e-12 (FP64) of each other."""
import numpy as np
import pytest

from aeroapps_gb300 import _lib

from rt_cases import MISSING, random_aop_case

CH = 2


def _device_case(torch, N, ncol, seed, km=48):
    c = random_aop_case(N, km, nobs=ncol, nch=CH, seed=seed)
    d = lambda a, dt=np.float64: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    t = {k: d(c[k]) for k in ("ROT", "depol", "tau", "ssa", "he", "albedo", "sza", "raa", "vza")}
    t["pmom"] = d(c["pmom"][..., 0])
    n = ncol * CH
    out = {"rad": torch.zeros(n, dtype=torch.float64, device="cuda"),
           "refl": torch.zeros(n, dtype=torch.float64, device="cuda"),
           "nf": torch.zeros(n, dtype=torch.int32, device="cuda"),
           "st": torch.zeros(n, dtype=torch.int32, device="cuda")}
    return c, t, out


def _launch(L, c, t, out, N, stream, precision):
    fn = (L.aerort_vlidort_scalar_lambert_mixed_batch_dev if precision == _lib.PREC_MIXED
          else L.aerort_vlidort_scalar_lambert_batch_dev)
    P = lambda x: x.data_ptr()
    return fn(c["km"], CH, c["ncol"], N, 0, c["nmom"], None, P(t["ROT"]), P(t["depol"]), P(t["tau"]), P(t["ssa"]),
              P(t["pmom"]), None, None, None, P(t["he"]), P(t["albedo"]), P(t["sza"]), P(t["raa"]), P(t["vza"]),
              MISSING, P(out["rad"]), P(out["refl"]), P(out["nf"]), P(out["st"]), stream)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_concurrent_streams_match_serial_runs(precision):
    import torch
    L = _lib.lib()
    cases = [(N, _device_case(torch, N, 40, seed=70 + i)) for i, N in enumerate((4, 8, 12, 16, 6))]
    # serial reference on the current stream
    ref = []
    s0 = torch.cuda.current_stream().cuda_stream
    for N, (c, t, out) in cases:
        assert _launch(L, c, t, out, N, s0, precision) == 0, _lib.last_error()
        torch.cuda.synchronize()
        ref.append({k: v.clone() for k, v in out.items()})
        for v in out.values():
            v.zero_()
    # the same five launches enqueued back to back on five streams
    streams = [torch.cuda.Stream() for _ in cases]
    for s in streams:
        s.wait_stream(torch.cuda.current_stream())
    for (N, (c, t, out)), s in zip(cases, streams):
        assert _launch(L, c, t, out, N, s.cuda_stream, precision) == 0, _lib.last_error()
    torch.cuda.synchronize()
    for (N, (c, t, out)), r in zip(cases, ref):
        for k in out:
            assert torch.equal(out[k], r[k]), (N, k)


@pytest.mark.gpu
def test_more_streams_than_scratch_pads():
    # 19 streams over 16 pads: the least recently used pad changes hands, and
    # the new stream waits on the device for the old stream's work
    import torch
    L = _lib.lib()
    N = 8
    c, t, out = _device_case(torch, N, 24, seed=5)
    s0 = torch.cuda.current_stream().cuda_stream
    assert _launch(L, c, t, out, N, s0, _lib.PREC_FP64) == 0
    torch.cuda.synchronize()
    ref = out["rad"].clone()
    outs = []
    streams = [torch.cuda.Stream() for _ in range(19)]
    for s in streams:
        o = {k: torch.zeros_like(v) for k, v in out.items()}
        assert _launch(L, c, t, o, N, s.cuda_stream, _lib.PREC_FP64) == 0, _lib.last_error()
        outs.append(o)
    torch.cuda.synchronize()
    for o in outs:
        assert torch.equal(o["rad"], ref)


@pytest.mark.gpu
def test_automatic_kernel_choice_on_a_large_batch():
    # 4-stream FP64 batch large enough for the thread kernel (>= 2 warps of 32
    # solves per SM): the automatic choice agrees with the team kernel
    import torch
    L = _lib.lib()
    N = 4
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    ncol = (2 * 32 * sms) // CH + 64
    c, t, out = _device_case(torch, N, ncol, seed=11, km=24)
    s0 = torch.cuda.current_stream().cuda_stream
    assert L.aerort_get_kernel(N, _lib.PREC_FP64) == _lib.KERNEL_AUTO
    assert _launch(L, c, t, out, N, s0, _lib.PREC_FP64) == 0
    torch.cuda.synchronize()
    auto = out["rad"].cpu().numpy()
    assert L.aerort_set_kernel(N, _lib.PREC_FP64, _lib.KERNEL_TEAM) == 0
    try:
        assert _launch(L, c, t, out, N, s0, _lib.PREC_FP64) == 0
        torch.cuda.synchronize()
    finally:
        L.aerort_set_kernel(N, _lib.PREC_FP64, _lib.KERNEL_AUTO)
    team = out["rad"].cpu().numpy()
    ok = team != MISSING
    assert np.array_equal(ok, auto != MISSING)
    assert np.max(np.abs(auto[ok] / team[ok] - 1.0)) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_empty_batch(precision):
    import torch
    L = _lib.lib()
    c, t, out = _device_case(torch, 8, 4, seed=3)
    c = dict(c)
    c["ncol"] = 0
    assert _launch(L, c, t, out, 8, torch.cuda.current_stream().cuda_stream, precision) == 0
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_team_kernel_batch_larger_than_one_setup_slice():
    # more solves than the two-pass team path sets up at once (2^17): the second
    # slice must give the same results as the thread kernel does for it
    import torch
    L = _lib.lib()
    N = 4
    ncol = (1 << 17) // CH + 4000
    c, t, out = _device_case(torch, N, ncol, seed=21, km=20)
    s0 = torch.cuda.current_stream().cuda_stream
    res = {}
    for kern in (_lib.KERNEL_TEAM, _lib.KERNEL_THREAD):
        assert L.aerort_set_kernel(N, _lib.PREC_FP64, kern) == 0
        try:
            assert _launch(L, c, t, out, N, s0, _lib.PREC_FP64) == 0, _lib.last_error()
            torch.cuda.synchronize()
        finally:
            L.aerort_set_kernel(N, _lib.PREC_FP64, _lib.KERNEL_AUTO)
        res[kern] = {k: v.cpu().numpy().copy() for k, v in out.items()}
    a, b = res[_lib.KERNEL_TEAM], res[_lib.KERNEL_THREAD]
    assert np.array_equal(a["st"], b["st"]) and np.array_equal(a["nf"], b["nf"])
    ok = b["rad"] != MISSING
    assert ok.sum() > (1 << 17)
    assert np.max(np.abs(a["rad"][ok] / b["rad"][ok] - 1.0)) <= 1e-12

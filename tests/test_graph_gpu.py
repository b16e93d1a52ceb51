"""CUDA-graph replay of a batched RT step (the form bench.py times): a mixed
and an FP64 batched launch on two streams captured in one CUDA graph and
replayed must give bit for bit the radiances, reflectances, Fourier counts
and status codes of the same launches enqueued eagerly.  Each solve's result
depends on its own inputs only, whichever warp runs it, so replay order and
scheduling cannot change a bit."""
import numpy as np
import pytest

from aeroapps_gb300 import _lib

from rt_cases import MISSING, random_aop_case


def _dev(torch, c, nl):
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    a = {k: d(c[k], np.float64) for k in ("ROT", "depol", "he", "albedo", "sza", "raa", "vza")}
    for k in ("tau", "ssa"):
        a[k] = d(c[k], np.float32)
    a["pmom"] = d(c["pmom"][..., 0], np.float32)
    a["nlay"] = d(nl, np.int32)
    return a


@pytest.mark.gpu
@pytest.mark.parametrize("N", [6, 12])
def test_graph_replay_is_bitwise_eager(N):
    import torch
    L = _lib.lib()
    c = random_aop_case(N, 60, nobs=300, nch=2, seed=900 + N)
    nl = np.random.default_rng(N).integers(20, 61, c["ncol"])
    a = _dev(torch, c, nl)
    n = c["ncol"] * c["nch"]
    P = lambda t: t.data_ptr()

    def outs():
        return [torch.full((n,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(2)] + \
               [torch.full((n,), -7, dtype=torch.int32, device="cuda") for _ in range(2)]

    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    fns = [L.aerort_vlidort_scalar_lambert_mixed_batch_dev, L.aerort_vlidort_scalar_lambert_batch_dev]

    def step(o):
        main = torch.cuda.current_stream()
        for fn, s, oo in zip(fns, streams, o):
            s.wait_stream(main)
            with torch.cuda.stream(s):
                rc = fn(c["km"], c["nch"], c["ncol"], N, 0, c["nmom"], P(a["nlay"]), P(a["ROT"]), P(a["depol"]),
                        None, None, None, P(a["tau"]), P(a["ssa"]), P(a["pmom"]), P(a["he"]), P(a["albedo"]),
                        P(a["sza"]), P(a["raa"]), P(a["vza"]), MISSING, P(oo[0]), P(oo[1]), P(oo[2]), P(oo[3]),
                        s.cuda_stream)
                assert rc == 0, _lib.last_error()
        for s in streams:
            main.wait_stream(s)

    eager = [outs(), outs()]
    step(eager)
    torch.cuda.synchronize()
    rep = [outs(), outs()]
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="thread_local"):
        step(rep)
    for _ in range(2):  # replayed twice: the second replay overwrites the first with the same bits
        g.replay()
    torch.cuda.synchronize()
    for e, r in zip(eager, rep):
        for te, tr in zip(e, r):
            assert torch.equal(te, tr)
    assert np.all(eager[0][3].cpu().numpy() == 0) and np.all(np.isfinite(eager[1][0].cpu().numpy()))

"""Serving loop: admission by device memory (host logic, CPU) and continuous
batching on the GPU -- every request gives the same result alone and in the
mix, and matches the oracle."""
import numpy as np
import pytest

from aeroapps_gb300 import serve


def test_admission_by_memory():
    GB = 1 << 30
    assert serve.can_admit(10 * GB, 100 * GB, 120 * GB, 50 * GB, 2 * GB)
    assert not serve.can_admit(30 * GB, 100 * GB, 120 * GB, 50 * GB, 2 * GB)   # over the budget
    assert not serve.can_admit(10 * GB, 0, 120 * GB, 11 * GB, 2 * GB)          # over free memory
    assert serve.can_admit(9 * GB, 0, 120 * GB, 11 * GB, 2 * GB)


def test_request_bytes_counts_every_group():
    sw = serve.make_swath(0, 40, [550.0, 865.0], seed=3)
    b = serve.request_bytes(sw, 1, 0)
    # at least the FP32 optics of every column
    nl, ns = sw.cols["nlayers"], sw.nstreams
    lower = sum(int(nl[ns == N].max()) * int((ns == N).sum()) * 2 * (3 + 2 * N) * 4
                for N in serve.STREAMS if (ns == N).any())
    assert b >= lower


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_results_identical_alone_and_in_the_mix(precision):
    from aeroapps_gb300 import mie
    chans = [470.0, 550.0, 670.0, 865.0]
    tabs = mie.generate_tables(chans, nmom=32)
    sizes = [64, 200, 90, 150, 64, 120]
    mk = lambda: [serve.make_swath(i, n, chans[: 1 + i % 4], seed=100 + i) for i, n in enumerate(sizes)]
    # alone: one slot, one request at a time
    srv = serve.Server(tabs, nslots=1, precision=precision, hbm_budget_gb=8)
    alone = []
    for sw in mk():
        srv.submit(sw)
        srv.drain()
        alone.append(sw)
    srv.close()
    # in the mix: three slots, all requests queued together
    srv = serve.Server(tabs, nslots=3, precision=precision, hbm_budget_gb=8)
    mix = mk()
    for sw in mix:
        srv.submit(sw)
    srv.drain()
    srv.close()
    for a, b in zip(alone, mix):
        assert np.all(a.status == 0) and np.all(b.status == 0)
        assert np.array_equal(a.nfourier, b.nfourier)
        assert np.array_equal(a.radiance, b.radiance)
    # overlap happened: some request was admitted before an earlier one completed
    mix.sort(key=lambda s: s.t_admit)
    assert any(mix[i + 1].t_admit < mix[i].t_done for i in range(len(mix) - 1))


@pytest.mark.gpu
def test_served_results_match_oracle():
    from aeroapps_gb300 import mie, synth
    from oracle import oracle
    chans = [550.0, 865.0]
    tabs = mie.generate_tables(chans, nmom=32)
    sw = serve.make_swath(0, 48, chans, seed=7)
    srv = serve.Server(tabs, nslots=2, precision="fp64", hbm_budget_gb=8)
    srv.submit(sw)
    srv.drain()
    srv.close()
    qidx = {}
    for ti, t in enumerate(tabs.tables):
        for b in range(t.bext.shape[2]):
            qidx["%s%03d" % (t.name, b + 1)] = (ti, b)
    qt, qb = zip(*[qidx[n] for n in synth.tracer_names()])
    for N in serve.STREAMS:
        idx = np.nonzero(sw.nstreams == N)[0]
        if len(idx) == 0:
            continue
        g = serve._group(sw.cols, idx)
        km, n = g["km"], g["ncol"]
        tau, ssa, gg, pm, rc = oracle.get_aop_vector(tabs, km, n, 2, 20, np.float32(chans), qt, qb, g["qm"], g["rh"],
                                                     2 * N, 1)
        pe = np.zeros((km + 1, n)); te = np.zeros((km + 1, n))
        orad, _, _, onf, ost = oracle.scalar_lambert(km, 2, n, np.array(chans), N, 0, 2 * N, 1, g["ROT"], g["depol"],
                                                     tau, ssa, gg, pm, pe, g["he"], te, g["albedo"], g["sza"],
                                                     g["raa"], g["vza"], serve.MISSING, nlay=g["nlayers"])
        assert np.max(np.abs(sw.radiance[idx] / orad - 1.0)) < 1e-9

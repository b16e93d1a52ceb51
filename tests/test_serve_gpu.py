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


def test_merge_group_over_the_union_of_wavelengths():
    # two requests with different wavelength sets merged into one launch per
    # stream count: each column's unrequested wavelengths get a MISSING
    # albedo, its requested ones its own inputs; the scatter of a launch's
    # outputs hands every request exactly its (column, wavelength) entries
    a = serve.make_swath(0, 30, [550.0, 865.0], seed=1)
    b = serve.make_swath(1, 25, [470.0, 550.0, 670.0], seed=2)
    chans = sorted({*a.channels, *b.channels})
    seen = {0: [], 1: []}
    outs = []
    for N in serve.STREAMS:
        g = serve.merge_group([a, b], N, chans)
        if g is None:
            continue
        n, nch = g["n"], len(chans)
        assert g["ROT"].shape == (g["km"], n, nch) and g["albedo"].shape == (n, nch)
        code = np.zeros((n, nch))
        for sw, idx, r, pos in g["rows"]:
            seen[sw.rid].extend(idx.tolist())
            assert np.all(g["nlayers"][r] == sw.cols["nlayers"][idx])
            for j, p in enumerate(pos):
                assert np.array_equal(g["albedo"][r, p], sw.cols["albedo"][idx, j])
                assert g["depol"][p] == sw.cols["depol"][j]
                km_c = int(sw.cols["nlayers"][idx].max())
                assert np.array_equal(g["ROT"][:km_c, r, p], sw.cols["ROT"][:km_c, idx, j])
            others = [p for p in range(nch) if p not in pos]
            assert np.all(g["albedo"][np.ix_(r, others)] == serve.MISSING)
            # a distinct value per (request, column, wavelength) as the launch output
            for j, p in enumerate(pos):
                code[r, p] = 1000.0 * sw.rid + 10.0 * idx + chans.index(sw.channels[j]) * 0.1
        import torch
        host = [torch.from_numpy(np.asfortranarray(x).ravel(order="F")) for x in
                (code, 2 * code, np.zeros((n, nch), np.int32), np.zeros((n, nch), np.int32))]
        outs.append((g["rows"], host, n, nch))
    assert sorted(seen[0]) == list(range(30)) and sorted(seen[1]) == list(range(25))
    serve.Server._finish([a, b], outs)
    for sw in (a, b):
        want = np.array([[1000.0 * sw.rid + 10.0 * i + chans.index(c) * 0.1 for c in sw.channels]
                         for i in range(sw.ncol)])
        assert np.array_equal(sw.radiance, want) and np.array_equal(sw.reflectance, 2 * want)


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

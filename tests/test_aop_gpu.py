"""GPU parity of aerort_get_aop_vector against the FP32 oracle: bit-identical."""
import numpy as np
import pytest

from aeroapps_gb300 import mie, synth
from oracle import oracle


@pytest.fixture(scope="module")
def tables():
    return mie.generate_tables([470.0, 550.0, 670.0, 865.0], nmom=32)


def _run_both(tables, cols, channels, nmom, npol=1):
    chem = mie.ChemMie(tables)
    names = synth.tracer_names()
    km, n = cols["km"], cols["ncol"]
    ch = np.asarray(channels, np.float32)
    got = mie.get_aop_vector(chem, km, n, len(ch), len(names), ch, names, 0, cols["qm"], cols["rh"], nmom, npol)
    qt, qb = zip(*[chem.query_idx(x) for x in names])
    want = oracle.get_aop_vector(tables, km, n, len(ch), len(names), ch, qt, qb, cols["qm"], cols["rh"], nmom, npol)
    chem.destroy()
    return got, want


@pytest.mark.gpu
def test_bit_identical(tables):
    cols = synth.make_columns(64, [470.0, 550.0, 670.0, 865.0], seed=20261204)
    rh = cols["rh"]
    rh[0, :8] = [-0.2, 0.0, 0.001, 0.0283, 0.5, 0.99, 0.995, 1.3]
    got, want = _run_both(tables, cols, [470.0, 550.0, 670.0, 865.0], 32)
    assert got[4] == 0 and want[4] == 0
    for a, b in zip(got[:4], want[:4]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.gpu
def test_subset_of_channels_and_zero_load(tables):
    cols = synth.make_columns(8, [550.0], seed=3)
    cols["qm"][:, :, 2] = 0.0
    got, want = _run_both(tables, cols, [550.0], 16)
    for a, b in zip(got[:4], want[:4]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.gpu
def test_rc_codes(tables):
    cols = synth.make_columns(2, [550.0], seed=4)
    chem = mie.ChemMie(tables)
    names = synth.tracer_names()
    a = lambda ch, nm, npol: mie.get_aop_vector(chem, cols["km"], 2, 1, 20, np.float32(ch), names, 0, cols["qm"],
                                                cols["rh"], nm, npol)[4]
    assert a([555.0], 8, 1) == 99
    assert a([550.0], 64, 1) == 666
    assert a([550.0], 8, 2) == 777
    chem.destroy()


@pytest.mark.gpu
def test_aop_scalar_equals_vector_without_moments(tables):
    # VLIDORT_getAOPscalar: tau, ssa, g of the vector routine, no moments and no 666/777 checks
    cols = synth.make_columns(40, [470.0, 550.0, 670.0, 865.0], seed=61)
    chem = mie.ChemMie(tables)
    names = synth.tracer_names()
    km, n = cols["km"], cols["ncol"]
    ch = np.asarray([550.0, 865.0], np.float32)
    sc = mie.get_aop_scalar(chem, km, n, 2, len(names), ch, names, 0, cols["qm"], cols["rh"])
    vec = mie.get_aop_vector(chem, km, n, 2, len(names), ch, names, 0, cols["qm"], cols["rh"], 8, 1)
    miss = mie.get_aop_scalar(chem, km, n, 1, len(names), np.float32([551.5]), names, 0, cols["qm"], cols["rh"])
    chem.destroy()
    assert sc[3] == 0 and vec[4] == 0 and miss[3] == 99
    for a, b in zip(sc[:3], vec[:3]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))

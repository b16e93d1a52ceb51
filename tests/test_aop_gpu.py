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


@pytest.fixture(scope="module")
def tables6():
    return mie.generate_tables([470.0, 550.0, 670.0, 865.0], nmom=40, npol=6)


@pytest.mark.gpu
@pytest.mark.parametrize("npol,nmom", [(6, 40), (6, 7), (3, 20), (1, 33)])
def test_bit_identical_six_element_tables(tables6, npol, nmom):
    # moment counts below, at and past one 16-moment chunk of the kernel
    cols = synth.make_columns(24, [470.0, 550.0, 670.0, 865.0], seed=77 + nmom)
    got, want = _run_both(tables6, cols, [470.0, 670.0, 865.0], nmom, npol)
    assert got[4] == 0 and want[4] == 0
    for a, b in zip(got[:4], want[:4]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.gpu
def test_bit_identical_six_elements_with_four_element_tables(tables6):
    # spherical species carry four elements (P11, P12, P33, P34); under
    # nPol = 6 the reference sets P22 and P44 to the running P11 and P33 sums
    # after each such tracer (VLIDORT_MieMod.F90:305-310), so the order of
    # four- and six-element tracers shows in the result.  The six-element
    # tables here get P22 != P11 and P44 != P33 (as non-spherical tables
    # have; Lorenz-Mie tables have them equal), and the last species is one
    # of them.
    tabs = []
    for j, t in enumerate(tables6.tables):
        if j % 2:
            pm = np.asfortranarray(t.pmom[..., :4])
        else:
            pm = np.array(t.pmom, order="F")
            pm[..., 4] *= np.float32(0.9)
            pm[..., 5] *= np.float32(0.8)
        tabs.append(mie.MieTable(t.name, t.rh, t.bext, t.bsca, t.g, pm))
    mixed = mie.MieTableSet(tables6.channels_m, tabs)
    cols = synth.make_columns(24, [470.0, 550.0, 670.0, 865.0], seed=91)
    got, want = _run_both(mixed, cols, [550.0, 865.0], 24, 6)
    assert got[4] == 0 and want[4] == 0
    for a, b in zip(got[:4], want[:4]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    p = got[3]
    assert not np.array_equal(p[..., 4], p[..., 0]) and not np.array_equal(p[..., 5], p[..., 2])


@pytest.mark.gpu
@pytest.mark.parametrize("npol", [1, 6])
def test_bit_identical_forty_tracers(tables6, npol):
    # 40 tracers: the staged kernel's shared rows fit for nPol = 1; for
    # nPol = 6 (two moment rows per tracer) they do not and the gathering
    # kernel runs -- both paths give the oracle's bits
    cols = synth.make_columns(16, [470.0, 550.0, 670.0, 865.0], seed=123 + npol)
    names = synth.tracer_names()
    names2 = names + names[::-1]
    qm = np.asfortranarray(np.concatenate([cols["qm"], np.float32(0.5) * cols["qm"][:, ::-1, :]], axis=1))
    chem = mie.ChemMie(tables6)
    km, n = cols["km"], cols["ncol"]
    ch = np.float32([550.0, 865.0])
    got = mie.get_aop_vector(chem, km, n, 2, len(names2), ch, names2, 0, qm, cols["rh"], 24, npol)
    qt, qb = zip(*[chem.query_idx(x) for x in names2])
    want = oracle.get_aop_vector(tables6, km, n, 2, len(names2), ch, qt, qb, qm, cols["rh"], 24, npol)
    chem.destroy()
    assert got[4] == 0 and want[4] == 0
    for a, b in zip(got[:4], want[:4]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))

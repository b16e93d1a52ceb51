"""Mie table ingest: the netCDF read and wavelength interpolation of
Chem_MieTableRead (src/Shared/GMAO_Shared/Chem_Base/Chem_MieTableMod.F90:238-719,
polint :671-717) and the tracer hash of Chem_MieCreate / Chem_MieQueryIdx
(Chem_MieMod.F90:345-399, 720-777).

CPU: the C oracle against an independent numpy restatement of polint, bit for
bit; the library's aerort_mie_table_interp (host code) against the oracle, bit
for bit, on tables read back from netCDF classic files written here (netCDF-4
files: test_nc4.py); the
edge cases the reference has (channels at, between, below and above the table
wavelengths, a one-wavelength table, too many moments requested).
GPU: AOP vectors from tables read from files, bit-identical to the oracle's.
Parity unpinned: the reference keeps no interpolated tables and its optics
files are not part of the tree."""
import ctypes
import os

import numpy as np
import pytest

from aeroapps_gb300 import _lib, mie, synth
from oracle import oracle

LAM_NM = np.array([250.0, 300.0, 350.0, 400.0, 470.0, 550.0, 670.0, 865.0, 1020.0, 1640.0])
# at a node, between nodes, below the first, above the last, and exactly the last
CH_NM = np.array([550.0, 388.0, 200.0, 2130.0, 1640.0, 354.0, 865.0])


def _np_polint(x, y, xw):
    """polint in numpy: x (n,) and y (n, ...) REAL*8, xw REAL*4."""
    n = len(x)
    xw64 = np.float64(xw)
    i = 0
    if xw64 < x[0]:
        i = 1
    if xw64 > x[-1]:
        i = n
    if i == 0:
        i = int(np.nonzero(xw64 >= x)[0].max()) + 1
    if i == n:
        slope = np.zeros(y.shape[1:], np.float32)
    else:
        slope = ((y[i] - y[i - 1]) / (x[i] - x[i - 1])).astype(np.float32)
    dx = np.float32(xw64 - x[i - 1])
    return (y[i - 1] + (slope * dx).astype(np.float64)).astype(np.float32)


def _raw_table(seed, nlam=len(LAM_NM), nrh=6, nbin=4, nmom=9, npol=2):
    r = np.random.default_rng(seed)
    lam = LAM_NM[:nlam] * 1e-9
    rh = np.concatenate([[0.0], np.sort(r.uniform(0.05, 0.99, nrh - 1))])
    ext = r.uniform(0.5e3, 8e3, (nlam, nrh, nbin)) * (lam[:, None, None] / 550e-9) ** -1.3
    bsca = ext * r.uniform(0.85, 1.0, ext.shape)
    g = r.uniform(0.55, 0.8, ext.shape)
    pmom = r.uniform(-1.0, 1.0, (nlam, nrh, nbin, nmom, npol)) / (1.0 + np.arange(nmom))[None, None, None, :, None]
    pmom[:, :, :, 0, 0] = 1.0
    return dict(lam=lam, rh=rh, bext=ext, bsca=bsca, g=g, pmom=pmom)


def _write_nc(path, t, reverse_dims=False):
    """A GEOS-style optics file (netCDF classic).  Fortran writers declare the
    dimensions slowest first, so the C-order data are (nPol, nMom, radius, rh,
    lambda); reverse_dims declares them the other way round."""
    from scipy.io import netcdf_file
    nlam, nrh, nbin, nmom, npol = t["pmom"].shape
    with netcdf_file(path, "w") as nc:
        for d, n in (("lambda", nlam), ("rh", nrh), ("radius", nbin), ("nMom", nmom), ("nPol", npol)):
            nc.createDimension(d, n)
        nc.createVariable("lambda", "d", ("lambda",))[:] = t["lam"]
        nc.createVariable("rh", "d", ("rh",))[:] = t["rh"]
        for name, dims in (("bext", ("lambda", "rh", "radius")), ("bsca", ("lambda", "rh", "radius")),
                           ("g", ("lambda", "rh", "radius")), ("pmom", ("lambda", "rh", "radius", "nMom", "nPol"))):
            a = t[name]
            if reverse_dims:
                nc.createVariable(name, "d", dims)[:] = a
            else:
                nc.createVariable(name, "d", dims[::-1])[:] = np.transpose(a)


def test_oracle_polint_matches_numpy_restatement_bitwise():
    t = _raw_table(1)
    ch = (CH_NM * 1e-9).astype(np.float32)
    rh, bext, bsca, g, pmom, warns = oracle.mie_table_interp(t["lam"], t["rh"], t["bext"], t["bsca"], t["g"],
                                                             t["pmom"], ch, 5)
    for n, c in enumerate(ch):
        assert np.array_equal(bext[:, n, :], _np_polint(t["lam"], t["bext"], c))
        assert np.array_equal(g[:, n, :], _np_polint(t["lam"], t["g"], c))
        assert np.array_equal(pmom[:, n], _np_polint(t["lam"], t["pmom"][:, :, :, :5, :], c))
    assert np.array_equal(rh, t["rh"].astype(np.float32))
    # one warning per polint call outside the range: 200 nm below, 2130 nm
    # above, and 1640 nm, whose REAL*4 value lies just above the REAL*8 node
    nout = sum(1 for c in ch if np.float64(c) < t["lam"][0] or np.float64(c) > t["lam"][-1])
    assert nout == 3
    nrh, nbin, npol = 6, 4, 2
    assert warns == nout * nrh * nbin * (3 + 5 * npol)


def test_polint_edges():
    x = np.array([1.0, 2.0, 4.0])
    y = np.array([10.0, 20.0, 0.0])
    f = lambda xw: _np_polint(x, y[:, None], np.float32(xw))[0]
    assert f(2.0) == 20.0 and f(4.0) == 0.0 and f(1.0) == 10.0
    assert f(3.0) == 10.0
    assert f(0.5) == 5.0       # below the range: the first segment extrapolated
    assert f(9.0) == 0.0       # above the range: the last value held
    out = ctypes.c_float()
    for xw in (0.5, 1.0, 3.0, 9.0):
        oracle.lib().oracle_mie_polint(x.ctypes.data_as(oracle.P_d), y.ctypes.data_as(oracle.P_d), 3,
                                       ctypes.c_float(xw), ctypes.byref(out))
        assert out.value == f(xw)


@pytest.mark.parametrize("reverse_dims", [False, True])
def test_library_interpolation_of_netcdf_file_bit_identical_to_oracle(tmp_path, reverse_dims):
    t = _raw_table(7)
    path = os.path.join(tmp_path, "optics_XX.nc")
    _write_nc(path, t, reverse_dims)
    a = mie.read_optics_file(path)
    for k in ("bext", "bsca", "g", "pmom"):
        assert np.array_equal(a[k], t[k])
    ch = (CH_NM * 1e-9).astype(np.float32)
    tab, nout = mie.table_from_file_arrays("xx", a["lambda"], a["rh"], a["bext"], a["bsca"], a["g"], a["pmom"], ch, 6)
    want = oracle.mie_table_interp(t["lam"], t["rh"], t["bext"], t["bsca"], t["g"], t["pmom"], ch, 6)
    assert nout == 3
    for got, w in zip((tab.rh, tab.bext, tab.bsca, tab.g, tab.pmom), want[:5]):
        assert got.shape == w.shape
        assert np.array_equal(got.view(np.uint32), w.view(np.uint32))


def test_one_wavelength_table_and_moment_checks():
    t = _raw_table(3, nlam=1, nmom=4)
    ch = np.array([300e-9, 250e-9, 200e-9], np.float32)
    tab, nout = mie.table_from_file_arrays("xx", t["lam"], t["rh"], t["bext"], t["bsca"], t["g"], t["pmom"], ch, 4)
    for n in range(3):  # every channel takes the single wavelength's values
        assert np.array_equal(tab.bext[:, n, :], t["bext"][0].astype(np.float32))
    # 300 and 200 nm lie outside [250, 250] nm, and so may the REAL*4 250 nm
    assert nout == sum(1 for c in ch if np.float64(c) != t["lam"][0])
    with pytest.raises(RuntimeError, match="rc=99"):
        mie.table_from_file_arrays("xx", t["lam"], t["rh"], t["bext"], t["bsca"], t["g"], t["pmom"], ch, 5)
    L = _lib.lib()
    z = np.zeros(64)
    zf = np.zeros(64, np.float32)
    nan = np.array([np.nan], np.float32)
    P = lambda a: a.ctypes.data_as(_lib.P_d if a.dtype == np.float64 else _lib.P_f)
    assert L.aerort_mie_table_interp(1, P(z), 1, P(z), 1, 0, 1, P(z), P(z), P(z), None, 1, P(nan), 0, P(zf), P(zf),
                                     P(zf), P(zf), None, None) == 1002
    assert L.aerort_mie_table_interp(0, P(z), 1, P(z), 1, 0, 1, P(z), P(z), P(z), None, 1, P(zf), 0, P(zf), P(zf),
                                     P(zf), P(zf), None, None) == 1002


def test_get_mie_dims(tmp_path):
    t = _raw_table(11, nlam=7, nrh=5, nbin=3, nmom=10, npol=4)
    path = os.path.join(tmp_path, "optics_dims.nc")
    _write_nc(path, t)
    assert mie.get_mie_dims(path) == (7, 5, 3, 10, 4, 0)
    # a table without phase moments: nMom = nPol = 0
    from scipy.io import netcdf_file
    path2 = os.path.join(tmp_path, "optics_nomom.nc")
    with netcdf_file(path2, "w") as nc:
        for d, n in (("lambda", 2), ("rh", 3), ("radius", 1)):
            nc.createDimension(d, n)
    assert mie.get_mie_dims(path2) == (2, 3, 1, 0, 0, 0)
    assert mie.get_mie_dims(os.path.join(tmp_path, "missing.nc"))[-1] != 0


def _write_rc(tmp_path, nmom=12, channels="4.70e-7 5.50d-7 6.70E-07"):
    for k, sp in enumerate(mie.RC_SPECIES):
        _write_nc(os.path.join(tmp_path, "optics_%s.nc" % sp.upper()), _raw_table(200 + k, nbin=4, nmom=24, npol=1))
    rc = os.path.join(tmp_path, "Aod_test.rc")
    with open(rc, "w") as f:
        f.write("# Mie resource file\n")
        f.write("n_channels: 3\n")
        f.write("n_moments: %d   # phase-function moments\n" % nmom)
        f.write("r_channels: %s\n" % channels)
        for sp in mie.RC_SPECIES:
            f.write("filename_optical_properties_%s: optics_%s.nc\n" % (sp.upper(), sp.upper()))
    return rc


def test_mie_resource_file(tmp_path):
    rc = _write_rc(tmp_path)
    r = mie.read_mie_rc(rc)
    assert r["nch"] == 3 and r["nmom"] == 12
    assert np.array_equal(r["channels_m"], np.array([4.70e-7, 5.50e-7, 6.70e-7], np.float32))
    assert r["files"]["brc"] == os.path.join(tmp_path, "optics_BRC.nc")  # not in the working directory
    # a table path that exists relative to the working directory is taken from there
    sub = os.path.join(tmp_path, "run")
    os.makedirs(sub)
    cwd = os.getcwd()
    try:
        os.chdir(sub)
        with open("optics_DU.nc", "w") as f:
            f.write("")
        assert mie.read_mie_rc(rc)["files"]["du"] == os.path.join(sub, "optics_DU.nc")
    finally:
        os.chdir(cwd)
    ts = mie.tables_from_rc(rc)
    assert [t.name for t in ts.tables] == list(mie.RC_SPECIES)
    ref = mie.read_tables(r["files"], None, 12, channels_m=r["channels_m"])
    for a, b in zip(ts.tables, ref.tables):
        assert np.array_equal(a.pmom, b.pmom) and a.pmom.shape == (6, 3, 4, 12, 1)
    # without n_moments the tables carry no moments
    with open(rc) as f:
        text = f.read()
    with open(rc, "w") as f:
        f.write("\n".join(l for l in text.splitlines() if not l.startswith("n_moments")) + "\n")
    assert mie.tables_from_rc(rc).tables[0].pmom.shape[3] == 0
    with open(rc, "w") as f:
        f.write("n_channels: 2\nr_channels: 5.5e-7\n")
    with pytest.raises(ValueError):
        mie.read_mie_rc(rc)


def test_chem_registry_names(tmp_path):
    path = os.path.join(tmp_path, "Chem_MieRegistry.rc")
    with open(path, "w") as f:
        f.write("""doing_DU:  yes  # dust
doing_SS:  no
doing_SU:  Yes
doing_BC:  yes
doing_NI:  yes
nbins_DU:   3
nbins_SS:   5
nbins_SU:   4
nbins_BC:   2
nbins_NI:   3
variable_table_SU::
DMS        kg/kg    Dimethylsulphide
SO2        kg/kg    Sulphur dioxide
SO4        kg/kg    Sulphate aerosol
MSA        kg/kg    Methanesulphonic acid
::
variable_table_BC::
BCphobic   kg/kg    Hydrophobic Black Carbon
BCphilic   kg/kg    Hydrophilic Black Carbon
::
variable_table_NI::
NH3        kg/kg    Ammonia
NO3an1     kg/kg    Nitrate size bin 001
NO3an2     kg/kg    Nitrate size bin 002
::
""")
    groups = mie.read_chem_registry(path)
    assert groups == {"du": ["du001", "du002", "du003"], "su": ["DMS", "SO2", "SO4", "MSA"],
                      "bc": ["BCphobic", "BCphilic"], "ni": ["NH3", "NO3an1", "NO3an2"]}
    reg = mie.registry_map(groups, list(mie.RC_SPECIES))
    assert reg["DU003"] == (0, 2) and reg["SO4"] == (2, 0) and reg["BCPHILIC"] == (4, 1)
    assert reg["NO3AN2"] == (5, 1) and "NH3" not in reg and "DMS" not in reg


def test_registry_map_and_query_idx():
    groups = {"du": ["du001", "du002", "du003"], "su": ["DMS", "SO2", "SO4", "MSA", "sulf2"],
              "ni": ["NH3", "NO3an1", "no3an2"], "bc": ["BCphobic", "BCphilic"]}
    tables = ["du", "su", "bc", "ni"]
    reg = mie.registry_map(groups, tables)
    assert reg["DU002"] == (0, 1)
    assert reg["SO4"] == (1, 0) and reg["SULF2"] == (1, 1)
    assert "DMS" not in reg and "MSA" not in reg and "NH3" not in reg
    assert reg["NO3AN1"] == (3, 0) and reg["NO3AN2"] == (3, 1)
    assert reg["BCPHILIC"] == (2, 1)
    # query_idx without a device table: the lookup itself is host code
    chem = object.__new__(mie.ChemMie)
    chem.tableset, chem.registry, chem.handle = None, reg, None
    assert chem.query_idx("GOCART::BCphilic") == (2, 1)
    assert chem.query_idx("so4") == (1, 0)
    assert chem.query_idx("DMS") == (-1, -1)
    chem.registry = None
    chem.tableset = mie.MieTableSet(np.zeros(1, np.float32), [mie.MieTable("du", *[np.zeros((1, 1, 5))] * 4,
                                                                           np.zeros((1, 1, 5, 1, 1)))])
    assert chem.query_idx("GOCART::DU005") == (0, 4)
    assert chem.query_idx("du006") == (-1, -1)


@pytest.mark.gpu
def test_aop_from_netcdf_tables_bit_identical_to_oracle(tmp_path):
    channels = [470.0, 550.0, 670.0]
    files = {}
    for k, (name, *_rest) in enumerate(mie.SPECIES):
        t = _raw_table(100 + k, nbin=4, nmom=24, npol=1)
        files[name] = os.path.join(tmp_path, "optics_%s.nc" % name)
        _write_nc(files[name], t)
    tables = mie.read_tables(files, channels, 16)
    chem = mie.ChemMie(tables)
    cols = synth.make_columns(48, channels, seed=77)
    names = synth.tracer_names()
    km, n = cols["km"], cols["ncol"]
    ch = np.asarray(channels, np.float32)
    got = mie.get_aop_vector(chem, km, n, len(ch), len(names), ch, names, 0, cols["qm"], cols["rh"], 16, 1)
    qt, qb = zip(*[chem.query_idx(x) for x in names])
    chem.destroy()
    want = oracle.get_aop_vector(tables, km, n, len(ch), len(names), ch, qt, qb, cols["qm"], cols["rh"], 16, 1)
    assert got[4] == 0 and want[4] == 0
    for a, b in zip(got[:4], want[:4]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.gpu
def test_chem_mie_from_resource_file(tmp_path):
    rc = _write_rc(tmp_path, nmom=16)
    chem = mie.ChemMie.from_rc(rc)
    cols = synth.make_columns(24, [470.0, 550.0, 670.0], seed=78)
    names = synth.tracer_names()
    km, n = cols["km"], cols["ncol"]
    ch = np.asarray([470.0, 550.0, 670.0], np.float32)
    got = mie.get_aop_vector(chem, km, n, 3, len(names), ch, names, 0, cols["qm"], cols["rh"], 16, 1)
    qt, qb = zip(*[chem.query_idx(x) for x in names])
    tables = chem.tableset
    chem.destroy()
    want = oracle.get_aop_vector(tables, km, n, 3, len(names), ch, qt, qb, cols["qm"], cols["rh"], 16, 1)
    assert got[4] == 0 and want[4] == 0
    for a, b in zip(got[:4], want[:4]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_unsorted_wavelength_grid_follows_polint():
    # polint assumes ascending wavelengths; on any other grid its segment search
    # (the last node at or below the channel) and end rules still decide the
    # result, and the library must follow them exactly
    t = _raw_table(21, nlam=6)
    perm = [0, 2, 1, 3, 5, 4]
    for k in ("bext", "bsca", "g", "pmom"):
        t[k] = np.ascontiguousarray(t[k][perm])
    t["lam"] = t["lam"][perm]
    ch = (np.array([260.0, 320.0, 390.0, 460.0, 500.0, 240.0]) * 1e-9).astype(np.float32)
    tab, _ = mie.table_from_file_arrays("xx", t["lam"], t["rh"], t["bext"], t["bsca"], t["g"], t["pmom"], ch, 9)
    want = oracle.mie_table_interp(t["lam"], t["rh"], t["bext"], t["bsca"], t["g"], t["pmom"], ch, 9)
    for got, w in zip((tab.bext, tab.bsca, tab.g, tab.pmom), want[1:5]):
        assert np.array_equal(got.view(np.uint32), w.view(np.uint32))

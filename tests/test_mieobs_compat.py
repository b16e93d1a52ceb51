"""The f2py-compatible MieObs_ module (aeroapps_gb300/MieObs_.py), called the way
Chem_Base/mieobs.py calls the reference's MieObs_ (MieObs_py.F90).

CPU: tracer-name input forms and getmiedims.  GPU: getaopvector,
getaopscalar and getedgevars against the oracle, with the tables named by a
resource file and the tracer names by a Chem_MieRegistry.rc in the working
directory."""
import os

import numpy as np
import pytest

from aeroapps_gb300 import MieObs_, mie, synth
from oracle import oracle

from test_mie_read import _raw_table, _write_nc, _write_rc


def test_tracer_name_forms():
    padded = ["%-16s" % v for v in ("du001", "SO4", "BCphilic")]
    assert MieObs_._names(padded) == ["du001", "SO4", "BCphilic"]
    chars = np.array([list("%-16s" % v) for v in ("du001", "SO4")])
    assert chars.shape == (2, 16)
    assert MieObs_._names(chars) == ["du001", "SO4"]
    assert MieObs_._names(np.array([[bytes([c]) for c in ("%-16s" % "ss002").encode()]], dtype="S1")) == ["ss002"]


def test_getmiedims(tmp_path):
    path = os.path.join(tmp_path, "optics_DU.nc")
    _write_nc(path, _raw_table(1, nlam=4, nrh=3, nbin=5, nmom=7, npol=6))
    assert MieObs_.getmiedims(path) == (4, 3, 5, 7, 6, 0)


@pytest.mark.gpu
def test_getaop_and_edge_vars_match_oracle(tmp_path, monkeypatch):
    rcfile = _write_rc(tmp_path, nmom=16, channels="4.70e-7 5.50e-7 6.70e-7")
    monkeypatch.chdir(tmp_path)
    with open("Chem_MieRegistry.rc", "w") as f:
        f.write("doing_DU: yes\ndoing_SS: yes\ndoing_SU: yes\ndoing_BC: yes\ndoing_OC: yes\n"
                "nbins_DU: 4\nnbins_SS: 4\nnbins_SU: 4\nnbins_BC: 4\nnbins_OC: 4\n"
                "variable_table_SU::\nDMS kg/kg x\nSO2 kg/kg x\nSO4 kg/kg x\nMSA kg/kg x\n::\n")
    cols = synth.make_columns(16, [470.0, 550.0, 670.0], seed=91)
    names = ["du001", "du002", "du003", "du004", "ss001", "ss002", "ss003", "ss004", "DMS", "SO2", "SO4", "MSA",
             "bc001", "bc002", "bc003", "bc004", "oc001", "oc002", "oc003", "oc004"]
    ch = np.array([470.0, 550.0, 670.0], np.float32)
    tau, ssa, g, pmom, rc = MieObs_.getaopvector(rcfile, ch, ["%-16s" % v for v in names], 0, cols["qm"], cols["rh"],
                                                 16, 1)
    assert rc == 0
    tables = mie.tables_from_rc(rcfile)
    reg = mie.registry_map(mie.read_chem_registry("Chem_MieRegistry.rc"), [t.name for t in tables.tables])
    qt = [reg.get(n.upper(), (-1, -1))[0] for n in names]
    qb = [reg.get(n.upper(), (-1, -1))[1] for n in names]
    assert qt[8] == -1 and qt[10] == 2  # DMS carries no optics, SO4 is the first sulfate bin
    want = oracle.get_aop_vector(tables, cols["km"], cols["ncol"], 3, len(names), ch, qt, qb, cols["qm"],
                                 cols["rh"], 16, 1)
    for a, b in zip((tau, ssa, g, pmom), want[:4]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    st, ss, sg, src = MieObs_.getaopscalar(rcfile, ch, names, 0, cols["qm"], cols["rh"])
    assert src == 0
    for a, b in zip((st, ss, sg), (tau, ssa, g)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    km = cols["km"]
    rho = np.asfortranarray(0.5 * (cols["pe"][1:] + cols["pe"][:-1]) / (287.04 * cols["te"][1:]), np.float32)
    dp = np.asfortranarray(np.diff(cols["pe"], axis=0), np.float32)
    pe, ze, te = MieObs_.getedgevars(rho, dp, 1.0)
    o = oracle.get_edge_vars(rho, dp, 1.0)
    assert pe.shape == (km + 1, 16)
    assert np.array_equal(pe, o[0]) and np.array_equal(ze, o[1])
    for c in list(MieObs_._cache.values()):
        c.destroy()
    MieObs_._cache.clear()

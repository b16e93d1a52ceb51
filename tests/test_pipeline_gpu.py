"""End-to-end Mie -> VLIDORT chain on the GPU (geo_vlidort.F90:558-620) against
the oracle chain, on a slice of the 1,024-column / 72-layer / 8-stream / 550 nm case."""
import numpy as np
import pytest

from aeroapps_gb300 import mie, pipeline, synth
from oracle import oracle

MISSING = -1.0e15


@pytest.mark.gpu
def test_config0_slice_matches_oracle():
    channels = [550.0]
    tabs = mie.generate_tables(channels, nmom=16)
    chem = mie.ChemMie(tabs)
    cols = synth.make_columns(48, channels, seed=20261203)
    rad, refl, rc, nf, st = pipeline.toa_radiance(chem, cols, 8, diagnostics=True)
    names = synth.tracer_names()
    qt, qb = zip(*[chem.query_idx(x) for x in names])
    tau, ssa, g, pm, orc = oracle.get_aop_vector(tabs, cols["km"], 48, 1, 20, np.float32(channels), qt, qb, cols["qm"],
                                                 cols["rh"], 16, 1)
    orad, orefl, orc2, onf, ost = oracle.scalar_lambert(cols["km"], 1, 48, cols["channels"], 8, 0, 16, 1, cols["ROT"],
                                                        cols["depol"], tau, ssa, g, pm, cols["pe"], cols["he"],
                                                        cols["te"], cols["albedo"], cols["sza"], cols["raa"],
                                                        cols["vza"], -1.0e15)
    chem.destroy()
    assert rc == 0 and orc == 0 and orc2 == 0
    assert np.array_equal(nf, onf) and np.array_equal(st, ost)
    assert np.max(np.abs(rad / orad - 1)) < 1e-9
    assert np.max(np.abs(refl / orefl - 1)) < 1e-9


def _model_fields(ncol, seed):
    """Layer fields of the kind geo_vlidort reads (AIRDENS, DELP, RH, tracer
    mixing ratios) for synthetic 72-layer columns, and their qm."""
    c = synth.make_columns(ncol, [470.0, 550.0, 670.0], seed=seed)
    pm = 0.5 * (c["pe"][1:] + c["pe"][:-1])
    tm = 0.5 * (c["te"][1:] + c["te"][:-1])
    airdens = np.asfortranarray(pm / (synth.RGAS * tm), np.float32)
    delp = np.asfortranarray(np.diff(c["pe"], axis=0), np.float32)
    return c, airdens, delp


@pytest.mark.gpu
def test_geo_chunk_matches_oracle_chain():
    # the whole per-pixel chain from model fields, against the oracle running
    # the same chain; te may differ by a few ulp (logf/powf), which moves ROT
    # and the radiance by a few 1e-7 at most, hence the 1e-6 bar here
    tabs = mie.generate_tables([470.0, 550.0, 670.0], nmom=32)
    chem = mie.ChemMie(tabs)
    c, airdens, delp = _model_fields(12, seed=33)
    names = synth.tracer_names()
    ch = np.array([470.0, 550.0, 670.0])
    rad, refl, rc, prof = pipeline.geo_chunk(chem, ch, 8, airdens, delp, 1.0, c["qm"], c["rh"], names, c["albedo"],
                                             c["sza"], c["raa"], c["vza"])
    qt, qb = zip(*[chem.query_idx(x) for x in names])
    chem.destroy()
    assert rc == 0
    pe, ze, te = oracle.get_edge_vars(airdens, delp, 1.0)
    assert np.array_equal(prof["pe"], pe) and np.array_equal(prof["ze"], ze)
    f64 = lambda a: np.asfortranarray(a, np.float64)
    rot, depol, _ = oracle.rot_calc(ch, f64(pe), f64(ze), f64(te))
    tau, ssa, g, pmom, orc = oracle.get_aop_vector(tabs, c["km"], 12, 3, len(names), ch.astype(np.float32), qt, qb,
                                                   c["qm"], c["rh"], 16, 1)
    assert orc == 0 and np.array_equal(prof["tau"], tau)
    orad, orefl, orc2, _, _ = oracle.scalar_lambert(c["km"], 3, 12, ch, 8, 0, 16, 1, rot, depol, f64(tau), f64(ssa),
                                                    f64(g), f64(pmom), f64(pe), f64(ze), f64(te), c["albedo"],
                                                    c["sza"], c["raa"], c["vza"], MISSING)
    ok = orad != MISSING
    assert ok.all()
    assert np.max(np.abs(rad / orad - 1.0)) <= 1e-6

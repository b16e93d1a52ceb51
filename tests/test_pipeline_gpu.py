"""End-to-end Mie -> VLIDORT chain on the GPU (geo_vlidort.F90:558-620) against
the oracle chain, on a slice of the 1,024-column / 72-layer / 8-stream / 550 nm case."""
import numpy as np
import pytest

from aeroapps_gb300 import mie, pipeline, synth
from oracle import oracle


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

"""CPU checks of the FP32 Mie/AOP oracle against the reference's rules
(Chem_MieTableMod.F90:612-627, Chem_MieMod.F90:856-945, VLIDORT_MieMod.F90:124-336)."""
import numpy as np

from oracle import oracle
from aeroapps_gb300 import mie


def _tables(nch=2, nrh=6, nmom=4, npol=1, seed=0):
    rng = np.random.default_rng(seed)
    rh = np.linspace(0, 0.99, nrh).astype(np.float32)
    tabs = []
    for s in range(2):
        shp = (nrh, nch, 4)
        bext = np.asfortranarray(rng.uniform(100, 5000, shp).astype(np.float32))
        bsca = np.asfortranarray((bext * rng.uniform(0.5, 1.0, shp)).astype(np.float32))
        g = np.asfortranarray(rng.uniform(0.3, 0.8, shp).astype(np.float32))
        pm = np.asfortranarray(rng.uniform(-1, 3, shp + (nmom, npol)).astype(np.float32))
        tabs.append(mie.MieTable("s%d" % s, rh, bext, bsca, g, pm))
    return mie.MieTableSet(np.array([470e-9, 550e-9][:nch], np.float32), tabs)


def test_rh_map_follows_reference_rule():
    # node i is the largest with (j-1) >= int(rh_i*1000); weight ((j-1)/1000 - rh_i)/(rh_i+1 - rh_i)
    # in REAL*4 (can be slightly negative: the node test truncates, the weight does not)
    rh = np.linspace(0, 0.99, 36).astype(np.float32)
    rhi, rha = oracle.rh_map(rh)
    f = np.float32
    for j in range(991):
        i = max(k for k in range(36) if j >= int(rh[k] * f(1000.0)))
        assert rhi[j] == i + 1
        if i + 1 < 36:
            want = (f(j) / f(1000.0) - rh[i]) / (rh[i + 1] - rh[i])
            assert rha[j] == np.float32(want)
            assert -0.05 < rha[j] < 1.05
        else:
            assert rha[j] == 0.0


def test_aop_rc_codes_and_mixing():
    t = _tables()
    km, nobs, nch, nq = 3, 2, 2, 3
    qm = np.asfortranarray(np.full((km, nq, nobs), 1e-6, np.float32))
    rh = np.asfortranarray(np.array([[-0.5, 0.3], [0.5, 0.995], [0.99, 0.0]], np.float32))
    ch = np.array([470.0, 550.0], np.float32)
    tau, ssa, g, pm, rc = oracle.get_aop_vector(t, km, nobs, nch, nq, ch, [0, 1, -1], [0, 3, 0], qm, rh, 4, 1)
    assert rc == 0
    assert np.all(tau > 0) and np.all((ssa > 0) & (ssa <= 1.0000001))
    # channel not in the table
    assert oracle.get_aop_vector(t, km, nobs, 1, nq, np.array([865.0], np.float32), [0, 1, -1], [0, 0, 0], qm, rh, 4, 1)[4] == 99
    # more moments than the table has
    assert oracle.get_aop_vector(t, km, nobs, nch, nq, ch, [0, 1, -1], [0, 0, 0], qm, rh, 5, 1)[4] == 666
    # more polarisation elements than the table has
    assert oracle.get_aop_vector(t, km, nobs, nch, nq, ch, [0, 1, -1], [0, 0, 0], qm, rh, 4, 2)[4] == 777


def test_aop_single_tracer_is_the_table_lookup():
    t = _tables(nch=1)
    km, nobs = 1, 1
    qm = np.full((1, 1, 1), 2e-5, np.float32, order="F")
    rh = np.full((1, 1), 0.0, np.float32, order="F")
    tau, ssa, g, pm, rc = oracle.get_aop_vector(t, km, nobs, 1, 1, np.array([470.0], np.float32), [0], [2], qm, rh, 4, 1)
    tb = t.tables[0]
    assert rc == 0
    assert tau[0, 0, 0] == np.float32(tb.bext[0, 0, 2] * np.float32(1.0)) * np.float32(2e-5)
    assert ssa[0, 0, 0] == np.float32(tb.bsca[0, 0, 2] / tb.bext[0, 0, 2]) or abs(ssa[0, 0, 0] / (tb.bsca[0, 0, 2] / tb.bext[0, 0, 2]) - 1) < 1e-6

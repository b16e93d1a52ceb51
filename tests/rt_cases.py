"""Shared input builders for the RT parity tests."""
import numpy as np

from aeroapps_gb300 import synth

MISSING = -1.0e15


def random_aop_case(nstreams, km, nobs, nch=2, seed=0, ssa_range=(0.8, 1.0)):
    """Columns from synth (grid, Rayleigh, geometry) with random Henyey-Greenstein-like aerosol optics."""
    rng = np.random.default_rng(seed)
    ch = [470.0, 550.0, 670.0, 865.0][:nch]
    c = synth.make_columns(nobs, ch, seed=seed + 11, nlayers=km)
    nmom = 2 * nstreams
    tau = np.exp(rng.normal(-4.0, 1.5, (km, nch, nobs)))
    ssa = rng.uniform(ssa_range[0], ssa_range[1], (km, nch, nobs))
    g = rng.uniform(0.5, 0.8, (km, nch, nobs))
    pmom = np.zeros((km, nch, nobs, nmom, 1))
    for l in range(nmom):
        pmom[..., l, 0] = (2 * l + 1) * g ** l
    F = np.asfortranarray
    c.update(tau=F(tau), ssa=F(ssa), g=F(g), pmom=F(pmom), nmom=nmom)
    return c


def rt_args(c, nstreams):
    return (c["km"], c["nch"], c["ncol"], c["channels"], nstreams, False, c["nmom"], 1, c["ROT"], c["depol"], c["tau"],
            c["ssa"], c["g"], c["pmom"], c["pe"], c["he"], c["te"], c["albedo"], c["sza"], c["raa"], c["vza"])


def vector_mie_case(nstreams, nobs, nch=2, seed=0, nlayers=72, chem_channels=(470.0, 550.0, 670.0, 865.0),
                    nmom=None):
    """Columns from synth with the six-element Mie optics of the aerosol tracers
    (oracle VLIDORT_getAOPvector with nPol = 6 on synthetic Lorenz-Mie tables):
    the inputs of VLIDORT_Vector_Lambert, FP64 as the reference driver passes them."""
    from aeroapps_gb300 import mie
    from oracle import oracle
    ch = list(chem_channels[:nch])
    c = synth.make_columns(nobs, ch, seed=seed + 11, nlayers=nlayers)
    nmom = nmom or 2 * nstreams
    tabs = mie.generate_tables(ch, nmom=nmom, npol=6)
    qidx = {}
    for ti, t in enumerate(tabs.tables):
        for b in range(t.bext.shape[2]):
            qidx["%s%03d" % (t.name, b + 1)] = (ti, b)
    qt, qb = zip(*[qidx[n] for n in synth.tracer_names()])
    km = c["km"]
    tau, ssa, g, pm, rc = oracle.get_aop_vector(tabs, km, nobs, nch, 20, np.float32(ch), qt, qb, c["qm"], c["rh"],
                                                nmom, 6)
    assert rc == 0
    F = np.asfortranarray
    c.update(tau=F(tau.astype(np.float64)), ssa=F(ssa.astype(np.float64)), g=F(g.astype(np.float64)),
             pmom=F(pm.astype(np.float64)), nmom=nmom, tau32=tau, ssa32=ssa, pmom32=pm, tables=tabs, qt=qt, qb=qb,
             flux=F(np.ones((nch, nobs))))
    return c


def modis_brdf(nobs, nch, seed=0, negative=()):
    """MODIS RTLS kernel amplitudes kernel_wt(3, nch, nobs) = (fiso, fgeo, fvol)
    and Li-sparse parameters param(2, nch, nobs) = (h/b, b/r) = (2, 1) as
    geo_vlidort.F90:543 sets them; `negative` lists (pixel, channel) pairs
    given a strongly negative fgeo (an unphysical combination, BR < 0)."""
    rng = np.random.default_rng(seed)
    kw = np.stack([rng.uniform(0.02, 0.35, (nch, nobs)), rng.uniform(0.0, 0.06, (nch, nobs)),
                   rng.uniform(0.0, 0.15, (nch, nobs))])
    for j, i in negative:
        kw[:, i, j] = (0.01, 5.0, 0.0)
    par = np.stack([np.full((nch, nobs), 2.0), np.full((nch, nobs), 1.0)])
    return np.asfortranarray(kw), np.asfortranarray(par)


def ocean_cx(nobs, nch, seed=0):
    """Cox-Munk ocean surface inputs of VLIDORT_Scalar_CX: wind components
    U10m, V10m (nobs) in m/s and the water refractive index mr (nch)."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(-12.0, 12.0, nobs)
    v = rng.uniform(-12.0, 12.0, nobs)
    mr = np.linspace(1.343, 1.330, nch) if nch > 1 else np.array([1.336])
    return u, v, np.ascontiguousarray(mr)

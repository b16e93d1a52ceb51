"""The AeroApps per-pixel chain on the GPU: Mie optics -> VLIDORT TOA radiance.

Follows geo_vlidort.F90:558-620: VLIDORT_getAOPvector on the layer loads and
RH, conversion of the FP32 optics to FP64, VLIDORT_Scalar_Lambert with the
Rayleigh optical depth, albedo and geometry of each pixel.
"""
import numpy as np

from . import mie as _mie
from . import synth as _synth
from . import vlidort as _vl


def aop_for_columns(chem_mie, cols, nmom, npol=1):
    """VLIDORT_getAOPvector for a synth.make_columns() dict."""
    names = _synth.tracer_names()
    ch32 = np.asarray(cols["channels"], np.float32)
    return _mie.get_aop_vector(chem_mie, cols["km"], cols["ncol"], cols["nch"], len(names), ch32, names, 0,
                               cols["qm"], cols["rh"], nmom, npol)


def toa_radiance(chem_mie, cols, nstreams, nmom=None, diagnostics=False):
    """Radiance/reflectance (nobs, nch) of the columns; nmom defaults to 2*nstreams."""
    nmom = 2 * nstreams if nmom is None else nmom
    tau, ssa, g, pmom, rc = aop_for_columns(chem_mie, cols, nmom)
    if rc != 0:
        raise RuntimeError("get_aop_vector rc=%d" % rc)
    km, nch, nobs = cols["km"], cols["nch"], cols["ncol"]
    return _vl.vlidort_scalar_lambert(km, nch, nobs, cols["channels"], nstreams, False, nmom, 1, cols["ROT"],
                                      cols["depol"], tau.astype(np.float64), ssa.astype(np.float64),
                                      g.astype(np.float64), pmom.astype(np.float64), cols["pe"], cols["he"],
                                      cols["te"], cols["albedo"], cols["sza"], cols["raa"], cols["vza"],
                                      diagnostics=diagnostics)


def geo_chunk(chem_mie, channels, nstreams, airdens, delp, ptop, qm, rh, vname, albedo, sza, raa, vza, nmom=None,
              MISSING=_vl.MISSING, diagnostics=False):
    """The per-pixel sequence of geo_vlidort.F90:499-600 for a block of
    pixels, every step on the GPU:
      getEdgeVars(airdens, delp, ptop)             -> pe, ze, te   (REAL*4)
      VLIDORT_ROT_CALC(dble(pe), dble(ze), dble(te)) -> ROT, depol
      VLIDORT_getAOPvector(qm, rh)                 -> tau, ssa, g, pmom (REAL*4)
      VLIDORT_Scalar_Lambert(dble(tau), ...)       -> radiance, reflectance
    Shapes: airdens, delp, rh (km, nobs); qm (km, nq, nobs) = mixing ratio x
    delp / g (calc_qm, geo_vlidort.F90:2124-2144); albedo (nobs, nch);
    angles (nobs); channels [nm].  Returns (radiance, reflectance, rc), or
    also (nfourier, status) with diagnostics, plus the intermediate
    profiles {"pe", "ze", "te", "ROT", "depol", "tau", "ssa", "g", "pmom"}."""
    airdens = np.asfortranarray(airdens, np.float32)
    km, nobs = airdens.shape
    nq = np.asarray(qm).shape[1]
    ch = np.asarray(channels, np.float64)
    nch = ch.size
    nmom = 2 * nstreams if nmom is None else nmom
    pe, ze, te = _mie.get_edge_vars(km, nobs, airdens, delp, ptop)
    pe64, ze64, te64 = (np.asfortranarray(a, np.float64) for a in (pe, ze, te))
    ROT, depol, rc = _vl.rot_calc(ch, pe64, ze64, te64, MISSING, 0)
    if rc != 0:
        raise RuntimeError("rot_calc rc=%d" % rc)
    tau, ssa, g, pmom, rc = _mie.get_aop_vector(chem_mie, km, nobs, nch, nq, ch.astype(np.float32), vname, 0, qm, rh,
                                                nmom, 1)
    if rc != 0:
        raise RuntimeError("get_aop_vector rc=%d" % rc)
    f64 = lambda a: np.asfortranarray(a, np.float64)
    out = _vl.vlidort_scalar_lambert(km, nch, nobs, ch, nstreams, False, nmom, 1, ROT, depol, f64(tau), f64(ssa),
                                     f64(g), f64(pmom), pe64, ze64, te64, albedo, sza, raa, vza, MISSING=MISSING,
                                     diagnostics=diagnostics)
    prof = {"pe": pe, "ze": ze, "te": te, "ROT": ROT, "depol": depol, "tau": tau, "ssa": ssa, "g": g, "pmom": pmom}
    return out + (prof,)

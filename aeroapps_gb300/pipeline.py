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

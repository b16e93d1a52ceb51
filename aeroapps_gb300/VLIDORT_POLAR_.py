"""Drop-in for the scalar and Rayleigh entries of the f2py module VLIDORT_POLAR_
(src/Components/rtms/leo_vlidort/VLIDORT_POLAR_py.F90), with the work on the GPU.

f2py exposes each subroutine under its lower-cased name and drops the size
arguments it can infer from the arrays (they become optional trailing
keywords), so the Python callers write, e.g.
(leo_vlidort/benchmark_polar_vlidort.py):
  ROT, depol, rc = VLIDORT_POLAR_.rot_calc(channels, pe, he, te, MISSING, verbose)
The same calls work here:
  rot_calc(channels, pe, he, te, MISSING, verbose)           -> (ROT, depol, rc)      (:9-41)
  scalar_lambert(channels, nstreams, plane_parallel, ROT, depol, tau, ssa, g, pmom, pe, he, te, albedo,
                 solar_zenith, relat_azymuth, sensor_zenith, MISSING, verbose)
                                                              -> (radiance, reflectance, rc)  (:606-671)
  vector_lambert(channels, nstreams, plane_parallel, ROT, depol, alpha, tau, ssa, pmom, pe, he, te, albedo,
                 solar_zenith, relat_azymuth, sensor_zenith, flux_factor, MISSING, verbose)
                                                              -> (radiance, reflectance, Q, U, rc)  (:457-526)
Shapes are the Fortran ones: ROT (km, nobs, nch), tau/ssa/g (km, nch, nobs),
pmom (km, nch, nobs, nMom, nPol), pe/he/te (km+1, nobs), albedo (nobs, nch).
The BRDF, BPDF, ocean and cloud entries of the module (VECTOR_BRDF_*,
VECTOR_*CX*, *_CLOUD; :43-455, :528-604, :673-1145) need the BRDF surface
supplement, which this package does not have; they are not defined, so a
call to one fails with AttributeError rather than running something else.
"""
import numpy as np

from . import vlidort


def rot_calc(channels, pe, he, te, MISSING, verbose=0, km=None, nch=None, nobs=None):
    rot, depol, rc = vlidort.rot_calc(channels, pe, he, te, MISSING, verbose)
    if (km is not None and km != rot.shape[0]) or (nobs is not None and nobs != rot.shape[1]) or \
            (nch is not None and nch != rot.shape[2]):
        raise ValueError("rot_calc: explicit sizes disagree with the arrays")
    return rot, depol, rc


def scalar_lambert(channels, nstreams, plane_parallel, ROT, depol, tau, ssa, g, pmom, pe, he, te, albedo,
                   solar_zenith, relat_azymuth, sensor_zenith, MISSING, verbose=0, km=None, nch=None, nobs=None,
                   nmom=None, npol=None):
    tau = np.asarray(tau)
    pmom = np.asarray(pmom)
    if pmom.ndim == 4:
        pmom = pmom[..., None]
    k, c, o = tau.shape
    m, p = pmom.shape[3], pmom.shape[4]
    for given, have, name in ((km, k, "km"), (nch, c, "nch"), (nobs, o, "nobs"), (nmom, m, "nmom"), (npol, p, "npol")):
        if given is not None and given != have:
            raise ValueError("scalar_lambert: %s = %d disagrees with the arrays (%d)" % (name, given, have))
    return vlidort.vlidort_scalar_lambert(k, c, o, channels, int(nstreams), plane_parallel, m, p, ROT, depol, tau,
                                          ssa, g, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth,
                                          sensor_zenith, MISSING, verbose)


def vector_lambert(channels, nstreams, plane_parallel, ROT, depol, alpha, tau, ssa, pmom, pe, he, te, albedo,
                   solar_zenith, relat_azymuth, sensor_zenith, flux_factor, MISSING, verbose=0, km=None, nch=None,
                   nobs=None, nmom=None, npol=None):
    """VECTOR_LAMBERT (VLIDORT_POLAR_py.F90:457-526) -> (radiance, reflectance, Q, U, rc)."""
    tau = np.asarray(tau)
    pmom = np.asarray(pmom)
    k, c, o = tau.shape
    m, p = pmom.shape[3], pmom.shape[4]
    for given, have, name in ((km, k, "km"), (nch, c, "nch"), (nobs, o, "nobs"), (nmom, m, "nmom"), (npol, p, "npol")):
        if given is not None and given != have:
            raise ValueError("vector_lambert: %s = %d disagrees with the arrays (%d)" % (name, given, have))
    return vlidort.vlidort_vector_lambert(k, c, o, channels, int(nstreams), plane_parallel, m, p, ROT, depol, alpha, tau,
                                          ssa, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth, sensor_zenith,
                                          flux_factor, MISSING, verbose)

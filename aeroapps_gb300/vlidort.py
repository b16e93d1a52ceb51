"""VLIDORT_Scalar_Lambert and VLIDORT_Vector_Lambert on the GPU, with the
reference's argument lists.

Mirrors src/Components/rtms/geo_vlidort/VLIDORT_LAMBERT.F90:34-168 (and its
f2py exposure, src/Components/rtms/leo_vlidort/VLIDORT_POLAR_py.F90): every
array has the reference's shape and Fortran order; the return value is
(radiance_VL, reflectance_VL, rc) as the f2py wrapper returns it.
"""
import numpy as np

from . import _lib

MISSING = -1.0e15
STREAMS = (4, 6, 8, 12, 16)


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


def vlidort_scalar_lambert(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g,
                           pmom, pe, he, te, albedo, solar_zenith, relat_azymuth, sensor_zenith, MISSING=MISSING,
                           verbose=0, diagnostics=False):
    """Scalar TOA radiance/reflectance for nobs pixels x nch channels.

    Shapes: channels(nch) [nm], ROT(km,nobs,nch), depol(nch), tau/ssa/g(km,nch,nobs),
    pmom(km,nch,nobs,nMom,nPol), pe/he/te(km+1,nobs), albedo(nobs,nch), angles(nobs).
    With diagnostics=True also returns nfourier(nobs,nch) and status(nobs,nch).
    """
    arrs = [_f64(channels), _f64(ROT), _f64(depol), _f64(tau), _f64(ssa), _f64(g), _f64(pmom), _f64(pe), _f64(he),
            _f64(te), _f64(albedo), _f64(solar_zenith), _f64(relat_azymuth), _f64(sensor_zenith)]
    ch, ROT, depol, tau, ssa, g, pmom, pe, he, te, albedo, sza, raa, vza = arrs
    if ROT.shape != (km, nobs, nch) or tau.shape != (km, nch, nobs) or he.shape != (km + 1, nobs):
        raise ValueError("array shapes do not match (km, nch, nobs) = (%d, %d, %d)" % (km, nch, nobs))
    if pmom.ndim != 5 or pmom.shape[:4] != (km, nch, nobs, nMom):
        raise ValueError("pmom must have shape (km, nch, nobs, nMom, nPol)")
    rad = np.zeros((nobs, nch), np.float64, order="F")
    refl = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    P = lambda a: _lib.ptr(a, _lib.P_d)
    rc = _lib.lib().aerort_vlidort_scalar_lambert_ex(
        km, nch, nobs, P(ch), nstreams, int(bool(plane_parallel)), nMom, nPol, P(ROT), P(depol), P(tau), P(ssa), P(g),
        P(pmom), P(pe), P(he), P(te), P(albedo), P(sza), P(raa), P(vza), float(MISSING), int(verbose), P(rad),
        P(refl), _lib.ptr(nf, _lib.P_i), _lib.ptr(st, _lib.P_i))
    if rc >= 1000:
        raise RuntimeError("aerort_vlidort_scalar_lambert rc=%d: %s" % (rc, _lib.last_error()))
    if diagnostics:
        return rad, refl, rc, nf, st
    return rad, refl, rc


def vlidort_scalar_landmodis(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g,
                             pmom, pe, he, te, kernel_wt, param, solar_zenith, relat_azymuth, sensor_zenith,
                             MISSING=MISSING, verbose=0, diagnostics=False):
    """VLIDORT_Scalar_LandMODIS: scalar TOA radiance/reflectance over the MODIS
    RTLS BRDF (geo_vlidort/VLIDORT_BRDF_MODIS.F90:34-200).

    As vlidort_scalar_lambert with the albedo replaced by kernel_wt(3,nch,nobs)
    (fiso, fgeo, fvol) and param(2,nch,nobs) (Li-sparse h/b, b/r).  Returns
    (radiance, reflectance, BR, rc), plus (nfourier, status) with
    diagnostics=True; BR(nobs,nch) is the exact direct-bounce BRDF (-500 where
    the kernel combination is negative, as the reference)."""
    arrs = [_f64(channels), _f64(ROT), _f64(depol), _f64(tau), _f64(ssa), _f64(g), _f64(pmom), _f64(pe), _f64(he),
            _f64(te), _f64(kernel_wt), _f64(param), _f64(solar_zenith), _f64(relat_azymuth), _f64(sensor_zenith)]
    ch, ROT, depol, tau, ssa, g, pmom, pe, he, te, kw, par, sza, raa, vza = arrs
    if ROT.shape != (km, nobs, nch) or tau.shape != (km, nch, nobs) or he.shape != (km + 1, nobs):
        raise ValueError("array shapes do not match (km, nch, nobs) = (%d, %d, %d)" % (km, nch, nobs))
    if kw.shape != (3, nch, nobs) or par.shape != (2, nch, nobs):
        raise ValueError("kernel_wt must have shape (3, nch, nobs) and param (2, nch, nobs)")
    rad = np.zeros((nobs, nch), np.float64, order="F")
    refl = np.zeros_like(rad)
    br = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    P = lambda a: _lib.ptr(a, _lib.P_d)
    rc = _lib.lib().aerort_vlidort_scalar_landmodis_ex(
        km, nch, nobs, P(ch), nstreams, int(bool(plane_parallel)), nMom, nPol, P(ROT), P(depol), P(tau), P(ssa), P(g),
        P(pmom), P(pe), P(he), P(te), P(kw), P(par), P(sza), P(raa), P(vza), float(MISSING), int(verbose), P(rad),
        P(refl), P(br), _lib.ptr(nf, _lib.P_i), _lib.ptr(st, _lib.P_i))
    if rc >= 1000:
        raise RuntimeError("aerort_vlidort_scalar_landmodis rc=%d: %s" % (rc, _lib.last_error()))
    if diagnostics:
        return rad, refl, br, rc, nf, st
    return rad, refl, br, rc


def vlidort_scalar_cx(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g, pmom,
                      pe, he, te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith, MISSING=MISSING,
                      verbose=0, diagnostics=False, giss=False):
    """VLIDORT_Scalar_CX: scalar TOA radiance/reflectance over the Cox-Munk
    ocean glint (geo_vlidort/VLIDORT_BRDF_CX.F90:420-584); giss=True:
    VLIDORT_Scalar_GissCX (:1553-1716), the GISS Cox-Munk kernel.

    As vlidort_scalar_lambert with the albedo replaced by the 10 m wind
    components U10m, V10m (nobs) and the water refractive index mr (nch).
    Returns (radiance, reflectance, BRDF, rc), plus (nfourier, status) with
    diagnostics=True; BRDF(nobs,nch) is the exact direct-bounce BRDF."""
    arrs = [_f64(channels), _f64(ROT), _f64(depol), _f64(tau), _f64(ssa), _f64(g), _f64(pmom), _f64(pe), _f64(he),
            _f64(te), _f64(U10m), _f64(V10m), _f64(mr), _f64(solar_zenith), _f64(relat_azymuth), _f64(sensor_zenith)]
    ch, ROT, depol, tau, ssa, g, pmom, pe, he, te, u, v, mr, sza, raa, vza = arrs
    if ROT.shape != (km, nobs, nch) or tau.shape != (km, nch, nobs) or he.shape != (km + 1, nobs):
        raise ValueError("array shapes do not match (km, nch, nobs) = (%d, %d, %d)" % (km, nch, nobs))
    if u.shape != (nobs,) or v.shape != (nobs,) or mr.shape != (nch,):
        raise ValueError("U10m, V10m must have shape (nobs,) and mr (nch,)")
    rad = np.zeros((nobs, nch), np.float64, order="F")
    refl = np.zeros_like(rad)
    br = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    P = lambda a: _lib.ptr(a, _lib.P_d)
    fn = _lib.lib().aerort_vlidort_scalar_gisscx_ex if giss else _lib.lib().aerort_vlidort_scalar_cx_ex
    rc = fn(
        km, nch, nobs, P(ch), nstreams, int(bool(plane_parallel)), nMom, nPol, P(ROT), P(depol), P(tau), P(ssa), P(g),
        P(pmom), P(pe), P(he), P(te), P(u), P(v), P(mr), P(sza), P(raa), P(vza), float(MISSING), int(verbose), P(rad),
        P(refl), P(br), _lib.ptr(nf, _lib.P_i), _lib.ptr(st, _lib.P_i))
    if rc >= 1000:
        raise RuntimeError("aerort_vlidort_scalar_%scx rc=%d: %s" % ("giss" if giss else "", rc, _lib.last_error()))
    if diagnostics:
        return rad, refl, br, rc, nf, st
    return rad, refl, br, rc


def vlidort_scalar_lambert_dev(km, nch, nobs, nstreams, nMom, ROT, depol, tau, ssa, pmom, he, albedo, solar_zenith,
                               relat_azymuth, sensor_zenith, radiance, reflectance, nfourier=None, status=None,
                               MISSING=MISSING, plane_parallel=False, stream=0):
    """Device-pointer form: every array argument is a CUDA device address (int)."""
    rc = _lib.lib().aerort_vlidort_scalar_lambert_dev(
        km, nch, nobs, nstreams, int(bool(plane_parallel)), nMom, ROT, depol, tau, ssa, pmom, he, albedo,
        solar_zenith, relat_azymuth, sensor_zenith, float(MISSING), radiance, reflectance, nfourier or 0,
        status or 0, stream)
    if rc != 0:
        raise RuntimeError("aerort_vlidort_scalar_lambert_dev rc=%d: %s" % (rc, _lib.last_error()))
    return rc


def vlidort_scalar_lambert_batch(km, nch, nobs, nstreams, nMom, nlay, ROT, depol, tau, ssa, pmom, he, albedo,
                                 solar_zenith, relat_azymuth, sensor_zenith, MISSING=MISSING, plane_parallel=False,
                                 precision="fp64"):
    """Batched host call for columns of different layer counts (nlay(nobs), each <= km).

    Same arrays as vlidort_scalar_lambert (pmom: the P11 moments, (km,nch,nobs,nMom));
    precision "fp64" (plain method) or "mixed" (FP32 Fourier series);
    returns (radiance, reflectance, rc, nfourier, status)."""
    if precision not in ("fp64", "mixed"):
        raise ValueError("precision must be 'fp64' or 'mixed'")
    ROT, depol, tau, ssa, pmom, he, albedo, sza, raa, vza = [_f64(a) for a in (ROT, depol, tau, ssa, pmom, he, albedo,
                                                                               solar_zenith, relat_azymuth,
                                                                               sensor_zenith)]
    nl = np.ascontiguousarray(nlay, np.int32)
    rad = np.zeros((nobs, nch), np.float64, order="F")
    refl = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    P = lambda a: _lib.ptr(a, _lib.P_d)
    fn = (_lib.lib().aerort_vlidort_scalar_lambert_batch if precision == "fp64"
          else _lib.lib().aerort_vlidort_scalar_lambert_mixed_batch)
    rc = fn(
        km, nch, nobs, nstreams, int(bool(plane_parallel)), nMom, _lib.ptr(nl, _lib.P_i), P(ROT), P(depol), P(tau),
        P(ssa), P(pmom), P(he), P(albedo), P(sza), P(raa), P(vza), float(MISSING), P(rad), P(refl),
        _lib.ptr(nf, _lib.P_i), _lib.ptr(st, _lib.P_i))
    if rc >= 1000:
        raise RuntimeError("aerort_vlidort_scalar_lambert_batch rc=%d: %s" % (rc, _lib.last_error()))
    return rad, refl, rc, nf, st



def vlidort_vector_lambert(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, alpha, tau, ssa,
                           pmom, pe, he, te, albedo, solar_zenith, relat_azymuth, sensor_zenith, flux_factor,
                           MISSING=MISSING, verbose=0, diagnostics=False):
    """VLIDORT_Vector_Lambert (geo_vlidort/VLIDORT_LAMBERT.F90:172-342), NSTOKES = 3.

    Shapes: channels(nch) [nm], ROT/alpha(km,nobs,nch) (alpha may be None),
    tau/ssa(km,nch,nobs), pmom(km,nch,nobs,nMom,6) (P11, P12, P33, P34, P22,
    P44), pe/he/te(km+1,nobs), albedo(nobs,nch), angles(nobs),
    flux_factor(nch,nobs).  Returns (radiance, reflectance, Q, U, rc), plus
    (nfourier, status) with diagnostics=True.
    """
    ch, ROT, depol, tau, ssa, pmom, pe, he, te, albedo, sza, raa, vza, ff = [
        _f64(a) for a in (channels, ROT, depol, tau, ssa, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth,
                          sensor_zenith, flux_factor)]
    al = None if alpha is None else _f64(alpha)
    if ROT.shape != (km, nobs, nch) or tau.shape != (km, nch, nobs) or he.shape != (km + 1, nobs):
        raise ValueError("array shapes do not match (km, nch, nobs) = (%d, %d, %d)" % (km, nch, nobs))
    if pmom.shape != (km, nch, nobs, nMom, nPol) or ff.shape != (nch, nobs):
        raise ValueError("pmom must have shape (km, nch, nobs, nMom, nPol) and flux_factor (nch, nobs)")
    out = [np.zeros((nobs, nch), np.float64, order="F") for _ in range(4)]
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    P = lambda a: None if a is None else _lib.ptr(a, _lib.P_d)
    rc = _lib.lib().aerort_vlidort_vector_lambert_ex(
        km, nch, nobs, P(ch), nstreams, int(bool(plane_parallel)), nMom, nPol, P(ROT), P(depol), P(al), P(tau), P(ssa),
        P(pmom), P(pe), P(he), P(te), P(albedo), P(sza), P(raa), P(vza), P(ff), float(MISSING), int(verbose),
        *[P(a) for a in out], _lib.ptr(nf, _lib.P_i), _lib.ptr(st, _lib.P_i))
    if rc >= 1000:
        raise RuntimeError("aerort_vlidort_vector_lambert rc=%d: %s" % (rc, _lib.last_error()))
    if diagnostics:
        return out[0], out[1], out[2], out[3], rc, nf, st
    return out[0], out[1], out[2], out[3], rc


def rot_calc(channels, pe, he, te, MISSING, verbose=0):
    """f2py-style ROT_CALC (leo_vlidort/VLIDORT_POLAR_py.F90:9-41): pe, he, te
    (km+1, nobs) in Pa, m, K; returns (ROT(km, nobs, nch), depol(nch), rc)."""
    pe, he, te = _f64(pe), _f64(he), _f64(te)
    ch = np.ascontiguousarray(channels, np.float64)
    km, nobs, nch = pe.shape[0] - 1, pe.shape[1], ch.size
    rot = np.zeros((km, nobs, nch), order="F")
    depol = np.zeros(nch)
    L = _lib.lib()
    rc = L.aerort_vlidort_rot_calc(km, nch, nobs, _lib.ptr(ch, _lib.P_d), _lib.ptr(pe, _lib.P_d),
                                   _lib.ptr(he, _lib.P_d), _lib.ptr(te, _lib.P_d), float(MISSING), int(verbose),
                                   _lib.ptr(rot, _lib.P_d), _lib.ptr(depol, _lib.P_d))
    return rot, depol, rc


def vlidort_scalar_gisscx(*args, **kw):
    """VLIDORT_Scalar_GissCX (geo_vlidort/VLIDORT_BRDF_CX.F90:1553-1716): the
    arguments and returns of vlidort_scalar_cx over the GISS Cox-Munk kernel."""
    return vlidort_scalar_cx(*args, giss=True, **kw)

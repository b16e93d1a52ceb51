"""ctypes access to the CPU oracle (test infrastructure only: imported by tests/,
__graft_entry__.smoke() and the cpu_baseline / reference arm of bench.py)."""
import ctypes

import numpy as np

from . import build as _build

_lib = None
P_d = ctypes.POINTER(ctypes.c_double)
P_f = ctypes.POINTER(ctypes.c_float)
P_i = ctypes.POINTER(ctypes.c_int)


class OracleOpts(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("do_focorr", "do_focorr_nadir", "do_focorr_outgoing", "do_deltam",
                                              "do_plane_parallel", "do_double_convtest", "nfinelayers",
                                              "taylor_order")] + \
               [(n, ctypes.c_double) for n in ("accuracy", "asymtx_tol", "earth_radius", "flux_factor")]


class OracleMieTable(ctypes.Structure):
    _fields_ = [("nrh", ctypes.c_int), ("nch", ctypes.c_int), ("nbin", ctypes.c_int), ("nmom", ctypes.c_int),
                ("npol", ctypes.c_int), ("rh", P_f), ("channels", P_f), ("bext", P_f), ("bsca", P_f), ("g", P_f),
                ("pmom", P_f), ("rhi", P_i), ("rha", P_f)]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build())
        _lib.oracle_vlidort_solve.restype = ctypes.c_int
        _lib.oracle_vlidort_solve_brdf.restype = ctypes.c_int
        _lib.oracle_brdf_supplement.restype = ctypes.c_int
        _lib.oracle_vlidort_vector_solve.restype = ctypes.c_int
        _lib.oracle_vector_lambert.restype = ctypes.c_int
        _lib.oracle_scalar_lambert.restype = ctypes.c_int
        _lib.oracle_scalar_landmodis.restype = ctypes.c_int
        _lib.oracle_scalar_cx.restype = ctypes.c_int
        _lib.oracle_scalar_gisscx.restype = ctypes.c_int
        _lib.oracle_get_aop_vector.restype = ctypes.c_int
        _lib.oracle_set_asymtx_tol.restype = None
        _lib.oracle_rot_calc.restype = ctypes.c_int
        _lib.oracle_coef_depol.restype = ctypes.c_double
        _lib.oracle_coef_depol.argtypes = [ctypes.c_double]
    return _lib


def _p(a, kind):
    return a.ctypes.data_as(kind)


def vlidort_solve(opts, heights, deltau, omega, greek, albedo, sza, vzas, raas, nstreams):
    """Single-beam solve (lattice of vzas x raas). greek: (L, ngreek+1). Returns (out[nvza, nraa], nfourier, status)."""
    heights = np.ascontiguousarray(heights, np.float64)
    deltau = np.ascontiguousarray(deltau, np.float64)
    omega = np.ascontiguousarray(omega, np.float64)
    greek = np.ascontiguousarray(greek, np.float64)
    L, g1 = greek.shape
    vz = np.ascontiguousarray(vzas, np.float64)
    ra = np.ascontiguousarray(raas, np.float64)
    out = np.zeros(len(vz) * len(ra))
    nf = ctypes.c_int(0)
    st = lib().oracle_vlidort_solve(ctypes.byref(opts), L, nstreams, g1 - 1, _p(heights, P_d), _p(deltau, P_d),
                                    _p(omega, P_d), _p(greek, P_d), ctypes.c_double(albedo), ctypes.c_double(sza),
                                    len(vz), _p(vz, P_d), len(ra), _p(ra, P_d), _p(out, P_d), ctypes.byref(nf))
    return out.reshape(len(vz), len(ra)), nf.value, st


def brdf_supplement(kernels, nstreams, sza, vzas, raas, nstreams_brdf=50, do_shadow=False, nmom=None):
    """VBRDF supplement for one solar beam (oracle/brdf_oracle.cpp).  kernels:
    [(which, factor, (p1, p2, p3)), ...] with `which` the VLIDORT kernel index
    (1 Lambertian, 2 Ross-thin, 3 Ross-thick, 4 Li-sparse, 5 Li-dense, 9
    Cox-Munk).  Returns dict f (m, i, j), f0 (m, i), uf (m, u, j), uf0 (m, u),
    exactdb (u, a), m = 0..nmom (default 2 nstreams - 1)."""
    nk = len(kernels)
    which = np.array([k[0] for k in kernels], np.int32)
    fac = np.array([k[1] for k in kernels], np.float64)
    pars = np.array([list(k[2]) + [0.0] * (3 - len(k[2])) for k in kernels], np.float64).ravel()
    vz = np.ascontiguousarray(vzas, np.float64)
    ra = np.ascontiguousarray(raas, np.float64)
    N, nu, na = nstreams, len(vz), len(ra)
    nmom = 2 * N - 1 if nmom is None else nmom
    M1 = nmom + 1
    f = np.zeros((M1, N, N)); f0 = np.zeros((M1, N)); uf = np.zeros((M1, nu, N)); uf0 = np.zeros((M1, nu))
    ex = np.zeros((nu, na))
    lib().oracle_brdf_supplement(nk, _p(which, P_i), _p(fac, P_d), _p(pars, P_d), int(do_shadow), nstreams_brdf, N,
                                 nmom, ctypes.c_double(sza), nu, _p(vz, P_d), na, _p(ra, P_d), _p(f, P_d),
                                 _p(f0, P_d), _p(uf, P_d), _p(uf0, P_d), _p(ex, P_d))
    return {"f": f, "f0": f0, "uf": uf, "uf0": uf0, "exactdb": ex}


def vlidort_solve_brdf(opts, heights, deltau, omega, greek, brdf, sza, vzas, raas, nstreams):
    """vlidort_solve with a BRDF surface: `brdf` from brdf_supplement for the
    same beam, user angles and azimuths."""
    heights = np.ascontiguousarray(heights, np.float64)
    deltau = np.ascontiguousarray(deltau, np.float64)
    omega = np.ascontiguousarray(omega, np.float64)
    greek = np.ascontiguousarray(greek, np.float64)
    L, g1 = greek.shape
    vz = np.ascontiguousarray(vzas, np.float64)
    ra = np.ascontiguousarray(raas, np.float64)
    arr = [np.ascontiguousarray(brdf[k], np.float64) for k in ("f", "f0", "uf", "uf0", "exactdb")]
    out = np.zeros(len(vz) * len(ra))
    nf = ctypes.c_int(0)
    st = lib().oracle_vlidort_solve_brdf(ctypes.byref(opts), L, nstreams, g1 - 1, _p(heights, P_d), _p(deltau, P_d),
                                         _p(omega, P_d), _p(greek, P_d), ctypes.c_double(0.0), ctypes.c_double(sza),
                                         len(vz), _p(vz, P_d), len(ra), _p(ra, P_d),
                                         *[_p(a, P_d) for a in arr], _p(out, P_d), ctypes.byref(nf))
    return out.reshape(len(vz), len(ra)), nf.value, st


def vlidort_vector_solve(opts, nstokes, heights, deltau, omega, greek16, albedo, sza, vzas, raas, nstreams):
    """Single-beam polarized solve (lattice of vzas x raas).  greek16: (16, L,
    ngreek+1), entry k of the row-major 4x4 Greek matrix.  Returns (out[nvza,
    nraa, nstokes], nfourier, status)."""
    heights = np.ascontiguousarray(heights, np.float64)
    deltau = np.ascontiguousarray(deltau, np.float64)
    omega = np.ascontiguousarray(omega, np.float64)
    greek = np.ascontiguousarray(greek16, np.float64)
    _, L, g1 = greek.shape
    vz = np.ascontiguousarray(vzas, np.float64)
    ra = np.ascontiguousarray(raas, np.float64)
    out = np.zeros(len(vz) * len(ra) * nstokes)
    nf = ctypes.c_int(0)
    st = lib().oracle_vlidort_vector_solve(ctypes.byref(opts), nstokes, L, nstreams, g1 - 1, _p(heights, P_d),
                                           _p(deltau, P_d), _p(omega, P_d), _p(greek, P_d), ctypes.c_double(albedo),
                                           ctypes.c_double(sza), len(vz), _p(vz, P_d), len(ra), _p(ra, P_d),
                                           _p(out, P_d), ctypes.byref(nf))
    return out.reshape(len(vz), len(ra), nstokes), nf.value, st


def scalar_lambert(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g, pmom, pe, he,
                   te, albedo, solar_zenith, relat_azymuth, sensor_zenith, MISSING, verbose=0, nlay=None):
    """Oracle VLIDORT_Scalar_Lambert; returns (radiance, reflectance, rc, nfourier, status)."""
    F = lambda a: np.asfortranarray(a, np.float64)
    arr = [F(x) for x in (channels, ROT, depol, tau, ssa, g, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth,
                          sensor_zenith)]
    rad = np.zeros((nobs, nch), order="F")
    refl = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    c, rot, dep, ta, ss, gg, pm, p_e, h_e, t_e, al, sz, ra, vz = arr
    rc = lib().oracle_scalar_lambert(km, nch, nobs, _p(c, P_d), nstreams, int(plane_parallel), nMom, nPol, _p(rot, P_d),
                                     _p(dep, P_d), _p(ta, P_d), _p(ss, P_d), _p(gg, P_d), _p(pm, P_d), _p(p_e, P_d),
                                     _p(h_e, P_d), _p(t_e, P_d), _p(al, P_d), _p(sz, P_d), _p(ra, P_d), _p(vz, P_d),
                                     ctypes.c_double(MISSING), int(verbose), _p(rad, P_d), _p(refl, P_d),
                                     _p(nf, P_i), _p(st, P_i),
                                     None if nlay is None else _p(np.ascontiguousarray(nlay, np.int32), P_i))
    return rad, refl, rc, nf, st


def scalar_landmodis(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g, pmom,
                     pe, he, te, kernel_wt, param, solar_zenith, relat_azymuth, sensor_zenith, MISSING, verbose=0,
                     nlay=None):
    """Oracle VLIDORT_Scalar_LandMODIS; kernel_wt (3, nch, nobs), param (2, nch, nobs).
    Returns (radiance, reflectance, BR, rc, nfourier, status)."""
    F = lambda a: np.asfortranarray(a, np.float64)
    arr = [F(x) for x in (channels, ROT, depol, tau, ssa, g, pmom, pe, he, te, kernel_wt, param, solar_zenith,
                          relat_azymuth, sensor_zenith)]
    rad = np.zeros((nobs, nch), order="F")
    refl = np.zeros_like(rad)
    br = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    rc = lib().oracle_scalar_landmodis(km, nch, nobs, _p(arr[0], P_d), nstreams, int(plane_parallel), nMom, nPol,
                                       *[_p(a, P_d) for a in arr[1:]], ctypes.c_double(MISSING), int(verbose),
                                       _p(rad, P_d), _p(refl, P_d), _p(br, P_d), _p(nf, P_i), _p(st, P_i),
                                       None if nlay is None else _p(np.ascontiguousarray(nlay, np.int32), P_i))
    return rad, refl, br, rc, nf, st


def scalar_cx(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol, tau, ssa, g, pmom, pe, he,
              te, U10m, V10m, mr, solar_zenith, relat_azymuth, sensor_zenith, MISSING, verbose=0, nlay=None,
              giss=False):
    """Oracle VLIDORT_Scalar_CX (Cox-Munk glint; giss=True: VLIDORT_Scalar_GissCX,
    the GISS Cox-Munk kernel); U10m, V10m (nobs), mr (nch).
    Returns (radiance, reflectance, BR, rc, nfourier, status)."""
    F = lambda a: np.asfortranarray(a, np.float64)
    arr = [F(x) for x in (channels, ROT, depol, tau, ssa, g, pmom, pe, he, te, U10m, V10m, mr, solar_zenith,
                          relat_azymuth, sensor_zenith)]
    rad = np.zeros((nobs, nch), order="F")
    refl = np.zeros_like(rad)
    br = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    fn = lib().oracle_scalar_gisscx if giss else lib().oracle_scalar_cx
    rc = fn(km, nch, nobs, _p(arr[0], P_d), nstreams, int(plane_parallel), nMom, nPol,
                                *[_p(a, P_d) for a in arr[1:]], ctypes.c_double(MISSING), int(verbose),
                                _p(rad, P_d), _p(refl, P_d), _p(br, P_d), _p(nf, P_i), _p(st, P_i),
                                None if nlay is None else _p(np.ascontiguousarray(nlay, np.int32), P_i))
    return rad, refl, br, rc, nf, st


def vector_lambert(km, nch, nobs, nstreams, plane_parallel, nMom, ROT, depol, alpha, tau, ssa, pmom, he, albedo,
                   solar_zenith, relat_azymuth, sensor_zenith, flux_factor, MISSING, nlay=None):
    """Oracle VLIDORT_Vector_Lambert (NSTOKES = 3); pmom (km, nch, nobs, nMom, 6).
    Returns (radiance, reflectance, Q, U, rc, nfourier, status), each (nobs, nch)."""
    F = lambda a: np.asfortranarray(a, np.float64)
    arr = [F(x) for x in (ROT, depol, tau, ssa, pmom, he, albedo, solar_zenith, relat_azymuth, sensor_zenith)]
    al = None if alpha is None else F(alpha)
    ff = None if flux_factor is None else F(flux_factor)
    out = [np.zeros((nobs, nch), order="F") for _ in range(4)]
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    rot, dep, ta, ss, pm, h_e, alb, sz, ra, vz = arr
    rc = lib().oracle_vector_lambert(km, nch, nobs, nstreams, int(plane_parallel), nMom, _p(rot, P_d), _p(dep, P_d),
                                     None if al is None else _p(al, P_d), _p(ta, P_d), _p(ss, P_d), _p(pm, P_d),
                                     _p(h_e, P_d), _p(alb, P_d), _p(sz, P_d), _p(ra, P_d), _p(vz, P_d),
                                     None if ff is None else _p(ff, P_d), ctypes.c_double(MISSING),
                                     *[_p(a, P_d) for a in out], _p(nf, P_i), _p(st, P_i),
                                     None if nlay is None else _p(np.ascontiguousarray(nlay, np.int32), P_i))
    return out[0], out[1], out[2], out[3], rc, nf, st


def set_threads(n):
    """Threads of the oracle's OpenMP loop over pixels (0: every host core)."""
    lib().oracle_set_threads(int(n))


def set_asymtx_tol(tol):
    """Tolerance of the oracle's ASYMTX in scalar_lambert (reference: 1e-12)."""
    lib().oracle_set_asymtx_tol(ctypes.c_double(tol))


def rh_map(rh):
    rh = np.ascontiguousarray(rh, np.float32)
    rhi = np.zeros(991, np.int32)
    rha = np.zeros(991, np.float32)
    lib().oracle_mie_rhmap(len(rh), _p(rh, P_f), _p(rhi, P_i), _p(rha, P_f))
    return rhi, rha


def mie_table_interp(lam, rh_table, bext, bsca, g, pmom, channels_m, nmom):
    """Chem_MieTableRead's wavelength interpolation (Chem_MieTableMod.F90:575-601).

    Table fields in file order, wavelength first: bext/bsca/g (nlam,nrh,nbin),
    pmom (nlam,nrh,nbin,nmom_table,npol).  Returns (rh, bext, bsca, g, pmom,
    warnings) in Chem_MieTable order, REAL*4."""
    lam = np.ascontiguousarray(lam, np.float64)
    rh_table = np.ascontiguousarray(rh_table, np.float64)
    f = lambda a: np.asfortranarray(a, np.float64)
    bext, bsca, g, pmom = f(bext), f(bsca), f(g), f(pmom)
    ch = np.ascontiguousarray(channels_m, np.float32)
    nlam, nrh, nbin, nmom_table, npol = pmom.shape
    nch = len(ch)
    out = [np.zeros(nrh, np.float32)] + [np.zeros((nrh, nch, nbin), np.float32, order="F") for _ in range(3)]
    opm = np.zeros((nrh, nch, nbin, nmom, npol), np.float32, order="F")
    warns = lib().oracle_mie_table_interp(nlam, _p(lam, P_d), nrh, _p(rh_table, P_d), nbin, nmom_table, npol,
                                          _p(bext, P_d), _p(bsca, P_d), _p(g, P_d), _p(pmom, P_d), nch, _p(ch, P_f),
                                          nmom, *[_p(a, P_f) for a in out], _p(opm, P_f))
    return out[0], out[1], out[2], out[3], opm, warns


def get_aop_vector(tableset, km, nobs, nch, nq, channels_nm, q_table, q_bin, qm, rh, nMom, nPol):
    """Oracle VLIDORT_getAOPvector on a mie.MieTableSet; returns (tau, ssa, g, pmom, rc)."""
    keep = []
    tabs = (OracleMieTable * len(tableset.tables))()
    ch = np.ascontiguousarray(tableset.channels_m, np.float32)
    keep.append(ch)
    for i, t in enumerate(tableset.tables):
        arrs = [np.ascontiguousarray(t.rh, np.float32)] + [np.asfortranarray(x, np.float32) for x in (t.bext, t.bsca, t.g, t.pmom)]
        rhi, rha = rh_map(t.rh)
        keep += arrs + [rhi, rha]
        tabs[i].nrh, tabs[i].nch, tabs[i].nbin = t.bext.shape
        tabs[i].nmom, tabs[i].npol = t.pmom.shape[3], t.pmom.shape[4]
        tabs[i].rh, tabs[i].bext, tabs[i].bsca, tabs[i].g, tabs[i].pmom = [_p(a, P_f) for a in arrs]
        tabs[i].channels = _p(ch, P_f)
        tabs[i].rhi = _p(rhi, P_i)
        tabs[i].rha = _p(rha, P_f)
    cn = np.ascontiguousarray(channels_nm, np.float32)
    qt = np.ascontiguousarray(q_table, np.int32)
    qb = np.ascontiguousarray(q_bin, np.int32)
    qm = np.asfortranarray(qm, np.float32)
    rh = np.asfortranarray(rh, np.float32)
    tau = np.zeros((km, nch, nobs), np.float32, order="F")
    ssa = np.zeros_like(tau)
    g = np.zeros_like(tau)
    pmom = np.zeros((km, nch, nobs, nMom, nPol), np.float32, order="F")
    rc = lib().oracle_get_aop_vector(len(tableset.tables), tabs, km, nobs, nch, nq, _p(cn, P_f), _p(qt, P_i), _p(qb, P_i),
                                     _p(qm, P_f), _p(rh, P_f), nMom, nPol, _p(tau, P_f), _p(ssa, P_f), _p(g, P_f),
                                     _p(pmom, P_f))
    return tau, ssa, g, pmom, rc


def get_edge_vars(airdens, delp, ptop):
    """getEdgeVars (MieObs_py.F90:27-83): (pe, ze, te), each (km+1, nobs), REAL*4."""
    rho = np.asfortranarray(airdens, np.float32)
    dp = np.asfortranarray(delp, np.float32)
    km, nobs = rho.shape
    out = [np.zeros((km + 1, nobs), np.float32, order="F") for _ in range(3)]
    lib().oracle_get_edge_vars(km, nobs, _p(rho, P_f), _p(dp, P_f), ctypes.c_float(ptop), *[_p(a, P_f) for a in out])
    return tuple(out)


def rot_calc(channels, pe, he, te):
    """VLIDORT_ROT_CALC restated (rot_oracle.c): pe, he, te (km+1, nobs) -> ROT (km, nobs, nch), depol (nch), rc."""
    pe, he, te = (np.asfortranarray(a, np.float64) for a in (pe, he, te))
    ch = np.ascontiguousarray(channels, np.float64)
    km, nobs, nch = pe.shape[0] - 1, pe.shape[1], ch.size
    rot = np.zeros((km, nobs, nch), order="F")
    depol = np.zeros(nch)
    rc = lib().oracle_rot_calc(km, nch, nobs, _p(ch, P_d), _p(pe, P_d), _p(he, P_d), _p(te, P_d), _p(rot, P_d),
                               _p(depol, P_d))
    return rot, depol, rc

"""Seeded synthetic columns with the shapes and value distributions of the
benchmark configurations (the reference runs on GEOS model fields, which are
not available here).

Per column: a 72-level hybrid sigma-pressure grid (top 1 Pa), a standard-
atmosphere temperature profile, edge heights from hydrostatic balance (as
getEdgeVars, src/Shared/GMAO_Shared/Chem_Base/MieObs_py.F90:27-83), uniform
relative humidity, lognormal aerosol mass mixing ratios for 5 species x 4 bins
converted to layer loads qm = q dp / g (geo_vlidort.F90:2124-2144), Rayleigh
optical depth 0.0976 dp/ps at 550 nm scaled as lambda^-4.08, King-factor
depolarisation (VLIDORT_ScatMod.F90:249-281), Lambertian albedo and angles.
"""
import numpy as np

GRAV = 9.80616    # MieObs_py.F90:52
RGAS = 287.04
PTOP = 1.0        # Pa
NLEV72 = 72
NTRACER = 20


def hybrid_coefficients(nlev=NLEV72, ptop=PTOP, ps_ref=101325.0):
    """(A, B) of a hybrid sigma-pressure grid: pe = A + B * ps, index 0 = top.

    Upper levels are log-spaced in pressure, the lowest ~25 levels thin out
    towards the surface; B rises smoothly from 0 above 10 kPa to 1 at the
    surface.  Own construction with the GEOS-5 72-level character.
    """
    k = np.arange(nlev + 1, dtype=np.float64)
    n_up = 46
    p_up = ptop * (20000.0 / ptop) ** (k[: n_up + 1] / n_up)
    v = (k[n_up:] - n_up) / (nlev - n_up)
    p_lo = 20000.0 + (ps_ref - 20000.0) * (1.0 - (1.0 - v) ** 1.6)
    p = np.concatenate([p_up, p_lo[1:]])
    pt = 10000.0
    B = np.where(p > pt, ((p - pt) / (ps_ref - pt)) ** 2, 0.0)
    A = p - B * ps_ref
    return A, B


def coef_depol(lam_um):
    """King-factor depolarisation ratio (Bodhaine et al. 1999 air mixture, 360 ppm CO2)."""
    xx2 = 1.0 / (np.asarray(lam_um, np.float64) ** 2)
    c = 360.0e-6
    d1 = 1.034 + 3.17e-4 * xx2
    d2 = 1.096 + 1.385e-3 * xx2 + 1.448e-4 * xx2 * xx2
    f_air = (78.084 * d1 + 20.946 * d2 + 0.934 * 1.0 + c * 100.0 * 1.15) / (78.084 + 20.946 + 0.934 + c * 100.0)
    return 6.0 * (f_air - 1.0) / (7.0 * f_air + 3.0)


def make_columns(ncol, channels_nm, seed, nlayers=72, albedo_max=0.30, sza_max=75.0, vza_max=60.0):
    """Columns for VLIDORT_getAOPvector + VLIDORT_Scalar_Lambert.

    nlayers: int (all columns) or int array (per column, <= 72; the lowest
    nlayers-1 levels are kept and the rest merged into one top layer).  The
    returned arrays are dimensioned with km = max(nlayers); a column with fewer
    layers uses the first nlayers entries (layer index 0 = top).
    """
    rng = np.random.default_rng(seed)
    nl = np.broadcast_to(np.asarray(nlayers, dtype=np.int64), (ncol,)).copy()
    km = int(nl.max())
    nch = len(channels_nm)
    lam = np.asarray(channels_nm, np.float64)
    A, B = hybrid_coefficients()
    ps = rng.uniform(95000.0, 103000.0, ncol)
    full = A[:, None] + B[:, None] * ps[None, :]                 # (73, ncol)
    # column j keeps the top edge and the lowest nl_j edges of the full grid
    k = np.arange(km + 1)[:, None]
    src = np.where(k == 0, 0, NLEV72 - nl[None, :] + k)           # source level of edge k
    src = np.minimum(src, NLEV72)
    pe = np.take_along_axis(full, src, axis=0)
    pe = np.where(k <= nl[None, :], pe, pe[np.minimum(nl, km)[None, :], np.arange(ncol)[None, :]])
    te = np.maximum(216.65, 288.15 * (pe / 101325.0) ** 0.1903)
    # heights: dz = dp / (rho g) accumulated upward from the surface (getEdgeVars)
    pm = 0.5 * (pe[1:] + pe[:-1])
    tm = 0.5 * (te[1:] + te[:-1])
    dz = (pe[1:] - pe[:-1]) / (pm / (RGAS * tm) * GRAV)            # zero in padded layers
    he = np.zeros((km + 1, ncol))
    he[:-1] = np.cumsum(dz[::-1], axis=0)[::-1]
    dp = np.diff(pe, axis=0)  # (km, ncol), zero in padded layers
    rh = rng.uniform(0.0, 0.99, (km, ncol)).astype(np.float32)
    q = np.exp(rng.normal(-20.0, 1.5, (km, NTRACER, ncol)))
    qm = (q * dp[:, None, :] / GRAV).astype(np.float32)
    rot = np.zeros((km, ncol, nch))
    for i in range(nch):
        rot[:, :, i] = 0.0976 * (550.0 / lam[i]) ** 4.08 * dp / ps[None, :]
    depol = coef_depol(lam * 1e-3)
    albedo = rng.uniform(0.02, albedo_max, (ncol, nch))
    sza = rng.uniform(0.0, sza_max, ncol)
    vza = rng.uniform(0.0, vza_max, ncol)
    raa = rng.uniform(0.0, 180.0, ncol)
    F = np.asfortranarray
    return {
        "km": km, "nch": nch, "ncol": ncol, "nlayers": nl, "channels": lam,
        "pe": F(pe), "he": F(he), "te": F(te), "rh": F(rh), "qm": F(qm), "ROT": F(rot), "depol": depol,
        "albedo": F(albedo), "sza": sza, "vza": vza, "raa": raa,
    }


def tracer_names():
    from .mie import SPECIES, NBIN
    return ["%s%03d" % (s[0], b + 1) for s in SPECIES for b in range(NBIN)]

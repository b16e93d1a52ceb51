"""Seeded synthetic columns with the shapes and value distributions of the
benchmark configurations (the reference runs on GEOS model fields, which are
not available here).

Per column: the GEOS-5 72-level hybrid sigma-pressure grid (top 1 Pa), a standard-
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


# GEOS-5 72-level hybrid sigma-pressure coefficients, edge 1 = model top:
# pe_k = A72_k + B72_k * ps, A72 in Pa (A72_1 = ptop = 1 Pa), B72 dimensionless
# (GMAO_hermes/m_set_eta.F90:512-549, the default 72-level branch).  A model
# grid is a data table, reproduced exactly so that the layer thicknesses, and
# with them the Rayleigh and aerosol loads, are the model's.
A72 = np.array([
    1.0000000, 2.0000002, 3.2700005, 4.7585009, 6.6000011, 8.9345014, 11.970302, 15.949503, 21.134903,
    27.852606, 36.504108, 47.580610, 61.677911, 79.513413, 101.94402, 130.05102, 165.07903, 208.49704,
    262.02105, 327.64307, 407.65710, 504.68010, 621.68012, 761.98417, 929.29420, 1127.6902, 1364.3402,
    1645.7103, 1979.1604, 2373.0405, 2836.7806, 3381.0007, 4017.5409, 4764.3911, 5638.7912, 6660.3412,
    7851.2316, 9236.5722, 10866.302, 12783.703, 15039.303, 17693.003, 20119.201, 21686.501, 22436.301,
    22389.800, 21877.598, 21214.998, 20325.898, 19309.696, 18161.897, 16960.896, 15625.996, 14290.995,
    12869.594, 11895.862, 10918.171, 9936.5219, 8909.9925, 7883.4220, 7062.1982, 6436.2637, 5805.3211,
    5169.6110, 4533.9010, 3898.2009, 3257.0809, 2609.2006, 1961.3106, 1313.4804, 659.37527, 4.8048257,
    0.0000000])
B72 = np.array([0.0] * 41 + [
    8.1754130e-09, 0.0069600246, 0.028010041, 0.063720063, 0.11360208, 0.15622409, 0.20035011, 0.24674112,
    0.29440312, 0.34338113, 0.39289115, 0.44374018, 0.49459020, 0.54630418, 0.58104151, 0.61581843,
    0.65063492, 0.68589990, 0.72116594, 0.74937819, 0.77063753, 0.79194696, 0.81330397, 0.83466097,
    0.85601798, 0.87742898, 0.89890800, 0.92038701, 0.94186501, 0.96340602, 0.98495195, 1.0000000])


def hybrid_coefficients(nlev=NLEV72):
    """(A, B) of the GEOS-5 72-level grid: pe = A + B * ps [Pa], index 0 = top."""
    if nlev != NLEV72:
        raise ValueError("only the 72-level GEOS-5 grid is tabulated")
    return A72.copy(), B72.copy()


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

"""Pin the BRDF oracle (oracle/brdf_oracle.cpp and the BRDF surface of
oracle/vlidort_oracle.cpp) to the reference's own saved VLIDORT 2.8.3 BRDF
results.

Fixture tests/golden/brdf_supcheck.json (tests/golden/make_brdf_golden.py):
the VBRDF supplement check of the reference's BRDF-plus tester
(vlidort_v_test/V2p8p3_brdfplus_tester.f90:331-560; kernels Ross-thin 0.3,
Li-dense 0.1, Cox-Munk 0.1 with shadowing; 8 streams, 100 azimuth streams;
lattice 4 SZA x 3 VZA x 3 RAA) -- exact direct-bounce BRDF at 12 digits,
Fourier components at 8 -- and the tester's TOA-upwelling Stokes I over that
surface, on the solar tester's atmosphere (tests/golden/solar_tester_iqu.json),
at 6 digits.
"""
import numpy as np
import pytest

from oracle import oracle


@pytest.fixture(scope="module")
def golden_brdf():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "brdf_supcheck.json")) as f:
        return json.load(f)


def _kernels(g):
    return [(k["which"], k["factor"], k["pars"]) for k in g["kernels"]]


def _supplement(g, ib):
    return oracle.brdf_supplement(_kernels(g), g["nstreams"], g["szas"][ib], g["vzas"], g["raas"],
                                  nstreams_brdf=g["nstreams_brdf"], do_shadow=g["shadow"])


def test_exact_direct_bounce_brdf(golden_brdf):
    g = golden_brdf
    for ib in range(len(g["szas"])):
        b = _supplement(g, ib)
        want = np.array(g["exact"][ib])
        assert np.max(np.abs(b["exactdb"] - want)) <= 2e-11 * np.max(np.abs(want))  # measured: <= 4.8e-12


def test_fourier_components(golden_brdf):
    # every m, quadrature-quadrature, beam-quadrature, user-quadrature and
    # user-beam component, to the saved 8 digits (relative to each array's scale)
    g = golden_brdf
    f = np.array(g["f"])            # (m, i, j)
    f0 = np.array(g["f0"])          # (m, i, beam)
    uf = np.array(g["uf"])          # (m, u, j)
    uf0 = np.array(g["uf0"])        # (m, u, beam)
    for ib in range(len(g["szas"])):
        b = _supplement(g, ib)
        for got, want in ((b["f"], f), (b["f0"], f0[:, :, ib]), (b["uf"], uf), (b["uf0"], uf0[:, :, ib])):
            scale = np.maximum(np.abs(want), 1e-3 * np.abs(want).max())
            assert np.max(np.abs(got - want) / scale) < 1e-6  # measured: 4.1e-8


def test_toa_radiance_over_brdf_surface(golden_brdf, golden_iqu):
    # the brdfplus tester's baseline: FO (regular pseudo-spherical), delta-M,
    # 8 streams, ASYMTX tolerance 1e-20, accuracy 1e-4, on the solar tester's
    # 23-layer atmosphere; every Fourier term summed (the reference's
    # convergence test also spans its downwelling outputs)
    g, a = golden_brdf, golden_iqu
    o = oracle.OracleOpts(do_plane_parallel=0, do_double_convtest=1, taylor_order=a["taylor_order"], accuracy=1e-30,
                          asymtx_tol=a["asymtx_tol"], earth_radius=a["earth_radius"], flux_factor=1.0,
                          **g["rt_options"])
    greek = np.transpose(np.array(a["greek_nstokes1"]), (1, 0, 2))[0]
    err = []
    for ib, s in enumerate(g["szas"]):
        b = _supplement(g, ib)
        out, nf, st = oracle.vlidort_solve_brdf(o, a["heights"], a["deltau"], a["omega"], greek, b, s, g["vzas"],
                                                g["raas"], g["nstreams"])
        assert st == 0
        for um in range(3):
            for ua in range(3):
                want = g["toa_up_I"][ib * 9 + um * 3 + ua]
                err.append(abs(out[um, ua] / want - 1.0))
    err = np.array(err)
    # measured: median 8.1e-7, max 5.2e-6 (the saved values carry 6 digits)
    assert np.median(err) < 3e-6, np.median(err)
    assert err.max() < 2e-5, err.max()


def test_lambertian_kernel_alone_is_the_lambertian_surface(golden_iqu):
    # a single Lambertian kernel of amplitude A through the BRDF path gives
    # the Lambertian-albedo solve (VBRDF_FOURIER: 1 in term 0, nothing after)
    a = golden_iqu
    o = oracle.OracleOpts(do_plane_parallel=0, do_double_convtest=1, taylor_order=3, accuracy=1e-4,
                          asymtx_tol=a["asymtx_tol"], earth_radius=a["earth_radius"], flux_factor=1.0,
                          do_focorr=1, do_focorr_nadir=1, do_focorr_outgoing=0, do_deltam=1, nfinelayers=0)
    greek = np.transpose(np.array(a["greek_nstokes1"]), (1, 0, 2))[0]
    for s in (35.0, 75.0):
        b = oracle.brdf_supplement([(1, 0.2, ())], 8, s, a["vzas"], a["raas"])
        ob, nfb, _ = oracle.vlidort_solve_brdf(o, a["heights"], a["deltau"], a["omega"], greek, b, s, a["vzas"],
                                               a["raas"], 8)
        ol, nfl, _ = oracle.vlidort_solve(o, a["heights"], a["deltau"], a["omega"], greek, 0.2, s, a["vzas"],
                                          a["raas"], 8)
        assert nfb == nfl
        assert np.max(np.abs(ob / ol - 1.0)) < 1e-13


def test_giss_cox_munk_kernel_against_the_self_tester():
    # the GISS Cox-Munk kernel of VLIDORT_Scalar_GissCX (index 10), (1,1)
    # element, through the supplement: the reference BRDF self tester's saved
    # exact BRDF and Fourier components m = 0, 1 (8 digits), fixture
    # tests/golden/brdf_gisscm_selftest.json (make_gisscm_golden.py)
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "brdf_gisscm_selftest.json")) as f:
        g = json.load(f)
    k = g["kernel"]
    b = oracle.brdf_supplement([(k["which"], k["factor"], k["pars"])], g["nstreams"], g["szas"][0], g["vzas"],
                               g["raas"], nstreams_brdf=g["nstreams_brdf"], do_shadow=g["shadow"])
    got = b["exactdb"].ravel()
    want = np.array(g["exact"])
    # measured: max 2.0e-8, median 8e-9 over the 11 values
    assert np.max(np.abs(got / want - 1.0)) < 1e-7, got / want - 1.0
    for m in (0, 1):
        w = g["fourier"][str(m)]
        pairs = ((b["f"][m, 0, 0], w["Stream-Stream"]), (b["f0"][m, 0], w["Solars-Stream"]),
                 (b["uf"][m, 0, 0], w["Stream-Users"]), (b["uf0"][m, 0], w["Solars-Users"]))
        for x, y in pairs:
            assert abs(x / y - 1.0) < 1e-7, (m, x, y)


@pytest.mark.parametrize("which", [1, 2, 3, 4, 5, 9, 10])
def test_supplement_kernels_against_the_scalar_self_tester(which):
    # every kernel of the scalar BRDF self tester that the oracle restates,
    # the MODIS RTLS pair (Ross-thick 3, Li-sparse 4) of VLIDORT_Scalar_LandMODIS
    # and the glint pair (9, 10) included: exact BRDF at three azimuths and
    # Fourier components m = 0, 1 against the saved 8 digits, fixture
    # tests/golden/brdf_selftest_scalar.json (make_brdf_selftest_golden.py)
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "brdf_selftest_scalar.json")) as f:
        g = json.load(f)
    k = next(x for x in g["kernels"] if x["which"] == which)
    b = oracle.brdf_supplement([(which, k["factor"], tuple(k["pars"]))], g["nstreams"], g["szas"][0], g["vzas"],
                               g["raas"], nstreams_brdf=g["nstreams_brdf"], do_shadow=k["shadow"])

    def close(x, y):  # measured: within 2.9e-8 relative for every kernel
        return abs(x - y) <= 5e-8 * abs(y) + 1e-12

    for x, y in zip(b["exactdb"].ravel(), k["exact"]):
        assert close(x, y), (which, x, y)
    for m in (0, 1):
        w = k["fourier"][str(m)]
        for x, y in ((b["f"][m, 0, 0], w["Stream-Stream"]), (b["f0"][m, 0], w["Solars-Stream"]),
                     (b["uf"][m, 0, 0], w["Stream-Users"]), (b["uf0"][m, 0], w["Solars-Users"])):
            assert close(x, y), (which, m, x, y)


def test_giss_and_cox_munk_scalar_elements_agree():
    # for a real refractive index the GISS kernel's (1,1) element with
    # parameters (sigma2 / 2, n) is the Cox-Munk kernel with (sigma2, n^2):
    # both are the Fresnel-weighted facet-slope density with the same
    # shadowing; the two restatements agree to rounding on random geometries
    rng = np.random.default_rng(7)
    for _ in range(5):
        sigma2 = 0.003 + 0.00512 * rng.uniform(0.0, 20.0)
        n = rng.uniform(1.32, 1.35)
        sza, vza, raa = rng.uniform(5.0, 75.0), rng.uniform(5.0, 65.0), rng.uniform(0.0, 180.0)
        vzas, raas = [vza], [raa]
        a = oracle.brdf_supplement([(9, 1.0, (sigma2, n * n, 0.0))], 8, sza, vzas, raas, nstreams_brdf=100,
                                   do_shadow=True)
        b = oracle.brdf_supplement([(10, 1.0, (0.5 * sigma2, n, 0.0))], 8, sza, vzas, raas, nstreams_brdf=100,
                                   do_shadow=True)
        assert abs(b["exactdb"].ravel()[0] / a["exactdb"].ravel()[0] - 1.0) < 1e-10
        for key in ("f", "f0", "uf", "uf0"):
            x, y = np.asarray(a[key]), np.asarray(b[key])
            scale = np.maximum(np.abs(x), 1e-3 * np.abs(x).max())  # Fourier components near 0 come from cancellation: measured up to 1.1e-11
            assert np.max(np.abs(x - y) / scale) < 1e-10, key

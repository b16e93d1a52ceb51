"""The per-thread RT solver of the CUDA kernel (aeroapps_gb300/csrc/rt_solve.cuh),
compiled for the host by this test only, against the oracle, in both working
precisions; and the team solver (rt_team.cuh, one std::thread per lane)
against the per-thread one.  This checks the GPU formulation (graded Jacobi
eigen-solution, block boundary-value sweep, team schedule) on the CPU; the
GPU tests check the kernels themselves."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import oracle

from rt_cases import MISSING, random_aop_case, rt_args

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def host_lib():
    d = tempfile.mkdtemp(prefix="aerort_host_")
    so = os.path.join(d, "librthost.so")
    subprocess.run(["g++", "-O1", "-std=c++17", "-fPIC", "-shared", "-o", so,
                    os.path.join(HERE, "host_harness", "rt_host.cpp")], check=True)
    return ctypes.CDLL(so)


@pytest.fixture(scope="module")
def team_lib():
    d = tempfile.mkdtemp(prefix="aerort_team_")
    so = os.path.join(d, "librtteam.so")
    subprocess.run(["g++", "-O1", "-std=c++20", "-pthread", "-fPIC", "-shared", "-o", so,
                    os.path.join(HERE, "host_harness", "rt_team_host.cpp")], check=True)
    return ctypes.CDLL(so)


def _host(lib, c, nstreams, fn="host_scalar_lambert"):
    P = lambda a: np.asfortranarray(a, np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    keep = [np.asfortranarray(c[k], np.float64) for k in ("ROT", "depol", "tau", "ssa", "pmom", "he", "albedo", "sza",
                                                            "raa", "vza")]
    ptrs = [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in keep]
    nobs, nch = c["ncol"], c["nch"]
    rad = np.zeros((nobs, nch), order="F")
    refl = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    first = np.array([nobs], np.int32)
    Ip = ctypes.POINTER(ctypes.c_int)
    getattr(lib, fn)(c["km"], nch, nobs, nstreams, c["nmom"], *ptrs, first.ctypes.data_as(Ip),
                            ctypes.c_double(MISSING), -1, rad.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                            refl.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nf.ctypes.data_as(Ip),
                            st.ctypes.data_as(Ip))
    return rad, nf, st


@pytest.mark.parametrize("nstreams,km", [(8, 72), (4, 20), (16, 12)])
def test_host_build_of_kernel_matches_oracle(host_lib, nstreams, km):
    c = random_aop_case(nstreams, km, nobs=4, nch=1, seed=km + nstreams)
    rad, nf, st = _host(host_lib, c, nstreams)
    orad, orefl, orc, onf, ost = oracle.scalar_lambert(*rt_args(c, nstreams), MISSING)
    assert np.array_equal(nf, onf) and np.all(st == 0)
    assert np.max(np.abs(rad / orad - 1)) < 1e-9


@pytest.mark.parametrize("nstreams,km", [(8, 24), (16, 8)])
def test_mixed_precision_solver_within_1e4(host_lib, nstreams, km):
    c = random_aop_case(nstreams, km, nobs=4, nch=1, seed=km + 3 * nstreams, ssa_range=(0.999, 1.0))
    rad, nf, st = _host(host_lib, c, nstreams, "host_scalar_lambert_mixed")
    orad = oracle.scalar_lambert(*rt_args(c, nstreams), MISSING)[0]
    assert np.all(st == 0)
    assert np.max(np.abs(rad / orad - 1)) < 1e-4


@pytest.mark.parametrize("nstreams,km", [(4, 6), (12, 3), (16, 4), (6, 4)])
def test_team_solver_matches_thread_solver(host_lib, team_lib, nstreams, km):
    c = random_aop_case(nstreams, km, nobs=1, nch=1, seed=km + 7 * nstreams)
    rad, nf, st = _host(host_lib, c, nstreams)
    trad, tnf, tst = _host(team_lib, c, nstreams, "team_scalar_lambert")
    assert np.array_equal(nf, tnf) and np.array_equal(st, tst)
    assert np.max(np.abs(trad / rad - 1)) < 1e-13
    mrad, _, mst = _host(host_lib, c, nstreams, "host_scalar_lambert_mixed")
    tmrad, _, tmst = _host(team_lib, c, nstreams, "team_scalar_lambert_mixed")
    assert np.all(tmst == 0) and np.max(np.abs(tmrad / mrad - 1)) < 1e-5


def test_more_input_moments_than_streams(host_lib):
    # nMom = 40 > 2N: delta-M truncates at 2N-1 while the single-scatter phase
    # function uses every input moment
    c = random_aop_case(6, 30, nobs=4, nch=1, seed=17)
    nmom = 40
    pm = np.zeros(c["g"].shape + (nmom, 1))
    for l in range(nmom):
        pm[..., l, 0] = (2 * l + 1) * c["g"] ** l
    c["pmom"] = np.asfortranarray(pm)
    c["nmom"] = nmom
    orad = oracle.scalar_lambert(*rt_args(c, 6), MISSING)[0]
    for fn, tol in (("host_scalar_lambert", 1e-9), ("host_scalar_lambert_mixed", 1e-4)):
        rad, nf, st = _host(host_lib, c, 6, fn)
        assert np.all(st == 0) and np.max(np.abs(rad / orad - 1)) < tol


@pytest.mark.parametrize("nstreams,km", [(8, 30), (4, 12), (16, 8)])
def test_plane_parallel_flag(host_lib, team_lib, nstreams, km):
    # VLIDORT_Scalar_Lambert's plane_parallel = .true.: plane-parallel beam
    # attenuation and single-scatter geometry instead of the pseudo-spherical ones
    c = random_aop_case(nstreams, km, nobs=4, nch=1, seed=5 * km + nstreams)
    args = list(rt_args(c, nstreams))
    args[5] = True
    orad, orefl, orc, onf, ost = oracle.scalar_lambert(*args, MISSING)
    sph = oracle.scalar_lambert(*rt_args(c, nstreams), MISSING)[0]
    assert orc == 0 and np.max(np.abs(orad / sph - 1)) > 1e-5  # the flag changes the answer
    # the team solver (one thread per lane on the host: slow) on one short column
    c1 = random_aop_case(nstreams, 4, nobs=1, nch=1, seed=km + nstreams)
    host_lib.host_set_plane_parallel(1)
    team_lib.team_set_plane_parallel(1)
    try:
        rad, nf, st = _host(host_lib, c, nstreams)
        mrad, _, mst = _host(host_lib, c, nstreams, "host_scalar_lambert_mixed")
        rad1, nf1, _ = _host(host_lib, c1, nstreams)
        trad, tnf, tst = _host(team_lib, c1, nstreams, "team_scalar_lambert")
    finally:
        host_lib.host_set_plane_parallel(0)
        team_lib.team_set_plane_parallel(0)
    assert np.array_equal(nf, onf) and np.all(st == 0) and np.all(mst == 0)
    assert np.max(np.abs(rad / orad - 1)) < 1e-9
    assert np.max(np.abs(mrad / orad - 1)) < 1e-4
    assert np.array_equal(tnf, nf1) and np.all(tst == 0) and np.max(np.abs(trad / rad1 - 1)) < 1e-12


def _host_brdf(lib, c, nstreams, kw, par):
    P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    keep = [np.asfortranarray(c[k], np.float64) for k in ("ROT", "depol", "tau", "ssa", "pmom", "he")]
    kwf, parf = np.asfortranarray(kw, np.float64), np.asfortranarray(par, np.float64)
    ang = [np.ascontiguousarray(c[k], np.float64) for k in ("sza", "raa", "vza")]
    nobs, nch = c["ncol"], c["nch"]
    rad = np.zeros((nobs, nch), order="F")
    refl = np.zeros_like(rad)
    br = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    first = np.array([nobs], np.int32)
    Ip = ctypes.POINTER(ctypes.c_int)
    lib.team_scalar_landmodis(c["km"], nch, nobs, nstreams, c["nmom"], *[P(a) for a in keep], P(kwf), P(parf),
                              *[P(a) for a in ang], first.ctypes.data_as(Ip), ctypes.c_double(MISSING), P(rad),
                              P(refl), P(br), nf.ctypes.data_as(Ip), st.ctypes.data_as(Ip))
    return rad, refl, br, nf, st


@pytest.mark.parametrize("nstreams,km", [(4, 10), (8, 6)])
def test_team_solver_over_modis_brdf_matches_oracle(team_lib, nstreams, km):
    # the RTLS surface of VLIDORT_Scalar_LandMODIS through the team solve
    # (one std::thread per lane): same Fourier terms, radiance within 1e-9,
    # BR exact; one (pixel, channel) with an unphysical kernel set gives -500
    from rt_cases import modis_brdf
    c = random_aop_case(nstreams, km, nobs=3, nch=2, seed=km + 5 * nstreams)
    kw, par = modis_brdf(3, 2, seed=nstreams, negative=[(1, 0)])
    rad, refl, br, nf, st = _host_brdf(team_lib, c, nstreams, kw, par)
    a = rt_args(c, nstreams)
    orad, orefl, obr, orc, onf, ost = oracle.scalar_landmodis(*a[:17], kw, par, c["sza"], c["raa"], c["vza"],
                                                              MISSING)
    assert orc == 0
    assert obr[1, 0] == -500.0 and br[1, 0] == -500.0 and rad[1, 0] == -500.0 and orad[1, 0] == -500.0
    ok = obr != -500.0
    assert np.max(np.abs(br[ok] - obr[ok])) < 1e-14
    assert np.array_equal(nf[ok], onf[ok]) and np.all(st == 0)
    assert np.max(np.abs(rad[ok] / orad[ok] - 1)) < 1e-9
    assert np.max(np.abs(refl[ok] / orefl[ok] - 1)) < 1e-9


def _host_cx(lib, c, nstreams, u10, v10, mr, giss=False):
    P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    keep = [np.asfortranarray(c[k], np.float64) for k in ("ROT", "depol", "tau", "ssa", "pmom", "he")]
    surf = [np.ascontiguousarray(a, np.float64) for a in (u10, v10, mr)]
    ang = [np.ascontiguousarray(c[k], np.float64) for k in ("sza", "raa", "vza")]
    nobs, nch = c["ncol"], c["nch"]
    rad = np.zeros((nobs, nch), order="F")
    refl = np.zeros_like(rad)
    br = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    first = np.array([nobs], np.int32)
    Ip = ctypes.POINTER(ctypes.c_int)
    lib.team_scalar_cx(int(giss), c["km"], nch, nobs, nstreams, c["nmom"], *[P(a) for a in keep], *[P(a) for a in surf],
                       *[P(a) for a in ang], first.ctypes.data_as(Ip), ctypes.c_double(MISSING), P(rad), P(refl),
                       P(br), nf.ctypes.data_as(Ip), st.ctypes.data_as(Ip))
    return rad, refl, br, nf, st


@pytest.mark.parametrize("nstreams,km,giss", [(4, 10, False), (8, 6, True)])
def test_team_solver_over_cox_munk_matches_oracle(team_lib, nstreams, km, giss):
    # the Cox-Munk glint of VLIDORT_Scalar_CX (giss: the GISS kernel of
    # VLIDORT_Scalar_GissCX) through the team solve: same Fourier terms,
    # radiance within 1e-9; a MISSING wind gives MISSING
    from rt_cases import ocean_cx
    c = random_aop_case(nstreams, km, nobs=3, nch=2, seed=km + 7 * nstreams)
    u, v, mr = ocean_cx(3, 2, seed=nstreams)
    u[2] = MISSING
    rad, refl, br, nf, st = _host_cx(team_lib, c, nstreams, u, v, mr, giss)
    a = rt_args(c, nstreams)
    orad, orefl, obr, orc, onf, ost = oracle.scalar_cx(*a[:17], u, v, mr, c["sza"], c["raa"], c["vza"], MISSING,
                                                       giss=giss)
    assert orc == 0
    assert np.all(rad[2] == MISSING) and np.all(orad[2] == MISSING) and np.all(br[2] == MISSING)
    ok = orad != MISSING
    assert np.max(np.abs(br[ok] / obr[ok] - 1)) < 1e-12
    assert np.array_equal(nf[ok], onf[ok]) and np.all(st == 0)
    assert np.max(np.abs(rad[ok] / orad[ok] - 1)) < 1e-9
    assert np.max(np.abs(refl[ok] / orefl[ok] - 1)) < 1e-9


def _refine(lib, sf, raa=0.0):
    a = np.ascontiguousarray(sf, np.float64)
    ml = ctypes.c_int(0)
    f = lib.host_refine_flag(len(a), a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_double(raa),
                             ctypes.byref(ml))
    return f, ml.value


def test_refinement_flags_convergence_tests_at_the_threshold(host_lib):
    # a mixed-method solve goes to the FP64 pass when a convergence test's
    # |term / sum| lies within 1e-3 (relative) of the accuracy threshold
    # (1e-4): its FP32 terms could decide that test the other way
    acc = 1e-4

    def series(q):  # term 1 at ratio q, then two converged terms
        s1 = q / (1.0 - q)
        return [1.0, s1, 1e-9, 1e-9]
    for q, want in ((acc * (1 + 5e-4), 1), (acc * (1 - 5e-4), 1), (acc * (1 + 5e-3), 0), (acc * (1 - 5e-3), 0),
                    (0.3, 0)):
        f, _ = _refine(host_lib, series(q))
        assert f == want, (q, f)
    # the 865 nm radiance of a 12-stream, 21-layer column whose FP64 series
    # stops after term 8 at |term / sum| = 0.99998e-4 (the FP32 one, at
    # 1.00018e-4, ran on to term 13, 7.9e-4 away): flagged
    terms = [2.107697e-02, 2.737219e-04, -8.405132e-04, -2.020928e-05, 2.019701e-05, 5.192561e-06, -6.980721e-06,
             -1.281008e-07, -2.050567e-06]
    f, ml = _refine(host_lib, terms)
    assert ml == 8 and f == 1
    # cancellation (sum |terms| > 10 |sum|) still flags on its own
    f, _ = _refine(host_lib, [1.0, -0.95, 1e-9, 1e-9])
    assert f == 1


def _host_termpar(lib, c, nstreams, W):
    keep = [np.asfortranarray(c[k], np.float64) for k in ("ROT", "depol", "tau", "ssa", "pmom", "he", "albedo", "sza",
                                                            "raa", "vza")]
    ptrs = [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in keep]
    nobs, nch = c["ncol"], c["nch"]
    rad = np.zeros((nobs, nch), order="F")
    refl = np.zeros_like(rad)
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    first = np.array([nobs], np.int32)
    Ip = ctypes.POINTER(ctypes.c_int)
    lib.team_scalar_lambert_termpar(W, c["km"], nch, nobs, nstreams, c["nmom"], *ptrs, first.ctypes.data_as(Ip),
                                    ctypes.c_double(MISSING), rad.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    refl.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nf.ctypes.data_as(Ip),
                                    st.ctypes.data_as(Ip))
    return rad, nf, st


@pytest.mark.parametrize("nstreams,km,W", [(8, 12, 3), (4, 20, 8)])
def test_term_parallel_fp64_resolve_is_the_sequential_series(team_lib, nstreams, km, W):
    # the refinement list's FP64 re-solve with each solve's Fourier terms
    # spread over W teams (k_refine_terms, emulated on the host: P~_m^m
    # carried over the skipped terms, the sum taken in term order) gives the
    # sequential team series bit for bit, Fourier-term counts included
    c = random_aop_case(nstreams, km, nobs=2, nch=1, seed=km + W)
    a = _host(team_lib, c, nstreams, "team_scalar_lambert")
    b = _host_termpar(team_lib, c, nstreams, W)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.all(b[2] == 0)

"""GPU parity of the BRDF paths -- MODIS RTLS (aerort_vlidort_scalar_landmodis*,
VLIDORT_Scalar_LandMODIS) and Cox-Munk glint (aerort_vlidort_scalar_cx*,
VLIDORT_Scalar_CX) -- against the oracle (oracle_scalar_landmodis,
oracle_scalar_cx), whose kernels and BRDF solve are pinned to the reference's
saved BRDF results (tests/test_oracle_golden_brdf.py).  Bar: identical Fourier-term counts and
status codes; radiance and reflectance within 1e-9 relative; BR to round-off;
-500 where the kernel combination is negative; MISSING where the angles are."""
import numpy as np
import pytest

from aeroapps_gb300 import _lib, vlidort
from oracle import oracle

from rt_cases import MISSING, modis_brdf, random_aop_case, rt_args

RTOL = 1e-9


def _both(c, N, kw, par):
    a = rt_args(c, N)
    got = vlidort.vlidort_scalar_landmodis(*a[:17], kw, par, c["sza"], c["raa"], c["vza"], MISSING=MISSING,
                                           diagnostics=True)
    ref = oracle.scalar_landmodis(*a[:17], kw, par, c["sza"], c["raa"], c["vza"], MISSING)
    return got, ref


def _check(got, ref):
    rad, refl, br, rc, nf, st = got
    orad, orefl, obr, orc, onf, ost = ref
    assert rc == 0 and orc == 0
    assert np.array_equal(st, ost) and np.array_equal(nf, onf)
    assert np.array_equal(rad == MISSING, orad == MISSING) and np.array_equal(rad == -500.0, orad == -500.0)
    ok = (orad != MISSING) & (orad != -500.0)
    assert np.max(np.abs(rad[ok] / orad[ok] - 1.0)) <= RTOL
    assert np.max(np.abs(refl[ok] / orefl[ok] - 1.0)) <= RTOL
    okb = obr != MISSING
    assert np.max(np.abs(br[okb] - obr[okb])) <= 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("N,km", [(4, 30), (8, 24), (12, 16), (16, 12)])
def test_landmodis_matches_oracle(N, km):
    c = random_aop_case(N, km, nobs=5, nch=2, seed=300 + N)
    kw, par = modis_brdf(5, 2, seed=N, negative=[(2, 1)])
    _check(*_both(c, N, kw, par))


@pytest.mark.gpu
def test_landmodis_missing_angles_distinct_parameters_and_72_layers():
    # a MISSING solar angle, and a different Li-sparse parameter pair for
    # every (pixel, channel) (one Fourier table each)
    N = 8
    c = random_aop_case(N, 72, nobs=4, nch=2, seed=77)
    kw, par = modis_brdf(4, 2, seed=5)
    rng = np.random.default_rng(9)
    par = np.asfortranarray(np.stack([rng.uniform(1.0, 3.0, (2, 4)), rng.uniform(0.5, 1.5, (2, 4))]))
    c["sza"][3] = MISSING
    got, ref = _both(c, N, kw, par)
    _check(got, ref)
    assert np.all(got[0][3] == MISSING) and np.all(got[2][3] == MISSING)


@pytest.mark.gpu
def test_lambertian_kernel_alone_is_the_lambertian_call():
    # fvol = fgeo = 0: the RTLS path gives the Lambertian solve with albedo fiso
    N = 6
    c = random_aop_case(N, 20, nobs=4, nch=2, seed=41)
    kw = np.asfortranarray(np.stack([c["albedo"].T, np.zeros((2, 4)), np.zeros((2, 4))]))
    par = np.asfortranarray(np.stack([np.full((2, 4), 2.0), np.ones((2, 4))]))
    a = rt_args(c, N)
    rad, refl, br, rc = vlidort.vlidort_scalar_landmodis(*a[:17], kw, par, c["sza"], c["raa"], c["vza"])
    lrad, lrefl, lrc = vlidort.vlidort_scalar_lambert(*a, MISSING=MISSING)
    assert rc == 0 and lrc == 0
    assert np.max(np.abs(rad / lrad - 1.0)) <= 1e-12
    assert np.max(np.abs(br - c["albedo"])) <= 1e-15


@pytest.mark.gpu
def test_batched_device_call_reads_fp32_optics():
    # aerort_vlidort_scalar_landmodis_batch_dev with per-column layer counts
    # and FP32 optics equals the host call on the same (FP64-converted) optics
    import torch
    N = 12
    c = random_aop_case(N, 24, nobs=6, nch=2, seed=123)
    kw, par = modis_brdf(6, 2, seed=3)
    tau32, ssa32, pm32 = [np.asfortranarray(c[k].astype(np.float32)) for k in ("tau", "ssa", "pmom")]
    for k, v in (("tau", tau32), ("ssa", ssa32), ("pmom", pm32)):
        c[k] = np.asfortranarray(v.astype(np.float64))
    a = rt_args(c, N)
    hrad, hrefl, hbr, hrc, hnf, hst = vlidort.vlidort_scalar_landmodis(*a[:17], kw, par, c["sza"], c["raa"], c["vza"],
                                                                       diagnostics=True)
    dev = lambda x, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(x, dt).ravel(order="F"))).cuda()
    d = {k: dev(c[k], np.float64) for k in ("ROT", "depol", "he", "sza", "raa", "vza")}
    t32, s32, p32 = dev(tau32, np.float32), dev(ssa32, np.float32), dev(pm32[..., 0], np.float32)
    dkw = dev(kw, np.float64)
    parh = np.asfortranarray(par, np.float64)
    nobs, nch = 6, 2
    out = {k: torch.zeros(nobs * nch, dtype=torch.float64, device="cuda") for k in ("rad", "refl", "br")}
    nf = torch.zeros(nobs * nch, dtype=torch.int32, device="cuda")
    st = torch.zeros_like(nf)
    nl = dev(np.full(nobs, c["km"]), np.int32)
    P = lambda t: t.data_ptr()
    rc = _lib.lib().aerort_vlidort_scalar_landmodis_batch_dev(
        c["km"], nch, nobs, N, 0, c["nmom"], P(nl), P(d["ROT"]), P(d["depol"]), None, None, None, P(t32), P(s32),
        P(p32), P(d["he"]), P(dkw), _lib.ptr(parh, _lib.P_d), P(d["sza"]), P(d["raa"]), P(d["vza"]), MISSING,
        P(out["rad"]), P(out["refl"]), P(out["br"]), P(nf), P(st), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    rad = out["rad"].cpu().numpy().reshape(nobs, nch, order="F")
    br = out["br"].cpu().numpy().reshape(nobs, nch, order="F")
    assert np.array_equal(nf.cpu().numpy().reshape(nobs, nch, order="F"), hnf)
    assert np.max(np.abs(rad / hrad - 1.0)) <= 1e-13 and np.max(np.abs(br - hbr)) <= 1e-15


# ---------------------------------------------------------------- Cox-Munk glint (VLIDORT_Scalar_CX)

def _both_cx(c, N, u, v, mr, giss=False):
    a = rt_args(c, N)
    got = vlidort.vlidort_scalar_cx(*a[:17], u, v, mr, c["sza"], c["raa"], c["vza"], MISSING=MISSING,
                                    diagnostics=True, giss=giss)
    ref = oracle.scalar_cx(*a[:17], u, v, mr, c["sza"], c["raa"], c["vza"], MISSING, giss=giss)
    return got, ref


def _check_cx(got, ref):
    rad, refl, br, rc, nf, st = got
    orad, orefl, obr, orc, onf, ost = ref
    assert rc == 0 and orc == 0
    assert np.array_equal(st, ost) and np.array_equal(nf, onf)
    assert np.array_equal(rad == MISSING, orad == MISSING) and np.array_equal(br == MISSING, obr == MISSING)
    ok = orad != MISSING
    assert np.max(np.abs(rad[ok] / orad[ok] - 1.0)) <= RTOL
    assert np.max(np.abs(refl[ok] / orefl[ok] - 1.0)) <= RTOL
    okb = (obr != MISSING) & (obr > 1e-30)
    assert np.max(np.abs(br[okb] / obr[okb] - 1.0)) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("N,km,giss", [(4, 30, False), (8, 24, False), (12, 16, False), (16, 12, False),
                                       (6, 20, True), (12, 40, True), (16, 24, True)])
def test_cox_munk_matches_oracle(N, km, giss):
    # VLIDORT_Scalar_CX, and with giss VLIDORT_Scalar_GissCX (the ocean driver's call)
    from rt_cases import ocean_cx
    c = random_aop_case(N, km, nobs=5, nch=2, seed=500 + N + int(giss))
    u, v, mr = ocean_cx(5, 2, seed=N)
    _check_cx(*_both_cx(c, N, u, v, mr, giss))


@pytest.mark.gpu
def test_cox_munk_missing_winds_and_angles_calm_and_storm():
    # a MISSING wind component (both channels), a MISSING refractive index (one
    # channel), a MISSING solar angle; calm (W = 0) and storm (W > 50 m/s,
    # clamped) seas; 72 layers
    from rt_cases import ocean_cx
    N = 8
    c = random_aop_case(N, 72, nobs=6, nch=2, seed=88)
    u, v, mr = ocean_cx(6, 2, seed=4)
    u[1] = MISSING
    c["sza"][2] = MISSING
    u[3], v[3] = 0.0, 0.0
    u[4], v[4] = 45.0, -40.0
    got, ref = _both_cx(c, N, u, v, mr)
    _check_cx(got, ref)
    assert np.all(got[0][1] == MISSING) and np.all(got[0][2] == MISSING)
    mr2 = mr.copy()
    mr2[1] = MISSING
    got2, ref2 = _both_cx(c, N, u, v, mr2)
    _check_cx(got2, ref2)
    assert np.all(got2[0][:, 1] == MISSING) and not np.any(got2[0][[0, 3, 4, 5], 0] == MISSING)


@pytest.mark.gpu
@pytest.mark.parametrize("giss", [False, True])
def test_cox_munk_batched_device_call(giss):
    # aerort_vlidort_scalar_(giss)cx_batch_dev with FP32 optics equals the host
    # call on the same (FP64-converted) optics
    import torch
    from rt_cases import ocean_cx
    N = 12
    c = random_aop_case(N, 24, nobs=6, nch=2, seed=321)
    u, v, mr = ocean_cx(6, 2, seed=7)
    tau32, ssa32, pm32 = [np.asfortranarray(c[k].astype(np.float32)) for k in ("tau", "ssa", "pmom")]
    for k, x in (("tau", tau32), ("ssa", ssa32), ("pmom", pm32)):
        c[k] = np.asfortranarray(x.astype(np.float64))
    a = rt_args(c, N)
    hrad, hrefl, hbr, hrc, hnf, hst = vlidort.vlidort_scalar_cx(*a[:17], u, v, mr, c["sza"], c["raa"], c["vza"],
                                                                diagnostics=True, giss=giss)
    dev = lambda x, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(x, dt).ravel(order="F"))).cuda()
    d = {k: dev(c[k], np.float64) for k in ("ROT", "depol", "he", "sza", "raa", "vza")}
    t32, s32, p32 = dev(tau32, np.float32), dev(ssa32, np.float32), dev(pm32[..., 0], np.float32)
    du, dv, dm = dev(u, np.float64), dev(v, np.float64), dev(mr, np.float64)
    nobs, nch = 6, 2
    out = {k: torch.zeros(nobs * nch, dtype=torch.float64, device="cuda") for k in ("rad", "refl", "br")}
    nf = torch.zeros(nobs * nch, dtype=torch.int32, device="cuda")
    st = torch.zeros_like(nf)
    nl = dev(np.full(nobs, c["km"]), np.int32)
    P = lambda t: t.data_ptr()
    fn = _lib.lib().aerort_vlidort_scalar_gisscx_batch_dev if giss else _lib.lib().aerort_vlidort_scalar_cx_batch_dev
    rc = fn(
        c["km"], nch, nobs, N, 0, c["nmom"], P(nl), P(d["ROT"]), P(d["depol"]), None, None, None, P(t32), P(s32),
        P(p32), P(d["he"]), P(du), P(dv), P(dm), P(d["sza"]), P(d["raa"]), P(d["vza"]), MISSING,
        P(out["rad"]), P(out["refl"]), P(out["br"]), P(nf), P(st), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    rad = out["rad"].cpu().numpy().reshape(nobs, nch, order="F")
    br = out["br"].cpu().numpy().reshape(nobs, nch, order="F")
    assert np.array_equal(nf.cpu().numpy().reshape(nobs, nch, order="F"), hnf)
    assert np.max(np.abs(rad / hrad - 1.0)) <= 1e-13 and np.max(np.abs(br - hbr)) <= 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("giss", [False, True])
def test_glint_plane_parallel_nadir_sun_and_view(giss):
    # plane-parallel beam attenuation; a pixel at solar zenith exactly 0 turns
    # on the wrapper's sticky nadir single-scatter flag for it and every later
    # pixel; a nadir view (VZA = 0, where the GISS kernel replaces the cosine
    # 1 by 0.999999999999)
    from rt_cases import ocean_cx
    N = 8
    c = random_aop_case(N, 30, nobs=6, nch=2, seed=71 + int(giss))
    u, v, mr = ocean_cx(6, 2, seed=12)
    c["sza"][2] = 0.0
    c["vza"][4] = 0.0
    for pp in (False, True):
        a = list(rt_args(c, N))
        a[5] = pp
        got = vlidort.vlidort_scalar_cx(*a[:17], u, v, mr, c["sza"], c["raa"], c["vza"], MISSING=MISSING,
                                        diagnostics=True, giss=giss)
        ref = oracle.scalar_cx(*a[:17], u, v, mr, c["sza"], c["raa"], c["vza"], MISSING, giss=giss)
        _check_cx(got, ref)


@pytest.mark.gpu
def test_gisscx_batched_ragged_columns():
    # aerort_vlidort_scalar_gisscx_batch_dev with per-column layer counts
    # (FP64 optics on the device) against the oracle with the same counts
    import torch
    from rt_cases import ocean_cx
    N = 16
    c = random_aop_case(N, 40, nobs=7, nch=2, seed=404)
    u, v, mr = ocean_cx(7, 2, seed=8)
    nl = np.array([40, 12, 25, 1, 33, 40, 7], np.int32)
    a = rt_args(c, N)
    orad, orefl, obr, orc, onf, ost = oracle.scalar_cx(*a[:17], u, v, mr, c["sza"], c["raa"], c["vza"], MISSING,
                                                       nlay=nl, giss=True)
    dev = lambda x, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(x, dt).ravel(order="F"))).cuda()
    d = {k: dev(c[k], np.float64) for k in ("ROT", "depol", "tau", "ssa", "he", "sza", "raa", "vza")}
    pm = dev(c["pmom"][..., 0], np.float64)
    du, dv, dm = dev(u, np.float64), dev(v, np.float64), dev(mr, np.float64)
    nobs, nch = 7, 2
    out = {k: torch.zeros(nobs * nch, dtype=torch.float64, device="cuda") for k in ("rad", "refl", "br")}
    nf = torch.zeros(nobs * nch, dtype=torch.int32, device="cuda")
    st = torch.zeros_like(nf)
    dnl = dev(nl, np.int32)
    P = lambda t: t.data_ptr()
    rc = _lib.lib().aerort_vlidort_scalar_gisscx_batch_dev(
        c["km"], nch, nobs, N, 0, c["nmom"], P(dnl), P(d["ROT"]), P(d["depol"]), P(d["tau"]), P(d["ssa"]), P(pm),
        None, None, None, P(d["he"]), P(du), P(dv), P(dm), P(d["sza"]), P(d["raa"]), P(d["vza"]), MISSING,
        P(out["rad"]), P(out["refl"]), P(out["br"]), P(nf), P(st), torch.cuda.current_stream().cuda_stream)
    assert rc == 0 and orc == 0, _lib.last_error()
    torch.cuda.synchronize()
    rad = out["rad"].cpu().numpy().reshape(nobs, nch, order="F")
    gnf = nf.cpu().numpy().reshape(nobs, nch, order="F")
    gst = st.cpu().numpy().reshape(nobs, nch, order="F")
    assert np.array_equal(gnf, onf) and np.array_equal(gst, ost)
    ok = orad != MISSING
    assert np.max(np.abs(rad[ok] / orad[ok] - 1.0)) <= RTOL

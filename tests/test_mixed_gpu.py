"""GPU accuracy of the mixed-precision RT path (AERORT_PREC_MIXED: FP32 Fourier
series) against the FP64 oracle.

Bar: relative TOA-radiance error <= 1e-4 against the FP64 oracle on the same
inputs, on columns of the synthetic configurations (Mie optics, 20-72 layers,
4-16 streams) and on the near-conservative stress set (layer SSA in
[0.999, 1)).  Every solve must succeed (status 0).
"""
import numpy as np
import pytest

from aeroapps_gb300 import _lib, mie, synth, vlidort
from oracle import oracle

from rt_cases import MISSING, random_aop_case, rt_args

RTOL = 1.0e-4
CH = [470.0, 550.0, 670.0, 865.0]


def _mixed(c, N, nlay=None):
    nl = np.full(c["ncol"], c["km"], np.int32) if nlay is None else nlay
    return vlidort.vlidort_scalar_lambert_batch(c["km"], c["nch"], c["ncol"], N, c["nmom"], nl, c["ROT"], c["depol"],
                                                c["tau"], c["ssa"], c["pmom"][..., 0], c["he"], c["albedo"], c["sza"],
                                                c["raa"], c["vza"], MISSING=MISSING, precision="mixed")


@pytest.mark.gpu
@pytest.mark.parametrize("N", [4, 6, 8, 12, 16])
def test_mixed_on_mie_columns(N):
    ncol = 24
    rng = np.random.default_rng(500 + N)
    nl = rng.integers(20, 73, ncol).astype(np.int32)
    cols = synth.make_columns(ncol, CH, seed=600 + N, nlayers=nl)
    tabs = mie.generate_tables(CH, nmom=2 * N)
    chem = mie.ChemMie(tabs)
    qt, qb = zip(*[chem.query_idx(x) for x in synth.tracer_names()])
    chem.destroy()
    km = cols["km"]
    tau, ssa, g, pm, rc = oracle.get_aop_vector(tabs, km, ncol, 4, 20, np.float32(CH), qt, qb, cols["qm"], cols["rh"],
                                                2 * N, 1)
    assert rc == 0
    orad, _, _, onf, ost = oracle.scalar_lambert(km, 4, ncol, np.array(CH), N, 0, 2 * N, 1, cols["ROT"], cols["depol"],
                                                 tau, ssa, g, pm, cols["pe"], cols["he"], cols["te"], cols["albedo"],
                                                 cols["sza"], cols["raa"], cols["vza"], MISSING, nlay=nl)
    rad, refl, rc, nf, st = vlidort.vlidort_scalar_lambert_batch(
        km, 4, ncol, N, 2 * N, nl, cols["ROT"], cols["depol"], tau.astype(np.float64), ssa.astype(np.float64),
        pm[..., 0].astype(np.float64), cols["he"], cols["albedo"], cols["sza"], cols["raa"], cols["vza"],
        MISSING=MISSING, precision="mixed")
    assert rc == 0 and np.all(st == 0) and np.all(ost == 0)
    err = np.abs(rad / orad - 1.0)
    assert err.max() <= RTOL, err.max()


@pytest.mark.gpu
@pytest.mark.parametrize("N,lo", [(8, 0.999), (16, 0.999), (8, 0.9999), (12, 0.9999)])
def test_mixed_near_conservative(N, lo):
    c = random_aop_case(N, 72, nobs=24, nch=2, seed=N * 7 + int(lo * 10), ssa_range=(lo, 1.0))
    orad, _, _, onf, ost = oracle.scalar_lambert(*rt_args(c, N), MISSING)
    rad, refl, rc, nf, st = _mixed(c, N)
    assert rc == 0 and np.all(st == 0)
    ok = orad != MISSING
    err = np.abs(rad[ok] / orad[ok] - 1.0)
    assert err.max() <= RTOL, err.max()


@pytest.mark.gpu
def test_mixed_device_path_reads_fp32_optics():
    import torch
    N, ncol = 8, 40
    rng = np.random.default_rng(77)
    nl = rng.integers(20, 73, ncol).astype(np.int32)
    cols = synth.make_columns(ncol, CH[:2], seed=78, nlayers=nl)
    km = cols["km"]
    tabs = mie.generate_tables(CH[:2], nmom=2 * N)
    chem = mie.ChemMie(tabs)
    names = synth.tracer_names()
    qt = np.array([chem.query_idx(x)[0] for x in names], np.int32)
    qb = np.array([chem.query_idx(x)[1] for x in names], np.int32)
    tau, ssa, g, pm, rc = oracle.get_aop_vector(tabs, km, ncol, 2, 20, np.float32(CH[:2]), qt, qb, cols["qm"],
                                                cols["rh"], 2 * N, 1)
    orad, _, _, _, _ = oracle.scalar_lambert(km, 2, ncol, np.array(CH[:2]), N, 0, 2 * N, 1, cols["ROT"],
                                             cols["depol"], tau, ssa, g, pm, cols["pe"], cols["he"], cols["te"],
                                             cols["albedo"], cols["sza"], cols["raa"], cols["vza"], MISSING, nlay=nl)
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    qm, rh = d(cols["qm"], np.float32), d(cols["rh"], np.float32)
    t_ = torch.zeros(km * 2 * ncol, dtype=torch.float32, device="cuda")
    s_, g_ = torch.zeros_like(t_), torch.zeros_like(t_)
    p_ = torch.zeros(km * 2 * ncol * 2 * N, dtype=torch.float32, device="cuda")
    rad = torch.zeros(ncol * 2, dtype=torch.float64, device="cuda")
    refl = torch.zeros_like(rad)
    nf = torch.zeros(ncol * 2, dtype=torch.int32, device="cuda")
    st = torch.zeros_like(nf)
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    ch = np.float32(CH[:2])
    rc = L.aerort_get_aop_vector_dev(chem.handle, km, ncol, 2, 20, _lib.ptr(ch, _lib.P_f), _lib.ptr(qt, _lib.P_i),
                                     _lib.ptr(qb, _lib.P_i), qm.data_ptr(), rh.data_ptr(), 2 * N, 1, t_.data_ptr(),
                                     s_.data_ptr(), g_.data_ptr(), p_.data_ptr(), stream)
    assert rc == 0
    dd = [d(cols[k], np.float64) for k in ("ROT", "depol", "he", "albedo", "sza", "raa", "vza")]
    nld = d(nl, np.int32)
    rc = L.aerort_vlidort_scalar_lambert_mixed_batch_dev(
        km, 2, ncol, N, 0, 2 * N, nld.data_ptr(), dd[0].data_ptr(), dd[1].data_ptr(), None, None, None,
        t_.data_ptr(), s_.data_ptr(), p_.data_ptr(), dd[2].data_ptr(), dd[3].data_ptr(), dd[4].data_ptr(),
        dd[5].data_ptr(), dd[6].data_ptr(), MISSING, rad.data_ptr(), refl.data_ptr(), nf.data_ptr(), st.data_ptr(),
        stream)
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    chem.destroy()
    r = rad.cpu().numpy().reshape(ncol, 2, order="F")
    assert np.all(st.cpu().numpy() == 0)
    assert np.max(np.abs(r / orad - 1)) <= RTOL


def test_schedule_api_validates():
    L = _lib.lib()
    assert L.aerort_set_schedule(7, 0, 64, 0) == 1003
    assert L.aerort_set_schedule(8, 2, 64, 0) == 1002
    assert L.aerort_set_schedule(8, 0, 48, 0) == 1002
    import ctypes
    t, b = ctypes.c_int(), ctypes.c_int()
    assert L.aerort_set_schedule(8, 1, 96, 2) == 0
    assert L.aerort_get_schedule(8, 1, ctypes.byref(t), ctypes.byref(b)) == 0
    assert (t.value, b.value) == (96, 2)
    assert L.aerort_set_schedule(8, 1, 32, 0) == 0


@pytest.mark.gpu
def test_cancelling_fourier_sum_is_refined_in_fp64():
    # a 4-stream column near backscatter (relative azimuth 173 deg) whose 670 nm
    # radiance is a 60x cancellation of its Fourier terms: the mixed method
    # lists it and re-solves it in FP64 (aerort_refined_count >= 1)
    import ctypes
    import bench
    full = bench.make_batch(8192, seed=20261204)
    g = bench.subset(full, np.array([3167, 3168, 3169]))
    N = int(g["nstreams"][0])
    assert N == 4
    tabs = mie.generate_tables(CH, nmom=32)
    chem = mie.ChemMie(tabs)
    qt, qb = zip(*[chem.query_idx(x) for x in synth.tracer_names()])
    chem.destroy()
    km, n = g["km"], 3
    nl = np.ascontiguousarray(g["nlayers"], np.int32)
    tau, ssa, gg, pm, rc = oracle.get_aop_vector(tabs, km, n, 4, 20, np.float32(CH), qt, qb, g["qm"], g["rh"], 2 * N, 1)
    orad = oracle.scalar_lambert(km, 4, n, np.array(CH), N, 0, 2 * N, 1, g["ROT"], g["depol"], tau, ssa, gg, pm, g["pe"],
                                 g["he"], g["te"], g["albedo"], g["sza"], g["raa"], g["vza"], MISSING, nlay=nl)[0]
    rad, _, rc, _, st = vlidort.vlidort_scalar_lambert_batch(
        km, 4, n, N, 2 * N, nl, g["ROT"], g["depol"], tau.astype(np.float64), ssa.astype(np.float64),
        pm[..., 0].astype(np.float64), g["he"], g["albedo"], g["sza"], g["raa"], g["vza"], MISSING=MISSING,
        precision="mixed")
    cnt = ctypes.c_int()
    assert _lib.lib().aerort_refined_count(None, ctypes.byref(cnt)) == 0  # the last mixed call (host pointers)
    assert rc == 0 and np.all(st == 0)
    assert cnt.value >= 1
    assert np.max(np.abs(rad / orad - 1.0)) <= RTOL


@pytest.mark.gpu
@pytest.mark.parametrize("N,cols", [(12, [2130, 2277, 2227]), (16, [7090, 7683])])
def test_team_kernel_mixed_on_long_layer_chains(N, cols):
    # columns of the bench batch whose mixed radiance went wrong by up to 3e-3
    # when the FP32 team kernel warm-started each layer's Jacobi from the
    # previous layer's rotations (orthogonality lost along the layer chain)
    import bench
    L = _lib.lib()
    full = bench.make_batch(8192, seed=20261204)
    g = bench.subset(full, np.array(cols))
    assert np.all(g["nstreams"] == N)
    tabs = mie.generate_tables(CH, nmom=32)
    chem = mie.ChemMie(tabs)
    qt, qb = zip(*[chem.query_idx(x) for x in synth.tracer_names()])
    chem.destroy()
    km, n = g["km"], len(cols)
    nl = np.ascontiguousarray(g["nlayers"], np.int32)
    tau, ssa, gg, pm, rc = oracle.get_aop_vector(tabs, km, n, 4, 20, np.float32(CH), qt, qb, g["qm"], g["rh"], 2 * N, 1)
    orad = oracle.scalar_lambert(km, 4, n, np.array(CH), N, 0, 2 * N, 1, g["ROT"], g["depol"], tau, ssa, gg, pm, g["pe"],
                                 g["he"], g["te"], g["albedo"], g["sza"], g["raa"], g["vza"], MISSING, nlay=nl)[0]
    old = L.aerort_get_kernel(N, _lib.PREC_MIXED)
    assert L.aerort_set_kernel(N, _lib.PREC_MIXED, _lib.KERNEL_TEAM) == 0
    try:
        rad, _, rc, _, st = vlidort.vlidort_scalar_lambert_batch(
            km, 4, n, N, 2 * N, nl, g["ROT"], g["depol"], tau.astype(np.float64), ssa.astype(np.float64),
            pm[..., 0].astype(np.float64), g["he"], g["albedo"], g["sza"], g["raa"], g["vza"], MISSING=MISSING,
            precision="mixed")
    finally:
        L.aerort_set_kernel(N, _lib.PREC_MIXED, old)
    assert rc == 0 and np.all(st == 0)
    assert np.max(np.abs(rad / orad - 1.0)) <= RTOL


@pytest.mark.gpu
@pytest.mark.parametrize("N,lo", [(8, 0.0), (12, 0.0), (16, 0.0), (16, 0.999)])
def test_tensor_core_contraction(N, lo):
    # AERORT_CONTRACT_TF32X3: the FP32 team solve forms the layer matrices'
    # moment sums with mma.sync (3xTF32); same 1e-4 bar against the FP64 oracle
    L = _lib.lib()
    assert L.aerort_get_moment_contraction() == _lib.CONTRACT_FMA
    assert L.aerort_set_moment_contraction(7) != 0
    kern = L.aerort_get_kernel(N, _lib.PREC_MIXED)
    assert L.aerort_set_kernel(N, _lib.PREC_MIXED, _lib.KERNEL_TEAM) == 0
    try:
        assert L.aerort_set_moment_contraction(_lib.CONTRACT_TF32X3) == 0
        rng = (lo, 1.0) if lo > 0 else None
        c = random_aop_case(N, 72, nobs=24, nch=2, seed=N * 13 + 5, **({"ssa_range": rng} if rng else {}))
        rad, refl, rc, nf, st = _mixed(c, N)
    finally:
        L.aerort_set_moment_contraction(_lib.CONTRACT_FMA)
        L.aerort_set_kernel(N, _lib.PREC_MIXED, kern)
    orad, _, _, onf, ost = oracle.scalar_lambert(*rt_args(c, N), MISSING)
    assert rc == 0 and np.all(st == 0)
    ok = orad != MISSING
    err = np.abs(rad[ok] / orad[ok] - 1.0)
    assert err.max() <= RTOL, err.max()


@pytest.mark.gpu
def test_refined_solves_are_the_fp64_solves():
    # the FP64 re-solve of the refinement list (k_refine_terms: each solve's
    # Fourier terms spread over the warps of a block) gives the plain FP64
    # team solve's result: at least as many radiances agree with it to 1e-9,
    # with the same Fourier-term count, as were refined (an FP32 series is
    # 1e-7 away or more on these solves).  Not bit for bit: the same device
    # code inlined into two kernels may fuse multiply-adds differently, and a
    # listed solve's cancelling Fourier sum amplifies that (measured on the 8-
    # and 12-stream cases: 19 of the 20 listed solves within 1e-12).  The host build of the same
    # logic is bitwise the sequential series (test_rt_core_host.py).
    import ctypes
    import bench
    full = bench.make_batch(8192, seed=20261204)
    tabs = mie.generate_tables(CH, nmom=32)
    chem = mie.ChemMie(tabs)
    qt, qb = zip(*[chem.query_idx(x) for x in synth.tracer_names()])
    chem.destroy()
    total = 0
    for N in (8, 12, 16):
        g = bench.subset(full, np.nonzero(full["nstreams"] == N)[0][:600])
        km, n = g["km"], g["ncol"]
        nl = np.ascontiguousarray(g["nlayers"], np.int32)
        tau, ssa, gg, pm, rc = oracle.get_aop_vector(tabs, km, n, 4, 20, np.float32(CH), qt, qb, g["qm"], g["rh"],
                                                     2 * N, 1)
        args = (km, 4, n, N, 2 * N, nl, g["ROT"], g["depol"], tau.astype(np.float64), ssa.astype(np.float64),
                pm[..., 0].astype(np.float64), g["he"], g["albedo"], g["sza"], g["raa"], g["vza"])
        rm, _, rcm, nfm, stm = vlidort.vlidort_scalar_lambert_batch(*args, MISSING=MISSING, precision="mixed")
        cnt = ctypes.c_int()
        assert _lib.lib().aerort_refined_count(None, ctypes.byref(cnt)) == 0
        L = _lib.lib()
        kern = L.aerort_get_kernel(N, _lib.PREC_FP64)
        assert L.aerort_set_kernel(N, _lib.PREC_FP64, _lib.KERNEL_TEAM) == 0
        try:
            rd, _, rcd, nfd, std = vlidort.vlidort_scalar_lambert_batch(*args, MISSING=MISSING, precision="fp64")
        finally:
            L.aerort_set_kernel(N, _lib.PREC_FP64, kern)
        assert rcm == 0 and rcd == 0 and np.all(stm == 0) and np.all(std == 0)
        ok = rd != MISSING
        same = ok & (np.abs(np.where(ok, rm / np.where(ok, rd, 1.0), 1.0) - 1.0) < 1e-9) & (nfm == nfd)
        assert same.sum() >= cnt.value, (N, int(same.sum()), cnt.value)
        assert np.max(np.abs(rm[ok] / rd[ok] - 1.0)) <= RTOL
        total += cnt.value
    assert total > 0

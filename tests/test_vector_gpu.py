"""GPU parity of the polarized path (aerort_vlidort_vector_lambert*, NSTOKES = 3)
against the polarized oracle (oracle/vlidort_vector_oracle.cpp), which is
pinned to the reference's saved I/Q/U results (tests/test_oracle_golden_vector.py).

Inputs: synthetic columns with the six-element Mie optics of 20 aerosol
tracers (nPol = 6 Greek coefficients from Lorenz-Mie tables, mixed by the
oracle's VLIDORT_getAOPvector), Rayleigh optical depth and depolarisation.
Bar: identical Fourier-term counts and status codes; I within 1e-9 relative
(the plain-method bar); Q and U within 1e-9 of I (they pass through zero).
"""
import numpy as np
import pytest

from aeroapps_gb300 import VLIDORT_POLAR_, _lib, vlidort
from oracle import oracle

from rt_cases import MISSING, vector_mie_case

RTOL = 1e-9


def _oracle(c, N, alpha=None, flux=None):
    return oracle.vector_lambert(c["km"], c["nch"], c["ncol"], N, 0, c["nmom"], c["ROT"], c["depol"], alpha, c["tau"],
                                 c["ssa"], c["pmom"], c["he"], c["albedo"], c["sza"], c["raa"], c["vza"],
                                 c["flux"] if flux is None else flux, MISSING, nlay=c["nlayers"])


def _check(got, ref):
    rad, refl, q, u, nf, st = got
    orad, orefl, oq, ou, rc, onf, ost = ref
    assert rc == 0 and np.array_equal(st, ost) and np.array_equal(nf, onf)
    ok = orad != MISSING
    assert np.array_equal(rad == MISSING, ~ok)
    assert np.max(np.abs(rad[ok] / orad[ok] - 1.0)) <= RTOL
    assert np.max(np.abs(refl[ok] / orefl[ok] - 1.0)) <= RTOL
    assert np.max(np.abs(q[ok] - oq[ok]) / orad[ok]) <= RTOL
    assert np.max(np.abs(u[ok] - ou[ok]) / orad[ok]) <= RTOL


def _host_call(c, N, alpha=None, flux=None):
    km, nch, nobs = c["km"], c["nch"], c["ncol"]
    assert np.all(c["nlayers"] == km)
    rad, refl, q, u, rc, nf, st = vlidort.vlidort_vector_lambert(
        km, nch, nobs, c["channels"], N, 0, c["nmom"], 6, c["ROT"], c["depol"], alpha, c["tau"], c["ssa"], c["pmom"],
        c["pe"], c["he"], c["te"], c["albedo"], c["sza"], c["raa"], c["vza"], c["flux"] if flux is None else flux,
        MISSING=MISSING, diagnostics=True)
    assert rc == 0
    return rad, refl, q, u, nf, st


@pytest.mark.gpu
@pytest.mark.parametrize("N,nobs", [(4, 6), (8, 4), (12, 3)])
def test_vector_lambert_matches_oracle(N, nobs):
    c = vector_mie_case(N, nobs=nobs, nch=2, seed=100 + N)
    _check(_host_call(c, N), _oracle(c, N))


@pytest.mark.gpu
def test_vector_lambert_twelve_streams_sixty_four_moments():
    # the polarized workload's sizes: N = 12, 64 Greek coefficients (> 2N, so
    # delta-M truncates and the single scatter uses all 64), 72 layers
    N = 12
    c = vector_mie_case(N, nobs=2, nch=2, seed=64, nmom=64, chem_channels=(340.0, 2130.0))
    _check(_host_call(c, N), _oracle(c, N))


@pytest.mark.gpu
def test_vector_lambert_gas_absorption_flux_and_missing():
    # trace-gas absorption alpha, per-pixel flux factor, and one pixel with a
    # MISSING albedo and one with MISSING angles: all four outputs MISSING there
    N = 6
    c = vector_mie_case(N, nobs=5, nch=2, seed=31, nlayers=40)
    rng = np.random.default_rng(5)
    alpha = np.asfortranarray(0.02 * rng.random(c["ROT"].shape))
    flux = np.asfortranarray(rng.uniform(0.5, 2.0, (2, 5)))
    c["albedo"][1, 0] = MISSING
    c["sza"][3] = MISSING
    got = _host_call(c, N, alpha=alpha, flux=flux)
    ref = _oracle(c, N, alpha=alpha, flux=flux)
    _check(got, ref)
    for arr in got[:4]:
        assert arr[1, 0] == MISSING and np.all(arr[3, :] == MISSING)
    # without absorption the radiance changes (the argument is used)
    assert not np.allclose(_host_call(c, N, flux=flux)[0][0], got[0][0])


@pytest.mark.gpu
def test_f2py_vector_lambert_is_the_package_call():
    N = 4
    c = vector_mie_case(N, nobs=3, nch=1, seed=9, nlayers=30)
    rad, refl, q, u, rc = VLIDORT_POLAR_.vector_lambert(c["channels"], N, False, c["ROT"], c["depol"], None, c["tau"],
                                                        c["ssa"], c["pmom"], c["pe"], c["he"], c["te"], c["albedo"],
                                                        c["sza"], c["raa"], c["vza"], c["flux"], MISSING, 0)
    r2 = _host_call(c, N)
    assert rc == 0
    for a, b in zip((rad, refl, q, u), r2[:4]):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_batched_device_call_reads_fp32_optics_of_the_aop_kernel():
    # ragged columns, FP32 optics straight from the AOP kernel (nPol = 6): the
    # same radiances as the FP64 call on the converted optics
    import torch
    from aeroapps_gb300 import mie, synth
    N = 8
    rng = np.random.default_rng(12)
    nl = rng.integers(20, 73, 6).astype(np.int32)
    c = vector_mie_case(N, nobs=6, nch=2, seed=44, nlayers=nl)
    chem = mie.ChemMie(c["tables"])
    km, nch, nobs = c["km"], 2, 6
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    qm, rh = d(c["qm"], np.float32), d(c["rh"], np.float32)
    tau = torch.empty(km * nch * nobs, dtype=torch.float32, device="cuda")
    ssa, g = torch.empty_like(tau), torch.empty_like(tau)
    pm = torch.empty(km * nch * nobs * c["nmom"] * 6, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ch32 = np.float32(c["channels"])
    qt, qb = np.int32(c["qt"]), np.int32(c["qb"])
    L = _lib.lib()
    P = lambda t: t.data_ptr()
    rc = L.aerort_get_aop_vector_dev(chem.handle, km, nobs, nch, 20, _lib.ptr(ch32, _lib.P_f), _lib.ptr(qt, _lib.P_i),
                                     _lib.ptr(qb, _lib.P_i), P(qm), P(rh), c["nmom"], 6, P(tau), P(ssa), P(g), P(pm),
                                     stream)
    assert rc == 0, _lib.last_error()
    dv = {k: d(c[k], np.float64) for k in ("ROT", "depol", "he", "albedo", "sza", "raa", "vza", "flux")}
    nld = d(nl, np.int32)
    out = [torch.zeros(nobs * nch, dtype=torch.float64, device="cuda") for _ in range(4)]
    nf = torch.zeros(nobs * nch, dtype=torch.int32, device="cuda")
    st = torch.zeros_like(nf)
    rc = L.aerort_vlidort_vector_lambert_batch_dev(km, nch, nobs, N, 0, c["nmom"], P(nld), P(dv["ROT"]),
                                                   P(dv["depol"]), None, None, None, None, P(tau), P(ssa), P(pm),
                                                   P(dv["he"]), P(dv["albedo"]), P(dv["sza"]), P(dv["raa"]),
                                                   P(dv["vza"]), P(dv["flux"]), MISSING, *[P(o) for o in out], P(nf),
                                                   P(st), stream)
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    chem.destroy()
    # the AOP kernel is bit-identical to the oracle's, so the oracle run on the same optics is the reference
    assert np.array_equal(tau.cpu().numpy().reshape(km, nch, nobs, order="F"), c["tau32"])
    got = [o.cpu().numpy().reshape(nobs, nch, order="F") for o in out]
    got += [nf.cpu().numpy().reshape(nobs, nch, order="F"), st.cpu().numpy().reshape(nobs, nch, order="F")]
    _check(tuple(got), _oracle(c, N))

"""Edge profiles from layer fields: getEdgeVars
(src/Shared/GMAO_Shared/Chem_Base/MieObs_py.F90:27-83), FP32 like the reference.

CPU: the C oracle against an independent numpy restatement (pe, ze bit for
bit; te within 4 units in the last place, since logf/powf of different
libraries may differ in the last bits), hydrostatic physics, argument checks.
GPU: the device kernel through the C ABI against the oracle: pe and ze
bit-identical, te within 4 units in the last place, on ragged sizes, a layer
count whose tile needs more than 48 KB of shared memory, and the largest
supported one.  Parity unpinned: the reference keeps no saved edge profiles."""
import numpy as np
import pytest

from aeroapps_gb300 import _lib, mie, synth
from oracle import oracle

ULP_TOL = 4


def _layers(nobs, km, seed):
    """airdens (kg m-3) and delp (Pa), (km, nobs) REAL*4, of synthetic columns
    with top pressure 1 Pa."""
    c = synth.make_columns(nobs, [550.0], seed=seed, nlayers=min(km, 72))
    pe, te = c["pe"], c["te"]
    if km > 72:  # split every layer of a 72-layer column into equal parts
        f = -(-km // 72)
        t = np.linspace(0.0, 1.0, 72 * f + 1)
        src = np.linspace(0.0, 1.0, 73)
        pe = np.stack([np.interp(t, src, pe[:, j]) for j in range(nobs)], axis=1)[: km + 1]
        te = np.stack([np.interp(t, src, te[:, j]) for j in range(nobs)], axis=1)[: km + 1]
    dp = np.diff(pe, axis=0)
    pm = 0.5 * (pe[1:] + pe[:-1])
    tm = 0.5 * (te[1:] + te[:-1])
    rho = pm / (synth.RGAS * tm)
    return np.asfortranarray(rho, np.float32), np.asfortranarray(dp, np.float32), np.float32(pe[0, 0])


def _numpy_edge(rho, dp, ptop):
    km, nobs = rho.shape
    f = np.float32
    pe = np.zeros((km + 1, nobs), f)
    ze = np.zeros((km + 1, nobs), f)
    te = np.zeros((km + 1, nobs), f)
    pe[0] = ptop
    for k in range(km):
        pe[k + 1] = pe[k] + dp[k]
    for k in range(km - 1, -1, -1):
        ze[k] = ze[k + 1] + dp[k] / (rho[k] * f(9.80616))
    pm = (pe[:-1] + pe[1:]) / f(2.0)
    tm = pm / (rho * f(287.0))
    te[0] = tm[0]
    # logarithm and power in double, rounded once: within an ulp of any libm
    lg = lambda x: np.log(x.astype(np.float64)).astype(f)
    for k in range(1, km):
        alpha = lg(pe[k] / pm[k - 1]) / lg(pm[k] / pm[k - 1])
        te[k] = tm[k - 1] + alpha * (tm[k] - tm[k - 1])
    kappa = f(2.0) / f(7.0)
    te[km] = tm[km - 1] * ((pe[km] / pm[km - 1]).astype(np.float64) ** np.float64(kappa)).astype(f)
    return pe, ze, te


def _ulps(a, b):
    return np.max(np.abs(a.astype(np.float64) - b.astype(np.float64)) / np.spacing(np.abs(b)))


def test_oracle_matches_numpy_restatement():
    rho, dp, ptop = _layers(24, 72, seed=5)
    o = oracle.get_edge_vars(rho, dp, ptop)
    n = _numpy_edge(rho, dp, ptop)
    assert np.array_equal(o[0], n[0])
    assert np.array_equal(o[1], n[1])
    assert _ulps(o[2], n[2]) <= ULP_TOL


def test_oracle_physics():
    rho, dp, ptop = _layers(8, 72, seed=6)
    pe, ze, te = oracle.get_edge_vars(rho, dp, ptop)
    assert np.all(pe[0] == ptop) and np.all(np.diff(pe, axis=0) > 0)
    assert np.allclose(pe[-1], ptop + dp.astype(np.float64).sum(axis=0), rtol=1e-5)
    assert np.all(ze[-1] == 0.0) and np.all(np.diff(ze, axis=0) < 0)
    # top of a 1 Pa column: about 80 km; temperatures of a standard atmosphere
    assert np.all((ze[0] > 60e3) & (ze[0] < 100e3)), ze[0]
    assert np.all((te > 180.0) & (te < 320.0))


def test_edge_argument_checks_without_gpu():
    L = _lib.lib()
    assert L.aerort_get_edge_vars(0, 1, None, None, 1.0, None, None, None) == 1002
    assert L.aerort_get_edge_vars(533, 1, None, None, 1.0, None, None, None) == 3
    assert L.aerort_get_edge_vars(72, 1, None, None, 1.0, None, None, None) == 1002


@pytest.mark.gpu
@pytest.mark.parametrize("nobs,km", [(1, 72), (37, 72), (300, 47), (5, 1), (33, 130), (70, 318), (9, 532)])
def test_device_edge_vars_match_oracle(nobs, km):
    rho, dp, ptop = _layers(nobs, km, seed=nobs + km)
    o = oracle.get_edge_vars(rho, dp, ptop)
    g = mie.get_edge_vars(km, nobs, rho, dp, ptop)
    assert np.array_equal(g[0], o[0])
    assert np.array_equal(g[1], o[1])
    assert _ulps(g[2], o[2]) <= ULP_TOL


@pytest.mark.gpu
def test_device_edge_vars_dev_entry_point_on_a_stream():
    import torch
    nobs, km = 2000, 72
    rho, dp, ptop = _layers(nobs, km, seed=8)
    o = oracle.get_edge_vars(rho, dp, ptop)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
    drho, ddp = d(rho), d(dp)
    out = [torch.zeros((km + 1) * nobs, dtype=torch.float32, device="cuda") for _ in range(3)]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    rc = _lib.lib().aerort_get_edge_vars_dev(km, nobs, drho.data_ptr(), ddp.data_ptr(), float(ptop),
                                             *[x.data_ptr() for x in out], s.cuda_stream)
    assert rc == 0, _lib.last_error()
    s.synchronize()
    g = [x.cpu().numpy().reshape((km + 1, nobs), order="F") for x in out]
    assert np.array_equal(g[0], o[0]) and np.array_equal(g[1], o[1])
    assert _ulps(g[2], o[2]) <= ULP_TOL

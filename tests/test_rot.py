"""Rayleigh optical thickness calculator (VLIDORT_ROT_CALC,
geo_vlidort/VLIDORT_ROT.F90:19-86; VLIDORT_Rayleigh / coef_depol / F_air,
RTSI/VLIDORT2p8p3/VLIDORT_ScatMod.F90:145-283).

CPU: the C oracle against an independent numpy evaluation of the same
formulas (default-REAL literals as float32, all-literal subexpressions in
float32), bit for bit, plus the physics it must reproduce (a standard column's
ROT and the King-factor depolarisation of Bodhaine et al. 1999).
GPU: the device kernel through the C ABI, bit-identical to the oracle, on
synthetic GEOS-5 columns including ragged sizes.  Parity unpinned: the
reference keeps no saved ROT values."""
import numpy as np
import pytest

from aeroapps_gb300 import _lib, synth, vlidort
from oracle import oracle

CH = np.array([354.0, 388.0, 470.0, 550.0, 670.0, 865.0, 1020.0])


def f(x):
    return np.float64(np.float32(x))


def _numpy_rot(channels, pe, he, te):
    c = np.float64(np.float32(360.0) * np.float32(1e-6))
    ns = (f(6.0221367e23) / f(22.4141)) * (f(273.15) / f(288.15)) * np.float64(np.float32(1.0) / np.float32(1000))
    den_lit = np.float64((np.float32(78.084) + np.float32(20.946)) + np.float32(0.934))

    def king(xx2):
        d1 = f(1.034) + f(3.17e-4) * xx2
        d2 = f(1.096) + f(1.385e-3) * xx2 + f(1.448e-4) * xx2 * xx2
        return (f(78.084) * d1 + f(20.946) * d2 + f(0.934) * 1.0 + c * f(100.0) * f(1.15)) / (den_lit + c * f(100.0))

    km, nobs = pe.shape[0] - 1, pe.shape[1]
    rot = np.zeros((km, nobs, len(channels)), order="F")
    depol = np.zeros(len(channels))
    pi = np.float64(np.float32(np.pi))
    for i, lam in enumerate(channels):
        x = lam * f(1.0e-3)
        xx2 = (1.0 / x) * (1.0 / x)
        cm = x / f(10000.0)
        ri = f(8060.51) + f(2480990.0) / (f(132.274) - xx2) + f(17455.7) / (f(39.32957) - xx2)
        ri = ri * f(1e-8) + 1.0
        ri = (ri - 1.0) * (1.0 + f(0.54) * (c - f(0.0003))) + 1.0
        ri2 = ri * ri
        a = 24.0 * (pi * pi * pi) * king(xx2) * ((ri2 - 1) * (ri2 - 1)) / (
            ns * ns * cm * cm * cm * cm * (ri2 + 2) * (ri2 + 2))
        vol = a * ns * ((pe * f(1e-2)) / f(1013.25)) * (f(288.15) / te) * f(1e5)
        h = he * f(1e-3)
        rot[:, :, i] = (h[:-1] - h[1:]) * (vol[:-1] + vol[1:]) / 2.0
        kf = king(xx2)
        depol[i] = 6.0 * (kf - 1.0) / (7.0 * kf + 3.0)
    return rot, depol


def _columns(n, km=72, seed=3):
    cols = synth.make_columns(n, [550.0], seed=seed, nlayers=km)
    return cols["pe"], cols["he"], cols["te"]


def test_oracle_matches_independent_restatement_bitwise():
    pe, he, te = _columns(16)
    rot, depol, rc = oracle.rot_calc(CH, pe, he, te)
    assert rc == 0
    nrot, ndep = _numpy_rot(CH, pe, he, te)
    assert np.array_equal(rot, nrot)
    assert np.array_equal(depol, ndep)


def test_oracle_physics():
    pe, he, te = _columns(8)
    rot, depol, _ = oracle.rot_calc(CH, pe, he, te)
    ps = pe[-1] / 100.0  # hPa
    tau550 = rot[:, :, 3].sum(axis=0) * 1013.25 / ps
    # Bodhaine et al. (1999): tau_R(550 nm) ~ 0.097 for a 1013.25 hPa column
    assert np.all(np.abs(tau550 - 0.097) < 0.004), tau550
    # lambda^-4 dependence and King-factor depolarisation ~0.028 in the visible
    tsum = rot.sum(axis=0).mean(axis=0)
    assert np.all(np.diff(tsum) < 0)
    assert 3.6 < np.log(tsum[2] / tsum[5]) / np.log(CH[5] / CH[2]) < 4.3
    assert np.all((depol > 0.026) & (depol < 0.034))
    assert np.all(rot > 0)


@pytest.mark.gpu
@pytest.mark.parametrize("n,km", [(1, 72), (37, 72), (300, 47), (5, 1)])
def test_device_rot_bit_identical_to_oracle(n, km):
    pe, he, te = _columns(n, km=km, seed=n + km)
    orot, odep, orc = oracle.rot_calc(CH, pe, he, te)
    rot, depol, rc = vlidort.rot_calc(CH, pe, he, te, -1.0e15, 0)
    assert rc == 0 and orc == 0
    assert np.array_equal(rot, orot)
    assert np.array_equal(depol, odep)


@pytest.mark.gpu
def test_device_rot_dev_entry_point_on_a_stream():
    import torch
    pe, he, te = _columns(64, seed=9)
    orot, odep, _ = oracle.rot_calc(CH, pe, he, te)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float64).ravel(order="F"))).cuda()
    dch, dpe, dhe, dte = d(CH), d(pe), d(he), d(te)
    rot = torch.zeros(orot.size, dtype=torch.float64, device="cuda")
    dep = torch.zeros(len(CH), dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    rc = _lib.lib().aerort_vlidort_rot_calc_dev(72, len(CH), 64, dch.data_ptr(), dpe.data_ptr(), dhe.data_ptr(),
                                                dte.data_ptr(), rot.data_ptr(), dep.data_ptr(), s.cuda_stream)
    assert rc == 0, _lib.last_error()
    s.synchronize()
    assert np.array_equal(rot.cpu().numpy().reshape(orot.shape, order="F"), orot)
    assert np.array_equal(dep.cpu().numpy(), odep)


def test_rot_argument_checks_without_gpu():
    L = _lib.lib()
    assert L.aerort_vlidort_rot_calc(0, 1, 1, None, None, None, None, -1e15, 0, None, None) == 1002
    assert L.aerort_vlidort_rot_calc(72, 1, 1, None, None, None, None, -1e15, 0, None, None) == 1002

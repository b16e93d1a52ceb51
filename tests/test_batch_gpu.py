"""GPU parity of the batched entry points (columns with different layer
counts in one launch; FP32 optics read directly) against the oracle."""
import numpy as np
import pytest

from aeroapps_gb300 import _lib, mie, synth, vlidort
from oracle import oracle

CH = [470.0, 865.0]


def _case(N, ncol, seed):
    rng = np.random.default_rng(seed)
    nl = rng.integers(20, 73, ncol)
    cols = synth.make_columns(ncol, CH, seed=seed, nlayers=nl)
    tabs = mie.generate_tables(CH, nmom=2 * N)
    names = synth.tracer_names()
    chem = mie.ChemMie(tabs)
    qt, qb = zip(*[chem.query_idx(x) for x in names])
    tau, ssa, g, pm, rc = oracle.get_aop_vector(tabs, cols["km"], ncol, 2, 20, np.float32(CH), qt, qb, cols["qm"],
                                                cols["rh"], 2 * N, 1)
    assert rc == 0
    orad, orefl, orc, onf, ost = oracle.scalar_lambert(cols["km"], 2, ncol, np.array(CH), N, 0, 2 * N, 1, cols["ROT"],
                                                       cols["depol"], tau, ssa, g, pm, cols["pe"], cols["he"],
                                                       cols["te"], cols["albedo"], cols["sza"], cols["raa"],
                                                       cols["vza"], -1.0e15, nlay=nl)
    return cols, nl, chem, (tau, ssa, g, pm), (orad, onf, ost)


@pytest.mark.gpu
@pytest.mark.parametrize("N", [4, 12])
def test_host_batch_ragged_layers(N):
    cols, nl, chem, (tau, ssa, g, pm), (orad, onf, ost) = _case(N, 40, 100 + N)
    rad, refl, rc, nf, st = vlidort.vlidort_scalar_lambert_batch(
        cols["km"], 2, 40, N, 2 * N, nl, cols["ROT"], cols["depol"], tau, ssa, pm[..., 0], cols["he"], cols["albedo"],
        cols["sza"], cols["raa"], cols["vza"])
    chem.destroy()
    assert rc == 0 and np.array_equal(st, ost) and np.array_equal(nf, onf)
    assert np.max(np.abs(rad / orad - 1)) < 1e-9


@pytest.mark.gpu
def test_device_batch_with_fp32_optics_from_aop_kernel():
    import torch
    N, ncol = 8, 48
    cols, nl, chem, (tau, ssa, g, pm), (orad, onf, ost) = _case(N, ncol, 7)
    km = cols["km"]
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    qm, rh = d(cols["qm"], np.float32), d(cols["rh"], np.float32)
    t_ = torch.zeros(km * 2 * ncol, dtype=torch.float32, device="cuda")
    s_, g_ = torch.zeros_like(t_), torch.zeros_like(t_)
    p_ = torch.zeros(km * 2 * ncol * 2 * N, dtype=torch.float32, device="cuda")
    rad = torch.zeros(ncol * 2, dtype=torch.float64, device="cuda")
    refl, nf, st = torch.zeros_like(rad), torch.zeros(ncol * 2, dtype=torch.int32, device="cuda"), None
    st = torch.zeros_like(nf)
    names = synth.tracer_names()
    qt = np.array([chem.query_idx(x)[0] for x in names], np.int32)
    qb = np.array([chem.query_idx(x)[1] for x in names], np.int32)
    ch = np.float32(CH)
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.aerort_get_aop_vector_dev(chem.handle, km, ncol, 2, 20, _lib.ptr(ch, _lib.P_f), _lib.ptr(qt, _lib.P_i),
                                     _lib.ptr(qb, _lib.P_i), qm.data_ptr(), rh.data_ptr(), 2 * N, 1, t_.data_ptr(),
                                     s_.data_ptr(), g_.data_ptr(), p_.data_ptr(), stream)
    assert rc == 0
    dd = [d(cols[k], np.float64) for k in ("ROT", "depol", "he", "albedo", "sza", "raa", "vza")]
    nld = d(nl, np.int32)
    rc = L.aerort_vlidort_scalar_lambert_batch_dev(km, 2, ncol, N, 0, 2 * N, nld.data_ptr(), dd[0].data_ptr(),
                                                   dd[1].data_ptr(), None, None, None, t_.data_ptr(), s_.data_ptr(),
                                                   p_.data_ptr(), dd[2].data_ptr(), dd[3].data_ptr(), dd[4].data_ptr(),
                                                   dd[5].data_ptr(), dd[6].data_ptr(), -1.0e15, rad.data_ptr(),
                                                   refl.data_ptr(), nf.data_ptr(), st.data_ptr(), stream)
    assert rc == 0
    torch.cuda.synchronize()
    chem.destroy()
    r = rad.cpu().numpy().reshape(ncol, 2, order="F")
    assert np.array_equal(st.cpu().numpy().reshape(ncol, 2, order="F"), ost)
    assert np.array_equal(nf.cpu().numpy().reshape(ncol, 2, order="F"), onf)
    assert np.max(np.abs(r / orad - 1)) < 1e-9

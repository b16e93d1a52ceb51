"""The polarized warp solve of the CUDA kernel (aeroapps_gb300/csrc/rt_vector.cuh),
compiled for the host by this test only (one std::thread per lane), against
the polarized oracle: same Fourier-term counts, I within 1e-9 relative, Q and
U within 1e-9 of I.  This checks the GPU formulation (Hessenberg-QR
eigen-decomposition, Riccati boundary-value sweep, warp schedule) on the CPU;
tests/test_vector_gpu.py checks the kernel itself."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import oracle

from rt_cases import MISSING, vector_mie_case

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def vec_lib():
    d = tempfile.mkdtemp(prefix="aerort_vec_")
    so = os.path.join(d, "librtvec.so")
    subprocess.run(["g++", "-O1", "-std=c++20", "-pthread", "-fPIC", "-shared", "-o", so,
                    os.path.join(HERE, "host_harness", "rt_vector_host.cpp")], check=True)
    return ctypes.CDLL(so)


def _host(lib, c, N):
    km, nch, nobs = c["km"], c["nch"], c["ncol"]
    F = lambda a: np.asfortranarray(a, np.float64)
    keep = [F(c[k]) for k in ("ROT", "depol", "tau", "ssa", "pmom", "he", "albedo", "sza", "raa", "vza", "flux")]
    P = lambda a: None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    outs = [np.zeros((nobs, nch), order="F") for _ in range(4)]
    nf = np.zeros((nobs, nch), np.int32, order="F")
    st = np.zeros_like(nf)
    first = np.array([nobs], np.int32)
    nl = np.ascontiguousarray(c["nlayers"], np.int32)
    Ip = ctypes.POINTER(ctypes.c_int)
    args = [P(keep[0]), P(keep[1]), None] + [P(a) for a in keep[2:]]
    lib.host_vector_lambert(km, nch, nobs, N, c["nmom"], *args, first.ctypes.data_as(Ip), nl.ctypes.data_as(Ip),
                            ctypes.c_double(MISSING), -1, *[P(a) for a in outs], nf.ctypes.data_as(Ip),
                            st.ctypes.data_as(Ip))
    return outs, nf, st


def test_host_build_of_polarized_kernel_matches_oracle(vec_lib):
    N = 4
    c = vector_mie_case(N, nobs=2, nch=2, seed=7, nlayers=np.array([9, 6]))
    (rad, refl, q, u), nf, st = _host(vec_lib, c, N)
    orad, orefl, oq, ou, rc, onf, ost = oracle.vector_lambert(
        c["km"], 2, 2, N, 0, c["nmom"], c["ROT"], c["depol"], None, c["tau"], c["ssa"], c["pmom"], c["he"],
        c["albedo"], c["sza"], c["raa"], c["vza"], c["flux"], MISSING, nlay=c["nlayers"])
    assert rc == 0 and np.all(st == 0) and np.all(ost == 0)
    assert np.array_equal(nf, onf)
    assert np.max(np.abs(rad / orad - 1.0)) < 1e-9
    assert np.max(np.abs(q - oq) / orad) < 1e-9 and np.max(np.abs(u - ou) / orad) < 1e-9
    assert np.max(np.abs(refl / orefl - 1.0)) < 1e-9


def test_host_build_with_more_moments_than_streams(vec_lib):
    # nMom = 13 > 2N = 8: delta-M truncates at 2N-1 while the single scatter
    # (I, Q and U) uses every input Greek coefficient
    N = 4
    c = vector_mie_case(N, nobs=1, nch=2, seed=19, nlayers=np.array([7]), nmom=13)
    (rad, refl, q, u), nf, st = _host(vec_lib, c, N)
    orad, orefl, oq, ou, rc, onf, ost = oracle.vector_lambert(
        c["km"], 2, 1, N, 0, c["nmom"], c["ROT"], c["depol"], None, c["tau"], c["ssa"], c["pmom"], c["he"],
        c["albedo"], c["sza"], c["raa"], c["vza"], c["flux"], MISSING, nlay=c["nlayers"])
    assert rc == 0 and np.all(st == 0) and np.array_equal(nf, onf)
    assert np.max(np.abs(rad / orad - 1.0)) < 1e-9
    assert np.max(np.abs(q - oq) / orad) < 1e-9 and np.max(np.abs(u - ou) / orad) < 1e-9

"""The team kernel (one warp per solve for the Fourier series, shared-memory
working set) against the thread-per-solve kernel and the oracle, both
precisions, on ragged columns.  Bar: FP64 team within 1e-12 of FP64 thread
and 1e-9 of the oracle; mixed team within 1e-4 of the oracle; identical
status codes."""
import numpy as np
import pytest

from aeroapps_gb300 import _lib, vlidort
from oracle import oracle

from rt_cases import MISSING, random_aop_case, rt_args


def _run(c, N, nl, precision, kernel):
    L = _lib.lib()
    prec = _lib.PREC_MIXED if precision == "mixed" else _lib.PREC_FP64
    old = L.aerort_get_kernel(N, prec)
    assert L.aerort_set_kernel(N, prec, kernel) == 0
    try:
        return vlidort.vlidort_scalar_lambert_batch(c["km"], c["nch"], c["ncol"], N, c["nmom"], nl, c["ROT"],
                                                    c["depol"], c["tau"], c["ssa"], c["pmom"][..., 0], c["he"],
                                                    c["albedo"], c["sza"], c["raa"], c["vza"], MISSING=MISSING,
                                                    precision=precision)
    finally:
        L.aerort_set_kernel(N, prec, old)


@pytest.mark.gpu
@pytest.mark.parametrize("N", [4, 8, 12, 16])
def test_team_matches_thread_and_oracle(N):
    c = random_aop_case(N, 48, nobs=70, nch=2, seed=900 + N)
    nl = np.random.default_rng(N).integers(1, 49, c["ncol"]).astype(np.int32)
    nl[0] = 48
    orad, _, _, onf, ost = oracle.scalar_lambert(*rt_args(c, N), MISSING, nlay=nl)
    rt, _, rc1, nft, stt = _run(c, N, nl, "fp64", _lib.KERNEL_TEAM)
    rp, _, rc2, nfp, stp = _run(c, N, nl, "fp64", _lib.KERNEL_THREAD)
    assert rc1 == 0 and rc2 == 0
    assert np.array_equal(stt, stp) and np.array_equal(stt, ost)
    assert np.array_equal(nft, nfp) and np.array_equal(nft, onf)
    assert np.max(np.abs(rt / rp - 1.0)) <= 1e-12
    assert np.max(np.abs(rt / orad - 1.0)) <= 1e-9
    rm, _, rc3, _, stm = _run(c, N, nl, "mixed", _lib.KERNEL_TEAM)
    assert rc3 == 0 and np.all(stm == 0)
    assert np.max(np.abs(rm / orad - 1.0)) <= 1e-4


def test_kernel_api_validates():
    L = _lib.lib()
    assert L.aerort_set_kernel(7, 0, 0) == 1003
    assert L.aerort_set_kernel(8, 0, 4) == 1002
    assert L.aerort_set_kernel(8, 0, _lib.KERNEL_TERMS) == 0 and L.aerort_get_kernel(8, 0) == _lib.KERNEL_TERMS
    assert L.aerort_set_kernel(8, 0, _lib.KERNEL_AUTO) == 0
    assert all(L.aerort_get_kernel(n, p) == _lib.KERNEL_AUTO for n in (4, 6, 8, 12, 16) for p in (0, 1))
    assert L.aerort_set_kernel(8, 1, _lib.KERNEL_TEAM) == 0 and L.aerort_get_kernel(8, 1) == _lib.KERNEL_TEAM
    assert L.aerort_set_kernel(8, 1, _lib.KERNEL_AUTO) == 0 and L.aerort_get_kernel(8, 1) == _lib.KERNEL_AUTO


@pytest.mark.gpu
@pytest.mark.parametrize("N", [4, 8, 12, 16])
def test_term_parallel_solve_matches_team_and_oracle(N):
    # AERORT_KERNEL_TERMS: each solve's Fourier terms spread over the warps of
    # a block (k_refine_terms), on ragged columns: the team solve's Fourier
    # terms and status, radiance within 1e-12 of it and 1e-9 of the oracle;
    # a mixed call with this choice runs the team kernel
    c = random_aop_case(N, 40, nobs=30, nch=2, seed=950 + N)
    nl = np.random.default_rng(N + 3).integers(1, 41, c["ncol"]).astype(np.int32)
    nl[0] = 40
    orad, _, _, onf, ost = oracle.scalar_lambert(*rt_args(c, N), MISSING, nlay=nl)
    rt, _, rc1, nft, stt = _run(c, N, nl, "fp64", _lib.KERNEL_TEAM)
    rp, _, rc2, nfp, stp = _run(c, N, nl, "fp64", _lib.KERNEL_TERMS)
    assert rc1 == 0 and rc2 == 0
    assert np.array_equal(stp, stt) and np.array_equal(stp, ost)
    assert np.array_equal(nfp, nft) and np.array_equal(nfp, onf)
    ok = orad != MISSING
    assert np.max(np.abs(rp[ok] / rt[ok] - 1.0)) <= 1e-12
    assert np.max(np.abs(rp[ok] / orad[ok] - 1.0)) <= 1e-9
    rm, _, rc3, _, stm = _run(c, N, nl, "mixed", _lib.KERNEL_TERMS)
    assert rc3 == 0 and np.all(stm == ost)
    assert np.max(np.abs(rm[ok] / orad[ok] - 1.0)) <= 1e-4

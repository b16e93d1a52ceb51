"""The f2py-compatible VLIDORT_POLAR_ module (aeroapps_gb300/VLIDORT_POLAR_.py),
called the way leo_vlidort's Python drivers call the reference's f2py module
(VLIDORT_POLAR_py.F90: ROT_CALC, SCALAR_LAMBERT).

CPU: size checks and the entries that are not provided.  GPU: results
identical to the package's own entry points, and to the oracle within the
plain-method bar."""
import numpy as np
import pytest

from aeroapps_gb300 import VLIDORT_POLAR_, synth, vlidort
from oracle import oracle

from rt_cases import MISSING, random_aop_case, rt_args


def _f2py_args(c, nstreams):
    return (c["channels"], nstreams, False, c["ROT"], c["depol"], c["tau"], c["ssa"], c["g"], c["pmom"], c["pe"],
            c["he"], c["te"], c["albedo"], c["sza"], c["raa"], c["vza"], MISSING, 0)


def test_sizes_and_missing_entries():
    c = random_aop_case(8, 12, nobs=3, seed=4)
    with pytest.raises(ValueError):
        VLIDORT_POLAR_.scalar_lambert(*_f2py_args(c, 8), km=c["km"] + 1)
    with pytest.raises(ValueError):
        VLIDORT_POLAR_.scalar_lambert(*_f2py_args(c, 8), nmom=c["nmom"] + 1)
    # the BRDF, ocean and cloud entries are not provided: a call fails loudly
    for name in ("vector_brdf_modis", "vector_cx", "vector_lambert_cloud"):
        assert not hasattr(VLIDORT_POLAR_, name)


@pytest.mark.gpu
def test_f2py_calls_match_package_entry_points_and_oracle():
    N = 8
    c = random_aop_case(N, 30, nobs=6, seed=12)
    rad, refl, rc = VLIDORT_POLAR_.scalar_lambert(*_f2py_args(c, N))
    r2, f2, rc2 = vlidort.vlidort_scalar_lambert(*rt_args(c, N), MISSING, 0)
    assert rc == rc2 == 0
    assert np.array_equal(rad, r2) and np.array_equal(refl, f2)
    o = oracle.scalar_lambert(*rt_args(c, N), MISSING)
    ok = o[0] != MISSING
    assert np.max(np.abs(rad[ok] / o[0][ok] - 1.0)) <= 1e-8  # the bar against the oracle at ASYMTX tolerance 1e-12
    cols = synth.make_columns(5, [470.0, 550.0], seed=3)
    rot, depol, rrc = VLIDORT_POLAR_.rot_calc(np.array([470.0, 550.0]), cols["pe"], cols["he"], cols["te"], MISSING, 0)
    orot, odep, _ = oracle.rot_calc(np.array([470.0, 550.0]), cols["pe"], cols["he"], cols["te"])
    assert rrc == 0 and np.array_equal(rot, orot) and np.array_equal(depol, odep)

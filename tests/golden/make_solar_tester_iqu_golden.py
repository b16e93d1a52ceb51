"""Build tests/golden/solar_tester_iqu.json from the reference's own polarized
VLIDORT test data.

Run with the path of an AeroApps checkout as the only argument
(`python make_solar_tester_iqu_golden.py <aeroapps-tree>`).  It reads

  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/input_atmos.dat
  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/ProblemIII.Moms
  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/saved_results/gfortran/nstokes3/results_solar_tester_IQU0.all
  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/saved_results/gfortran/results_solar_tester_I000.all

and reproduces, in double precision, the atmosphere the reference's vector
solar tester builds (vlidort_v_test/V2p8p3_solar_tester.f90:206-410):
- 23 Rayleigh layers with the Rayleigh Greek coefficients of the tester
  (PROBLEM_RAY: beta0 = 1, beta2, gamma2 = -sqrt(6) beta2, alpha2 = 6 beta2,
  beta2 from the bottom layer), entries masked by GMASK/RMASK (:208-209);
- a Mie aerosol (ProblemIII.Moms, six expansion coefficients read up to the
  tester's 1e-6 cutoff, mapped by CMASK/SMASK, :211-212) with tau = 0.5 and
  omega = 0.99999 spread over the lowest 6 layers;
- Lambertian albedo 0.05, flux factor 1, 8 streams, ASYMTX tolerance 1e-20,
  lattice geometry 4 SZA x 3 VZA x 3 RAA (V2p8p3_VLIDORT_ReadInput.cfg).
The expected values are the gfortran TOA-upwelling Stokes I, Q, U of the 36
geometries for tasks 1-4 (NSTOKES = 3), and Stokes I of the same tasks with
NSTOKES = 1 through the vector code.  The JSON is small and is committed; the
GPU machine never reads the reference tree.
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python %s <path of an AeroApps checkout>" % os.path.basename(__file__))
REF = sys.argv[1]
BASE = os.path.join(REF, "src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test")

GMASK = (1, 2, 5, 6, 11, 12, 15, 16)
RMASK = (1, 5, 5, 2, 3, 6, 6, 4)
CMASK = (1, 2, 2, 3, 4, 5, 5, 6)
SMASK = (1, -1, -1, 1, 1, -1, 1, 1)


def read_moms(path):
    """The six expansion coefficients per moment, with the tester's stopping rule (:294-318)."""
    lines = open(path).read().splitlines()[5:]
    moms, lcheck = [], 0
    for ln in lines:
        if len(moms) >= 107 or lcheck >= 2:
            break
        v = [float(x) for x in ln.split()[1:7]]
        if v[0] > 1.0e-6:
            moms.append(v)
            if lcheck == 1:
                lcheck += 1
        else:
            lcheck += 1
            if lcheck == 1:
                moms.append(v)
    return moms


def read_block(path, title):
    """TOA-upwelling values per geometry (tasks 1-6) of one STOKES block."""
    out, inside = {}, False
    for ln in open(path).read().splitlines():
        if "STOKES-" in ln:
            inside = (title in ln)
            continue
        if not inside:
            continue
        p = ln.split()
        if len(p) >= 10 and p[1] == "Upwelling" and p[3] == "0.00":
            out[int(p[0])] = [float(x) for x in p[4:10]]
    return out


def atmosphere(nstokes):
    lines = open(os.path.join(BASE, "input_atmos.dat")).read().splitlines()
    nlayers = 23
    raymoms = [[float(x) for x in lines[r].split()[1:]][:nlayers] for r in range(3)]
    height = [60.0]
    molext, molomg = [], []
    for n in range(nlayers):
        parts = lines[3 + n].split()
        height.append(float(parts[1]))
        molext.append(float(parts[2]))
        molomg.append(float(parts[3]))
    moms = read_moms(os.path.join(BASE, "ProblemIII.Moms"))
    ngreek = len(moms) - 1
    beta2 = raymoms[2][nlayers - 1]
    depol = (1.0 - 2.0 * beta2) / (1.0 + beta2)
    ray = [[0.0] * 3 for _ in range(6)]  # PROBLEM_RAY(row 1..6, L 0..2)
    ray[0][0] = 1.0
    ray[3][1] = 3.0 * (1.0 - 2.0 * depol) / (2.0 + depol)
    ray[0][2] = beta2
    ray[4][2] = -(6.0 ** 0.5) * beta2
    ray[1][2] = 6.0 * beta2
    nent = {1: 1, 3: 5, 4: 8}[nstokes]
    n6 = nlayers - 6
    deltau, omega = [], []
    greek = [[[0.0] * (ngreek + 1) for _ in range(16)] for _ in range(nlayers)]
    for n in range(n6):
        deltau.append(molext[n])
        omega.append(molomg[n])
        for k in range(nent):
            gk, rk = GMASK[k] - 1, RMASK[k] - 1
            for l in range(3):
                greek[n][gk][l] = ray[rk][l]
        greek[n][0][0] = 1.0
    waer, taer = 0.99999, 0.5
    parcel = taer / (height[n6] - height[nlayers])
    for n in range(n6 + 1, nlayers + 1):
        i = n - 1
        aerext = parcel * (height[n - 1] - height[n])
        aersca = aerext * waer
        molsca = molomg[i] * molext[i]
        totext = molext[i] + aerext
        totsca = molsca + aersca
        raywt = molsca / totsca
        aerwt = aersca / totsca
        deltau.append(totext)
        omega.append(totsca / totext)
        for k in range(nent):
            gk, sk, ck, rk = GMASK[k] - 1, float(SMASK[k]), CMASK[k] - 1, RMASK[k] - 1
            for l in range(3):
                greek[i][gk][l] = raywt * ray[rk][l] + aerwt * sk * moms[l][ck]
            for l in range(3, ngreek + 1):
                greek[i][gk][l] = aerwt * sk * moms[l][ck]
        greek[i][0][0] = 1.0
    return height, deltau, omega, greek, ngreek


def main():
    height, deltau, omega, greek3, ngreek = atmosphere(3)
    _, _, _, greek1, _ = atmosphere(1)
    sv = os.path.join(BASE, "saved_results/gfortran")
    iqu = os.path.join(sv, "nstokes3/results_solar_tester_IQU0.all")
    i000 = os.path.join(sv, "results_solar_tester_I000.all")
    I3, Q3, U3 = read_block(iqu, "STOKES-I"), read_block(iqu, "STOKES-Q"), read_block(iqu, "STOKES-U")
    I1 = read_block(i000, "STOKES-I")
    szas, vzas, raas = [35.0, 67.0, 75.0, 82.0], [10.0, 20.0, 40.0], [10.0, 90.0, 170.0]
    out = {
        "source": "vlidort_v_test/saved_results/gfortran/nstokes3/results_solar_tester_IQU0.all and "
                  "results_solar_tester_I000.all (reference VLIDORT 2.8.3)",
        "nstreams": 8, "nlayers": 23, "ngreek": ngreek, "albedo": 0.05, "accuracy": 1.0e-4, "asymtx_tol": 1.0e-20,
        "taylor_order": 3, "earth_radius": 6371.0, "flux_factor": 1.0,
        "heights": height, "deltau": deltau, "omega": omega, "greek_nstokes3": greek3, "greek_nstokes1": greek1,
        "szas": szas, "vzas": vzas, "raas": raas,
        "tasks": {
            "1": {"do_focorr": 0, "do_focorr_nadir": 0, "do_focorr_outgoing": 0, "do_deltam": 0, "nfinelayers": 0},
            "2": {"do_focorr": 0, "do_focorr_nadir": 0, "do_focorr_outgoing": 0, "do_deltam": 1, "nfinelayers": 0},
            "3": {"do_focorr": 1, "do_focorr_nadir": 1, "do_focorr_outgoing": 0, "do_deltam": 1, "nfinelayers": 0},
            "4": {"do_focorr": 1, "do_focorr_nadir": 0, "do_focorr_outgoing": 1, "do_deltam": 1, "nfinelayers": 4},
        },
        "toa_up_I": {str(k): v[:4] for k, v in sorted(I3.items())},
        "toa_up_Q": {str(k): v[:4] for k, v in sorted(Q3.items())},
        "toa_up_U": {str(k): v[:4] for k, v in sorted(U3.items())},
        "toa_up_I_nstokes1": {str(k): v[:4] for k, v in sorted(I1.items())},
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "solar_tester_iqu.json")
    with open(dst, "w") as f:
        json.dump(out, f)
    print(dst, "ngreek", ngreek, "geometries", len(I3), len(Q3), len(U3), len(I1))


if __name__ == "__main__":
    main()

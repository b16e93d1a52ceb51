"""Build tests/golden/obsgeo_lpcs.json from the reference's own VLIDORT test data.

Run with the path of an AeroApps checkout as the only argument
(`python make_obsgeo_golden.py <aeroapps-tree>`).  It reads

  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/input_atmos.dat
  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/ProblemIII.Moms
  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/config/obsgeo/V2p8p3_VLIDORT_ReadInput.cfg_obsgeo (values below)
  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/saved_results/gfortran/obsgeo/results_solar_lps_tester_obsgeo_I000.all

and reproduces, in double precision and for NSTOKES = 1, the atmosphere the
reference's linearized solar tester builds in observation-geometry mode
(vlidort_v_test/V2p8p3_solar_lpcs_tester.f90:448-600):
- 23 Rayleigh layers, the Rayleigh phase moments (1, 0, beta2) with beta2 from
  the bottom layer;
- a Mie aerosol (ProblemIII.Moms, a1 column, read up to the reference's 1e-6
  cutoff) with tau = 0.5 and omega = 0.99999 spread over the lowest 6 layers;
- Lambertian albedo 0.05 and flux factor 1e-3.
The configuration is 8 streams, delta-M, pseudo-spherical, double convergence
test at 1e-4, ASYMTX tolerance 1e-20, and the FO single-scatter correction in
its regular pseudo-spherical form (the tester sets DO_FOCORR and
DO_FOCORR_NADIR itself, :392-405, overriding the configuration file).  The expected values
are the gfortran TOA-upwelling Stokes-I numbers of the three observation
geometries (SZA, VZA, RAA) = (35, 10, 10), (67, 20, 90), (75, 40, 170).
The JSON is small and is committed; the GPU machine never reads the reference tree.
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python %s <path of an AeroApps checkout>" % os.path.basename(__file__))
REF = sys.argv[1]
BASE = os.path.join(REF, "src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test")


def read_a1(path):
    """The a1 (P11) expansion coefficients, with the tester's stopping rule (:463-483)."""
    lines = open(path).read().splitlines()[5:]
    a1, lcheck = [], 0
    for ln in lines:
        if len(a1) >= 107 or lcheck >= 2:
            break
        v = float(ln.split()[1])
        if v > 1.0e-6:
            a1.append(v)
            if lcheck == 1:
                lcheck += 1
        else:
            lcheck += 1
            if lcheck == 1:
                a1.append(v)
    return a1


def main():
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
    a1 = read_a1(os.path.join(BASE, "ProblemIII.Moms"))
    ngreek = len(a1) - 1
    beta2 = raymoms[2][nlayers - 1]
    ray = [1.0, 0.0, beta2]
    n6 = nlayers - 6
    deltau, omega, greek = [], [], []
    for n in range(n6):
        deltau.append(molext[n])
        omega.append(molomg[n])
        g = [0.0] * (ngreek + 1)
        g[0], g[1], g[2] = ray
        greek.append(g)
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
        g = [0.0] * (ngreek + 1)
        for l in range(3):
            g[l] = raywt * ray[l] + aerwt * a1[l]
        for l in range(3, ngreek + 1):
            g[l] = aerwt * a1[l]
        g[0] = 1.0
        greek.append(g)
    res = open(os.path.join(BASE, "saved_results/gfortran/obsgeo/results_solar_lps_tester_obsgeo_I000.all"))
    toa = {}
    for ln in res.read().splitlines():
        p = ln.split()
        if len(p) >= 5 and p[1] == "Upwelling" and p[3] == "0.00" and int(p[0]) not in toa:
            toa[int(p[0])] = float(p[4])
    out = {
        "source": "vlidort_v_test/saved_results/gfortran/obsgeo/results_solar_lps_tester_obsgeo_I000.all",
        "nstreams": 8, "albedo": 0.05, "flux_factor": 1.0e-3, "accuracy": 1.0e-4, "asymtx_tol": 1.0e-20,
        "taylor_order": 3, "earth_radius": 6371.0, "ngreek": ngreek,
        "flags": {"do_focorr": 1, "do_focorr_nadir": 1, "do_focorr_outgoing": 0, "do_deltam": 1, "nfinelayers": 4},
        "heights": height, "deltau": deltau, "omega": omega, "greek": greek,
        "geometries": [[35.0, 10.0, 10.0], [67.0, 20.0, 90.0], [75.0, 40.0, 170.0]],
        "toa_up_I": [toa[1], toa[2], toa[3]],
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "obsgeo_lpcs.json")
    with open(dst, "w") as f:
        json.dump(out, f)
    print(dst, "ngreek", ngreek, "toa", out["toa_up_I"])


if __name__ == "__main__":
    main()

"""Build tests/golden/solar_tester.json from the reference's own VLIDORT test data.

Run with the path of an AeroApps checkout as the only argument
(`python make_solar_tester_golden.py <aeroapps-tree>`).  It reads

  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_s_test/input_atmos.dat
  src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_s_test/saved_results/gfortran/results_solar_tester.all

and reproduces, in double precision, the atmosphere the reference scalar solar
tester builds (vlidort_s_test/2p8p3_solar_tester.f90:245-320: 23 Rayleigh
layers, aerosol tau=0.5 / omega=0.95 spread over the lowest 6 layers, 80
Henyey-Greenstein moments with g=0.8, Lambertian albedo 0.05).  The expected
values are the gfortran TOA-upwelling Stokes-I numbers for the 36 lattice
geometries (4 SZA x 3 VZA x 3 RAA) and tasks 1-6.  The JSON is small and is
committed; the GPU machine never reads the reference tree.
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python %s <path of an AeroApps checkout>" % os.path.basename(__file__))
REF = sys.argv[1]
BASE = os.path.join(REF, "src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_s_test")


def main():
    lines = open(os.path.join(BASE, "input_atmos.dat")).read().splitlines()
    nlayers = 23
    raymoms = []
    for r in range(3):
        vals = [float(x) for x in lines[r].split()[1:]]
        raymoms.append(vals[:nlayers])
    height = [60.0]
    molext, molomg = [], []
    for n in range(nlayers):
        parts = lines[3 + n].split()
        height.append(float(parts[1]))
        molext.append(float(parts[2]))
        molomg.append(float(parts[3]))
    # aerosol in the bottom 6 layers (2p8p3_solar_tester.f90:266-320)
    n6 = nlayers - 6
    waer, taer, gaer, ngreek = 0.95, 0.5, 0.8, 80
    aermoms = [1.0] + [float(2 * l + 1) * gaer ** float(l) for l in range(1, ngreek + 1)]
    deltau, omega = [], []
    greek = []  # greek[n][l]
    for n in range(n6):
        deltau.append(molext[n])
        omega.append(molomg[n])
        g = [0.0] * (ngreek + 1)
        for l in range(3):
            g[l] = raymoms[l][n]
        greek.append(g)
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
            g[l] = raywt * raymoms[l][i] + aerwt * aermoms[l]
        for l in range(3, ngreek + 1):
            g[l] = aerwt * aermoms[l]
        greek.append(g)
    # expected TOA upwelling (level 0.00) per geometry, tasks 1..6
    res = open(os.path.join(BASE, "saved_results/gfortran/results_solar_tester.all")).read().splitlines()
    toa = {}
    for ln in res:
        p = ln.split()
        if len(p) >= 10 and p[1] == "Upwelling" and p[3] == "0.00":
            toa[int(p[0])] = [float(x) for x in p[4:10]]
    geoms = []
    szas, vzas, raas = [35.0, 67.0, 75.0, 82.0], [10.0, 20.0, 40.0], [0.0, 90.0, 180.0]
    for ib, s in enumerate(szas):
        for um, v in enumerate(vzas):
            for ua, a in enumerate(raas):
                geoms.append({"index": ib * 9 + um * 3 + ua + 1, "sza": s, "vza": v, "raa": a})
    out = {
        "source": "vlidort_s_test/saved_results/gfortran/results_solar_tester.all (reference VLIDORT 2.8.3)",
        "nstreams": 8, "nlayers": nlayers, "ngreek": ngreek, "albedo": 0.05,
        "accuracy": 1.0e-4, "asymtx_tol": 1.0e-20, "taylor_order": 3, "earth_radius": 6371.0,
        "flux_factor": 1.0,
        "heights": height, "deltau": deltau, "omega": omega, "greek": greek,
        "szas": szas, "vzas": vzas, "raas": raas, "geometries": geoms,
        "tasks": {
            "1": {"do_focorr": 0, "do_focorr_nadir": 0, "do_focorr_outgoing": 0, "do_deltam": 0, "nfinelayers": 0},
            "2": {"do_focorr": 0, "do_focorr_nadir": 0, "do_focorr_outgoing": 0, "do_deltam": 1, "nfinelayers": 0},
            "3": {"do_focorr": 1, "do_focorr_nadir": 1, "do_focorr_outgoing": 0, "do_deltam": 1, "nfinelayers": 4},
            "4": {"do_focorr": 1, "do_focorr_nadir": 0, "do_focorr_outgoing": 1, "do_deltam": 1, "nfinelayers": 4},
        },
        "toa_up": {str(k): v for k, v in sorted(toa.items())},
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "solar_tester.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, len(toa), "geometries")


if __name__ == "__main__":
    main()

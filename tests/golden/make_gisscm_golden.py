"""Build tests/golden/brdf_gisscm_selftest.json from the reference's saved
GISS Cox-Munk BRDF results.

Run with the path of an AeroApps checkout as the only argument
(`python make_gisscm_golden.py <aeroapps-tree>`).  It reads, under
src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/,

  VBRDF_ReadInput_self_test.cfg                  the inputs of the BRDF self tester
  saved_results/gfortran/results_brdf_self_tester.res

The self tester (V2p8p3_brdf_self_tester.f90) reads that configuration (1
quadrature stream, 100 BRDF azimuth streams, NSTOKES = 3, one solar beam of
35 deg, one view of 10 deg, relative azimuths 0, 79, 180 deg) and then sets
the kernel itself in GET_VBRDF_PLUS (:1051-1066 and the GISS Cox-Munk branch):
index 10, amplitude 1, slope parameter sigma^2 / 2 with sigma^2 = 0.003 +
0.00512 x 15 m/s, real refractive index of sea water at 0.5 um and salinity
34.3 ppt from VBRDF_Water_RefracIndex (vsup/vbrdf/vbrdf_sup_kernels.f90
:3814-3921, single-precision table lookup: 1.335 + 0.006), shadowing on.  The
first result block of results_brdf_self_tester.res is that kernel's exact
direct-bounce BRDF and Fourier components m = 0, 1 (stream-stream,
solar-stream, stream-user, solar-user); this keeps their (1,1) elements, the
scalar BRDF.  The JSON is small and is committed; the GPU machine never reads the
reference tree.
"""
import json
import os
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: python %s <path of an AeroApps checkout>" % os.path.basename(__file__))
BASE = os.path.join(sys.argv[1], "src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test")


def read_cfg():
    lines = open(os.path.join(BASE, "VBRDF_ReadInput_self_test.cfg")).read().splitlines()

    def after(title):
        for i, ln in enumerate(lines):
            if ln.strip().startswith(title):
                return i + 1
        raise KeyError(title)

    def values(title, n):
        i = after(title)
        return [float(lines[i + k].split()[0].rstrip(",")) for k in range(n)]
    out = {"nstreams": int(lines[after("BRDFSUP - Number of half-space streams")].split()[0]),
           "nstreams_brdf": int(lines[after("BRDFSUP - Number of BRDF azimuth angles")].split()[0]),
           "shadow": lines[after("BRDFSUP - Do shadow effect for glitter kernels?")].strip().lower().startswith("t")}
    nb = int(lines[after("BRDFSUP - Number of solar zenith angles")].split()[0])
    na = int(lines[after("BRDFSUP - Number of user-defined relative azimuth angles")].split()[0])
    nu = int(lines[after("BRDFSUP - Number of user-defined viewing zenith angles")].split()[0])
    out["szas"] = values("BRDFSUP - Solar zenith angles (degrees)", nb)
    out["raas"] = values("BRDFSUP - User-defined relative azimuth angles (degrees)", na)
    out["vzas"] = values("BRDFSUP - User-defined viewing zenith angles (degrees)", nu)
    # the GISS Cox-Munk settings of GET_VBRDF_PLUS (the configuration's kernel
    # line and shadow flag are overridden there)
    sigma_sq = 0.003 + 0.00512 * 15.0
    refrac_r = float(np.float32(np.float32(1.335) + np.float32(0.006) * (np.float32(34.3) / np.float32(34.3))))
    out["kernel"] = {"name": "GissCoxMnk", "which": 10, "factor": 1.0, "pars": [0.5 * sigma_sq, refrac_r, 0.0]}
    out["shadow"] = True
    return out


def read_results():
    lines = open(os.path.join(BASE, "saved_results/gfortran/results_brdf_self_tester.res")).read().splitlines()
    exact, four, m = [], {}, None
    blocks = 0
    for ln in lines:
        t = ln.split()
        if "Exact BRDF, all geometries" in ln:
            blocks += 1
            if blocks > 1:
                break
            continue
        if blocks == 0:
            continue
        if ln.strip().startswith("Fourier component #"):
            m = int(t[-1])
            four[m] = {}
            continue
        if m is None and len(t) >= 6 and all(x.isdigit() for x in t[:3]):
            exact.append(float(t[3]))
        for key in ("Stream-Stream", "Solars-Stream", "Stream-Users", "Solars-Users"):
            if m is not None and ln.strip().startswith(key):
                four[m][key] = float(t[3])
    return exact, four


def main():
    out = read_cfg()
    exact, four = read_results()
    out["exact"] = exact
    out["fourier"] = {str(k): v for k, v in sorted(four.items())}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "brdf_gisscm_selftest.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, out)


main()

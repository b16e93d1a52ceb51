"""Build tests/golden/brdf_selftest_scalar.json from the reference's saved
scalar BRDF self-test results.

Run with the path of an AeroApps checkout as the only argument
(`python make_brdf_selftest_golden.py <aeroapps-tree>`).  It reads, under
src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_s_test/,

  VBRDF_ReadInput_self_test.cfg                  the inputs of the BRDF self tester
  saved_results/gfortran/results_brdf_self_tester.res

The scalar self tester (2p8p3_brdf_self_tester.f90) reads that configuration
(1 quadrature stream, 100 BRDF azimuth streams, NSTOKES = 1, one solar beam of
35 deg, one view of 10 deg, relative azimuths 0, 79, 180 deg) and then, for
each kernel index, sets the kernel in GET_VBRDF_PLUS (:1008-1445): Lambertian
with albedo 0.1; Ross-thin, Ross-thick with amplitude 0.99; Li-sparse with
0.99 and parameters (1, 2); Li-dense with 0.99 and (2.5, 2); Cox-Munk with
amplitude 1, slope variance sigma^2 = 0.003 + 0.00512 x 15 m/s and the
squared real refractive index of sea water at 0.5 um and 34.3 ppt
(VBRDF_Water_RefracIndex, vsup/vbrdf/vbrdf_sup_kernels.f90:3814-3921,
single-precision table lookup 1.335 + 0.006), shadowing on; GISS Cox-Munk
with sigma^2 / 2 and the refractive index itself.  The result file holds, for
each kernel, the exact direct-bounce BRDF at the three azimuths and the
Fourier components m = 0, 1 (stream-stream, solar-stream, stream-user,
solar-user), 8 digits.  This keeps the blocks of those seven kernels (the
ones the MODIS RTLS and Cox-Munk surfaces use, and their neighbours).  The
JSON is small and is committed; the GPU machine never reads the reference tree.
"""
import json
import os
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: python %s <path of an AeroApps checkout>" % os.path.basename(__file__))
BASE = os.path.join(sys.argv[1], "src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_s_test")

SIGMA_SQ = 0.003 + 0.00512 * 15.0
REFRAC_R = float(np.float32(np.float32(1.335) + np.float32(0.006) * (np.float32(34.3) / np.float32(34.3))))
# (index, name, amplitude, parameters, shadowing) of GET_VBRDF_PLUS
KERNELS = [(1, "Lambertian", 0.1, [], False), (2, "Ross-thin", 0.99, [], False), (3, "Ross-thick", 0.99, [], False),
           (4, "Li-sparse", 0.99, [1.0, 2.0], False), (5, "Li-dense", 0.99, [2.5, 2.0], False),
           (9, "Cox-Munk", 1.0, [SIGMA_SQ, REFRAC_R ** 2, 0.0], True),
           (10, "GissCoxMnk", 1.0, [0.5 * SIGMA_SQ, REFRAC_R, 0.0], True)]


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
           "nstreams_brdf": int(lines[after("BRDFSUP - Number of BRDF azimuth angles")].split()[0])}
    nb = int(lines[after("BRDFSUP - Number of solar zenith angles")].split()[0])
    na = int(lines[after("BRDFSUP - Number of user-defined relative azimuth angles")].split()[0])
    nu = int(lines[after("BRDFSUP - Number of user-defined viewing zenith angles")].split()[0])
    out["szas"] = values("BRDFSUP - Solar zenith angles (degrees)", nb)
    out["raas"] = values("BRDFSUP - User-defined relative azimuth angles (degrees)", na)
    out["vzas"] = values("BRDFSUP - User-defined viewing zenith angles (degrees)", nu)
    return out


def read_results():
    """{kernel index: (exact values, {m: {pair: value}})}"""
    lines = open(os.path.join(BASE, "saved_results/gfortran/results_brdf_self_tester.res")).read().splitlines()
    out, idx, m = {}, None, None
    for ln in lines:
        t = ln.split()
        if "VBRDF Index:" in ln:
            idx, m = int(t[-1]), None
            out[idx] = ([], {})
            continue
        if idx is None:
            continue
        if ln.strip().startswith("Fourier component #"):
            m = int(t[-1])
            out[idx][1][m] = {}
            continue
        if m is None and len(t) == 4 and all(x.isdigit() for x in t[:3]):
            out[idx][0].append(float(t[3]))
        for key in ("Stream-Stream", "Solars-Stream", "Stream-Users", "Solars-Users"):
            if m is not None and ln.strip().startswith(key):
                out[idx][1][m][key] = float(t[3])
    return out


def main():
    out = read_cfg()
    res = read_results()
    out["kernels"] = []
    for which, name, factor, pars, shadow in KERNELS:
        exact, four = res[which]
        out["kernels"].append({"which": which, "name": name, "factor": factor, "pars": pars, "shadow": shadow,
                               "exact": exact, "fourier": {str(k): v for k, v in sorted(four.items())}})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "brdf_selftest_scalar.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


main()

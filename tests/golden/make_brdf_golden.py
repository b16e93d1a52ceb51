"""Build tests/golden/brdf_supcheck.json from the reference's own saved BRDF
test results.

Run with the path of an AeroApps checkout as the only argument
(`python make_brdf_golden.py <aeroapps-tree>`).  It reads, under
src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test/,

  VBRDF_ReadInput.cfg                   the kernel set of the BRDF testers
  saved_results/gfortran/results_brdf_supcheck_lattice.res
  saved_results/gfortran/results_brdfplus_tester_lattice_I000.all

The supplement check (V2p8p3_brdfplus_tester.f90:331-560) writes the exact
direct-bounce BRDF of the lattice (4 SZA x 3 VZA x 3 RAA) and the Fourier
components BRDF_F, BRDF_F_0, USER_BRDF_F, USER_BRDF_F_0 for m = 0..15 of the
kernel sum Ross-thin 0.3 + Li-dense 0.1 (2, 1) + Cox-Munk 0.1 (0.0798,
1.779556, shadowing), 8 streams, 100 BRDF azimuth streams.  The BRDF-plus
tester then runs VLIDORT on the atmosphere of the solar tester (the one
tests/golden/solar_tester_iqu.json holds: 23 layers, Rayleigh + a Mie
aerosol in the lowest 6) over that surface with FO correction (regular
pseudo-spherical), delta-M, 8 streams, and saves the TOA-upwelling Stokes I
of the 36 geometries (column "Stokes-I" of "Upwelling @ 0.00").  The JSON is
small and is committed; the GPU machine never reads the reference tree.
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python %s <path of an AeroApps checkout>" % os.path.basename(__file__))
BASE = os.path.join(sys.argv[1], "src/Components/rtms/RTSI/VLIDORT2p8p3/vlidort_v_test")
SAVED = os.path.join(BASE, "saved_results/gfortran")


def read_cfg():
    lines = open(os.path.join(BASE, "VBRDF_ReadInput.cfg")).read().splitlines()
    out = {}

    def after(title):
        for i, ln in enumerate(lines):
            if ln.strip().startswith(title):
                return i + 1
        raise KeyError(title)
    out["nstreams"] = int(lines[after("BRDFSUP - Number of half-space streams")].split()[0])
    out["nstreams_brdf"] = int(lines[after("BRDFSUP - Number of BRDF azimuth angles")].split()[0])
    out["shadow"] = lines[after("BRDFSUP - Do shadow effect for glitter kernels?")].strip().lower().startswith("t")
    nk = int(lines[after("BRDFSUP - Number of BRDF kernels")].split()[0])
    i = after("BRDFSUP - Kernel names, indices, amplitudes, # parameters, parameters")
    kernels = []
    for ln in lines[i:i + nk]:
        name, rest = ln[:10].strip(), ln[10:].split()
        kernels.append({"name": name, "which": int(rest[0]), "factor": float(rest[1]),
                        "pars": [float(x) for x in rest[3:6]]})
    out["kernels"] = kernels
    return out


def read_supcheck(nstreams):
    lines = open(os.path.join(SAVED, "results_brdf_supcheck_lattice.res")).read().splitlines()
    head = next(ln for ln in lines if ln.split() and ln.split()[0].isdigit())
    nb, nq, nu, na = [int(x) for x in head.split()[:4]]
    assert nq == nstreams
    exact = [[[0.0] * na for _ in range(nu)] for _ in range(nb)]
    i = 0
    while "Exact BRDF" not in lines[i]:
        i += 1
    i += 1
    while "Fourier component" not in lines[i]:
        p = lines[i].split()
        if len(p) == 4:
            exact[int(p[0]) - 1][int(p[1]) - 1][int(p[2]) - 1] = float(p[3])
        i += 1
    f, f0, uf, uf0 = [], [], [], []
    while i < len(lines):
        if "Fourier component" not in lines[i]:
            i += 1
            continue
        rows = []
        i += 1
        while i < len(lines) and "Fourier component" not in lines[i]:
            p = lines[i].split()
            if p:
                rows.append([float(x) for x in p[1:]])
            i += 1
        assert len(rows) == 2 * nq + 2 * nu, len(rows)
        f.append([rows[2 * j] for j in range(nq)])
        f0.append([rows[2 * j + 1] for j in range(nq)])
        uf.append([rows[2 * nq + 2 * u] for u in range(nu)])
        uf0.append([rows[2 * nq + 2 * u + 1] for u in range(nu)])
    return {"nbeams": nb, "nuser": nu, "nazim": na, "exact": exact, "f": f, "f0": f0, "uf": uf, "uf0": uf0}


def read_rt():
    out = {}
    for ln in open(os.path.join(SAVED, "results_brdfplus_tester_lattice_I000.all")).read().splitlines():
        if "FLUX" in ln:
            break  # the STOKES-I block comes first; the flux blocks follow
        p = ln.split()
        if len(p) >= 5 and p[1] == "Upwelling" and p[3] == "0.00":
            out[int(p[0])] = float(p[4])
    return [out[k] for k in sorted(out)]


def main():
    cfg = read_cfg()
    sup = read_supcheck(cfg["nstreams"])
    rt = read_rt()
    out = {
        "source": "vlidort_v_test/saved_results/gfortran/results_brdf_supcheck_lattice.res and "
                  "results_brdfplus_tester_lattice_I000.all (reference VLIDORT 2.8.3, VBRDF_ReadInput.cfg)",
        "kernels": cfg["kernels"], "nstreams": cfg["nstreams"], "nstreams_brdf": cfg["nstreams_brdf"],
        "shadow": cfg["shadow"], "szas": [35.0, 67.0, 75.0, 82.0], "vzas": [10.0, 20.0, 40.0],
        "raas": [10.0, 90.0, 170.0],
        "rt_options": {"do_focorr": 1, "do_focorr_nadir": 1, "do_focorr_outgoing": 0, "do_deltam": 1,
                       "nfinelayers": 4},
        "toa_up_I": rt,
    }
    out.update(sup)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "brdf_supcheck.json")
    with open(dst, "w") as f:
        json.dump(out, f)
    print(dst, "kernels", [k["name"] for k in cfg["kernels"]], "moments", len(sup["f"]), "rt", len(rt))


if __name__ == "__main__":
    main()

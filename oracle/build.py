"""Build recipe of the CPU oracle (test infrastructure only).

Compiles the oracle's own C/C++ restatement (vlidort_oracle.cpp,
vlidort_vector_oracle.cpp, brdf_oracle.cpp, mie_oracle.c,
rot_oracle.c, edge_oracle.c)
into oracle/_build/liboracle.so with strict IEEE semantics (no contraction of
a*b+c into FMA, so the FP32 Mie path reproduces the reference arithmetic).
The reference itself (Fortran 90) cannot be compiled on these machines: no
Fortran compiler is installed, and its Mie module also needs MAPL/ESMF/netCDF.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
SRCS = ["vlidort_oracle.cpp", "vlidort_vector_oracle.cpp", "brdf_oracle.cpp", "mie_oracle.c", "rot_oracle.c",
        "edge_oracle.c"]


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SRCS]
    deps = srcs + [__file__, os.path.join(HERE, "vlidort_oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in deps):
        return LIB
    objs = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        if s.endswith(".c"):
            cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-c", s, "-o", o]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-c", s, "-o", o]
        subprocess.run(cmd, check=True)
        objs.append(o)
    tmp = LIB + ".tmp"
    subprocess.run(["g++", "-shared", "-fopenmp", "-o", tmp] + objs, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

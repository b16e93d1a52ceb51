"""Build the in-tree CUDA library (libaerort.so) for sm_103a.

Each translation unit is compiled by its own nvcc process (the per-stream-count
RT instantiations are the slow ones), then linked into one shared library.
Nothing is installed: the library lands in aeroapps_gb300/_build/ and is found
there by aeroapps_gb300._lib.
"""
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libaerort.so")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_TUS = ["aerort.cu", "rt_ns4.cu", "rt_ns6.cu", "rt_ns8.cu", "rt_ns12.cu", "rt_ns16.cu", "rt_static.cu", "rt_rot.cu", "edge_vars.cu",
            "rt_vector.cu", "rt_brdf.cu"]
HOST_TUS = ["miegen.cpp", "mie_read.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build aerort")


def _sources_digest():
    h = hashlib.sha256()
    files = sorted(os.listdir(CSRC)) + ["../../include/aerort.h", "../build.py"]
    for f in files:
        p = os.path.normpath(os.path.join(CSRC, f))
        if os.path.isfile(p):
            h.update(f.encode())
            with open(p, "rb") as fh:
                h.update(fh.read())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile libaerort.so if sources changed; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "libaerort.digest")
    digest = _sources_digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == digest:
        return LIB
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(ROOT, "include")]
    jobs = []
    for tu in CUDA_TUS:
        obj = os.path.join(BUILD, tu + ".o")
        jobs.append([nvcc] + GENCODE + common + ["-c", os.path.join(CSRC, tu), "-o", obj])
    for tu in HOST_TUS:
        obj = os.path.join(BUILD, tu + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-I",
                     os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, tu), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, tu + ".o") for tu in CUDA_TUS + HOST_TUS]
    tmp = LIB + ".tmp"
    run([nvcc] + GENCODE + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

"""Benchmark: TOA radiances/s of the aerosol-optics + VLIDORT path on GB300.

Metric: TOA radiances per second of the mixed-precision GPU solve, whose
error against the FP64 oracle is measured per wavelength and must stay
<= 1e-4, reported beside the plain FP64 GPU solve of the same batch, with
serving p50/p95/p99 latency.

Workload (one step): the 262,144-column batching configuration -- 4
wavelengths (470, 550, 670, 865 nm), per-column layer count uniform in
20..72 (GEOS-5 72-level grid, upper layers merged), half-space streams drawn
from {4,6,8,12,16}, 2 x streams Legendre moments.  A step runs, for every
stream-count group, the Mie-table AOP kernel (FP32) and the RT solve on
device-resident inputs, concurrently on one CUDA stream per group, and is
replayed from a CUDA graph captured after the warm-up.  The optics and
scratch of a step are tens of GB, far more than the 129 MB L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Beside the headline line's standard keys it reports: the per-wavelength
error of the mixed and plain GPU solves against the FP64 oracle (first 4,096
columns of the batch, plus a near-conservative stress set with aerosol SSA in
[0.999, 1)), the plain FP64 throughput and mixed/plain ratio, the 1,024-column
plain-method configuration (columns/s, FP64 roofline, oracle on the host
cores), end-to-end throughput through the host-pointer C ABI, the serving
loop at 2,000 requests/s, and the HBM rooflines of the front-end kernels.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

STREAMS = (4, 6, 8, 12, 16)
CHANNELS = (470.0, 550.0, 670.0, 865.0)
SERVE_CHANNELS = (340.0, 380.0, 470.0, 550.0, 670.0, 865.0, 1640.0, 2130.0)
MISSING = -1.0e15
METRIC = ("TOA radiances/sec at <=1e-4 rel err vs FP64 (mixed-precision GPU solve; plain FP64 GPU solve and "
          "serving p50/p99 latency reported beside it)")
WORKLOAD = ("batching config: 262,144 columns x 4 wavelengths (470, 550, 670, 865 nm), 20-72 layers (GEOS-5 "
            "72-level grid, top layers merged), streams {4,6,8,12,16}, moments 2x streams; Mie AOP (FP32) + scalar "
            "Lambertian RT per stream group")
SEED = 20261204
# DRAM bytes (read + write) per solve-layer of the 16-stream FP32 series
# kernel: 17,592,320 B in one ncu capture of a launch of 2,300 solves with
# 104,216 solve-layers (the 8,192-column batch's 37-54-layer group;
# profiles/k_team_series_16_float_cols8192.md).  Its inputs are per layer,
# so the traffic of a launch scales with its solve-layers.
TEAM16_DRAM_BYTES_PER_SOLVE_LAYER = 17592320 / 104216


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cols", type=int, default=262144, help="columns per step per GPU (x4 wavelengths = solves)")
    ap.add_argument("--plain-steps", type=int, default=1, help="timed steps of the plain FP64 solve")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-cols", type=int, default=0, help="oracle sample columns (0 = 4096, or 512 per step "
                    "of --impl reference)")
    ap.add_argument("--stress-cols", type=int, default=96, help="columns per stream count of the SSA stress set")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-config0", action="store_true")
    ap.add_argument("--config3-cols", type=int, default=2048, help="columns of the polarized sample (0 = skip)")
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="Poisson arrival rate [requests/s]")
    ap.add_argument("--serve-max-cols", type=int, default=16384, help="largest swath of the serving run")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--tune", action="store_true", help="re-run the schedule autotuner before timing")
    ap.add_argument("--contraction", default="fma", choices=["fma", "tf32x3"],
                    help="moment contraction of the FP32 team solve for the whole run (aerort_set_moment_contraction)")
    ap.add_argument("--eager", action="store_true", help="launch the timed steps eagerly instead of replaying "
                    "the captured CUDA graph")
    ap.add_argument("--buckets", default="36,54,72", help="upper layer counts of the launch groups' layer buckets "
                    "(one launch per stream count and bucket; '72' = one launch per stream count)")
    ap.add_argument("--serial", action="store_true", help="run the stream-count groups one after another on one "
                    "CUDA stream instead of concurrently on one stream each")
    return ap.parse_args(argv)


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def bench_config(args):
    """The `config` object of both arms (the reference arm times a bounded
    sample of this same workload)."""
    return {"workload": WORKLOAD, "columns_per_step": args.cols, "solves_per_step": args.cols * len(CHANNELS),
            "wavelengths": list(CHANNELS), "streams": list(STREAMS), "layers": [20, 72],
            "l2": "inputs larger than L2 (optics + scratch of a step: tens of GB); no flush needed"}


def make_batch(ncol, seed):
    """Config-1 columns: per-column layers U{20..72}, streams from STREAMS."""
    from aeroapps_gb300 import synth
    rng = np.random.default_rng(seed)
    nl = rng.integers(20, 73, ncol)
    ns = rng.choice(np.array(STREAMS), ncol)
    cols = synth.make_columns(ncol, list(CHANNELS), seed=seed + 1, nlayers=nl)
    cols["nstreams"] = ns
    return cols


def subset(cols, idx):
    """Columns idx of a make_columns dict (km trimmed to the deepest column)."""
    out = dict(cols)
    out["ncol"] = len(idx)
    for k in ("pe", "he", "te", "rh"):
        out[k] = np.asfortranarray(cols[k][..., idx])
    out["albedo"] = np.asfortranarray(cols["albedo"][idx, :])
    out["qm"] = np.asfortranarray(cols["qm"][:, :, idx])
    out["ROT"] = np.asfortranarray(cols["ROT"][:, idx, :])
    for k in ("sza", "vza", "raa", "nlayers", "nstreams"):
        if k in cols:
            out[k] = np.ascontiguousarray(cols[k][idx])
    km = int(out["nlayers"].max())
    out["km"] = km
    for k in ("pe", "he", "te"):
        out[k] = np.asfortranarray(out[k][: km + 1])
    for k in ("rh", "qm", "ROT"):
        out[k] = np.asfortranarray(out[k][:km])
    return out


def alg_flops(N, L, nfourier, K=None):
    """Reference-algorithm flops of one (column, wavelength) solve (banded-LU
    formulation of the reference), summed over the Fourier terms the solve
    executed: for m = 0..M, with n = 2NL, kl = ku = 3N - 1, K_m = NMOMENTS - m + 1:
      L(4N^2 K_m + 2N K_m + 2N^3) + 10 L N^3 + L(6N^2 + 20N)
      + 2n kl (kl+ku) + 2n (2kl+ku) + 10 L N,  plus FO: L(2K + 60)."""
    NM = 2 * N - 1
    K = 2 * N if K is None else K
    n = 2.0 * N * L
    kl = ku = 3.0 * N - 1.0
    tot = L * (2.0 * K + 60.0)
    for m in range(int(nfourier) + 1):
        Km = NM - m + 1
        tot += L * (4.0 * N * N * Km + 2.0 * N * Km + 2.0 * N ** 3) + 10.0 * L * N ** 3 + L * (6.0 * N * N + 20.0 * N)
        tot += 2.0 * n * kl * (kl + ku) + 2.0 * n * (2.0 * kl + ku) + 10.0 * L * N
    return tot


def flops_table(nmax=64):
    """alg_flops for every stream count, layer count 1..72 and last Fourier
    term 0..nmax-1: {N: array (73, nmax)}."""
    return {N: np.array([[alg_flops(N, L, m) if L > 0 else 0.0 for m in range(nmax)] for L in range(73)])
            for N in STREAMS}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def pipe_peaks(torch, lib, stream):
    """Measured FP64 and FP32 FMA pipe rates (probe kernels, TFLOP/s) and cuBLAS DGEMM."""
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    blocks, threads = 152 * 16, 256

    def rate(fn, iters):
        fn(blocks, threads, 64, out.data_ptr(), stream)
        best = 0.0
        for _ in range(3):
            s.record()
            fn(blocks, threads, iters, out.data_ptr(), stream)
            e.record()
            torch.cuda.synchronize()
            best = max(best, blocks * threads * iters * 16.0 / (s.elapsed_time(e) * 1e-3))
        return best / 1e12
    fp64 = rate(lib.aerort_probe_dfma, 4096)
    fp32 = rate(lib.aerort_probe_ffma, 65536)
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    dg = 0.0
    for _ in range(3):
        s.record()
        torch.matmul(a, b)
        e.record()
        torch.cuda.synchronize()
        dg = max(dg, 2.0 * 4096 ** 3 / (s.elapsed_time(e) * 1e-3))
    return fp64, fp32, dg / 1e12


def oracle_radiances(batch, ncols, channels, threads=0, ssa_override=None):
    """The oracle (C++ restatement of Chem_MieQuery + VLIDORT 2.8.3, FP64 RT,
    OpenMP over pixels on `threads` host cores, 0 = all) on the first `ncols`
    columns of a batch; returns (radiance (ncols, nch), nfourier, seconds).
    ssa_override(N, ssa) may replace the FP32 AOP single-scattering albedo
    before the RT solve (stress sets)."""
    from oracle import oracle
    from aeroapps_gb300 import mie, synth
    sub = subset(batch, np.arange(ncols))
    nch = len(channels)
    oracle.set_threads(threads)
    tabs = mie.generate_tables(list(channels), nmom=32)
    qidx = {}
    for ti, t in enumerate(tabs.tables):
        for b in range(t.bext.shape[2]):
            qidx["%s%03d" % (t.name, b + 1)] = (ti, b)
    qt, qb = zip(*[qidx[n] for n in synth.tracer_names()])
    rad = np.full((ncols, nch), np.nan)
    nfo = np.zeros((ncols, nch), np.int32)
    dt = 0.0
    for N in STREAMS:
        idx = np.nonzero(sub["nstreams"] == N)[0]
        if len(idx) == 0:
            continue
        g = subset(sub, idx)
        km, n = g["km"], g["ncol"]
        t0 = time.perf_counter()
        tau, ssa, gg, pm, rc = oracle.get_aop_vector(tabs, km, n, nch, 20, np.float32(channels), qt, qb, g["qm"],
                                                     g["rh"], 2 * N, 1)
        if ssa_override is not None:
            ssa = ssa_override(N, ssa)
        r, _, rc2, nf, st = oracle.scalar_lambert(km, nch, n, np.array(channels), N, 0, 2 * N, 1, g["ROT"],
                                                  g["depol"], tau, ssa, gg, pm, g["pe"], g["he"], g["te"],
                                                  g["albedo"], g["sza"], g["raa"], g["vza"], MISSING,
                                                  nlay=g["nlayers"])
        dt += time.perf_counter() - t0
        rad[idx] = r
        nfo[idx] = nf
    oracle.set_threads(0)
    return rad, nfo, dt


def run_reference(args):
    """The reference arm: the oracle port timed on the host cores (the
    reference Fortran cannot be built here or on the GPU host), each step a
    bounded sample of the same workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    ncols = max(args.cpu_cols or 512, 8)
    batch = make_batch(ncols, seed=SEED)  # about 2-5 s per step on 8-16 cores
    times = []
    for i in range(args.warmup + args.steps):
        _, _, dt = oracle_radiances(batch, ncols, CHANNELS)
        if i >= args.warmup:
            times.append(dt)
    v = ncols * len(CHANNELS) * len(times) / sum(times)
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": v, "unit": "radiances/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": bench_config(args),
            "cpu_baseline": {"value": v, "unit": "radiances/s", "cores": cores, "kind": "port",
                             "sample": "each step: the first %d columns x 4 wavelengths of the same workload "
                                       "(seed %d); the reference Fortran cannot be built here or on the GPU host "
                                       "(no Fortran compiler), so its C++ restatement runs (Mie AOP FP32 + VLIDORT "
                                       "FP64, OpenMP over pixels, %d threads)" % (ncols, SEED, cores)},
            "e2e": {"value": v, "unit": "radiances/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _hbm_peak():
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        return peak, "MEASURED_PEAKS.json hbm_gbs (STREAM-style copy), of measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s, of fallback"


def _time_flushed(torch, call, reps=20):
    """Mean CUDA-event time [ms] of call() on the current stream, L2 flushed
    (512 MB write) before each launch so that every launch reads from HBM."""
    from aeroapps_gb300 import _lib
    for _ in range(3):
        assert call() == 0, _lib.last_error()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    ms = 0.0
    for _ in range(reps):
        flush.zero_()
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record()
        call()
        r1.record()
        torch.cuda.synchronize()
        ms += r0.elapsed_time(r1) / reps
    return ms


def front_end_rooflines(torch, L, batch, stream, ncr=262144, chem=None, qt=None, qb=None):
    """Rooflines of the front-end kernels on the 262,144 columns of the
    batching configuration (this batch's profiles tiled), against the measured
    copy bandwidth:
    - k_rot_calc (VLIDORT_ROT_CALC, FP64): algorithmic bytes = pe, he, te read
      once per pixel + ROT written per pixel and channel (+ depol);
    - k_edge_vars (getEdgeVars, FP32): airdens, delp read + pe, ze, te written;
    - k_aop (VLIDORT_getAOPvector, FP32; when a Mie object is given): qm, rh
      read + tau, ssa, g, pmom written, 72 layers, 4 channels, 16 moments."""
    from aeroapps_gb300 import synth
    P = lambda t: t.data_ptr()
    kmb = batch["km"]
    my_cols = min(batch["ncol"], 16384)
    nch = len(CHANNELS)
    peak, src = _hbm_peak()
    # Fortran (k, columns) = C (columns, k), tiled to ncr columns
    tile = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a[..., :my_cols], dt).T)).cuda().repeat(
        (ncr + my_cols - 1) // my_cols, 1)[:ncr].contiguous()
    dpe, dhe, dte = (tile(batch[k], np.float64) for k in ("pe", "he", "te"))
    dch = torch.from_numpy(np.array(CHANNELS, np.float64)).cuda()
    drot = torch.empty(kmb * ncr * nch, dtype=torch.float64, device="cuda")
    ddep = torch.empty(nch, dtype=torch.float64, device="cuda")
    ms_rot = _time_flushed(torch, lambda: L.aerort_vlidort_rot_calc_dev(kmb, nch, ncr, P(dch), P(dpe), P(dhe), P(dte),
                                                                      P(drot), P(ddep), stream))
    del dpe, dhe, dte, drot
    alg = 3 * (kmb + 1) * 8 * ncr + kmb * ncr * nch * 8 + nch * 8
    ach = alg / (ms_rot * 1e-3) / 1e9
    rot_line = {"kernel": "k_rot_calc (VLIDORT_ROT_CALC)", "bound": "hbm", "ms_per_launch": ms_rot,
                "algorithmic_bytes": alg, "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "peak_source": src, "columns": ncr, "wavelengths": nch, "layers": kmb,
                "note": "L2 flushed (512 MB write) before each timed launch"}
    # layer air density and pressure thickness of full-height columns with km
    # layers (the batch's shorter columns are padded with empty layers)
    ue = synth.make_columns(min(my_cols, 4096), [550.0], seed=3, nlayers=kmb)
    pe, te = ue["pe"], ue["te"]
    pm = 0.5 * (pe[1:] + pe[:-1])
    rho = pm / (synth.RGAS * 0.5 * (te[1:] + te[:-1]))
    my_cols = ue["ncol"]
    drho, ddp = tile(rho, np.float32), tile(np.diff(pe, axis=0), np.float32)
    out = torch.empty(3 * (kmb + 1) * ncr, dtype=torch.float32, device="cuda")
    ne = (kmb + 1) * ncr
    ptop = float(pe[0, 0])
    ms_edge = _time_flushed(torch, lambda: L.aerort_get_edge_vars_dev(kmb, ncr, P(drho), P(ddp), ptop, P(out),
                                                                    P(out) + 4 * ne, P(out) + 8 * ne, stream))
    del drho, ddp, out
    alg = 2 * kmb * 4 * ncr + 3 * (kmb + 1) * 4 * ncr
    ach = alg / (ms_edge * 1e-3) / 1e9
    edge_line = {"kernel": "k_edge_vars (getEdgeVars)", "bound": "hbm", "ms_per_launch": ms_edge,
                 "algorithmic_bytes": alg, "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                 "peak_source": src, "columns": ncr, "layers": kmb,
                 "note": "L2 flushed (512 MB write) before each timed launch"}
    aop_line = None
    if chem is not None:
        from aeroapps_gb300 import _lib
        km, nq, nmom = 72, len(qt), 16
        ua = synth.make_columns(4096, list(CHANNELS), seed=5, nlayers=km)
        reps = (ncr + ua["ncol"] - 1) // ua["ncol"]
        # Fortran (km, nq, columns) = C (columns, nq, km)
        dqm = torch.from_numpy(np.ascontiguousarray(np.asarray(ua["qm"], np.float32).T)).cuda().repeat(
            reps, 1, 1)[:ncr].contiguous()
        drh = torch.from_numpy(np.ascontiguousarray(np.asarray(ua["rh"], np.float32).T)).cuda().repeat(
            reps, 1)[:ncr].contiguous()
        no = km * nch * ncr
        out = torch.empty(no * (3 + nmom), dtype=torch.float32, device="cuda")
        ch32 = np.array(CHANNELS, np.float32)
        qt32, qb32 = np.asarray(qt, np.int32), np.asarray(qb, np.int32)
        ms_aop = _time_flushed(torch, lambda: L.aerort_get_aop_vector_dev(
            chem.handle, km, ncr, nch, nq, _lib.ptr(ch32, _lib.P_f), _lib.ptr(qt32, _lib.P_i),
            _lib.ptr(qb32, _lib.P_i), P(dqm), P(drh), nmom, 1, P(out), P(out) + 4 * no, P(out) + 8 * no,
            P(out) + 12 * no, stream))
        del dqm, drh, out
        alg = (km * nq + km) * 4 * ncr + no * (3 + nmom) * 4
        ach = alg / (ms_aop * 1e-3) / 1e9
        aop_line = {"kernel": "k_aop (VLIDORT_getAOPvector + Chem_MieQuery)", "bound": "hbm",
                    "ms_per_launch": ms_aop, "algorithmic_bytes": alg, "achieved": ach, "peak": peak, "unit": "GB/s",
                    "frac": ach / peak, "peak_source": src, "columns": ncr, "layers": km, "tracers": nq,
                    "wavelengths": nch, "moments": nmom,
                    "note": "L2 flushed (512 MB write) before each timed launch; Mie-table reads (L2-resident) "
                            "not counted"}
    return rot_line, edge_line, aop_line


def rel_err_stats(got, ref, ok):
    e = np.abs(got[ok] / ref[ok] - 1.0)
    return (float(e.max()) if e.size else None), (float(np.median(e)) if e.size else None), int(e.size)


def config0(torch, L, fp64_peak, ftab, cpu=True):
    """The plain-method configuration: FP64, 1,024 columns x 72 layers, one
    wavelength (550 nm), 8 streams, 16 moments.  GPU columns/s (CUDA events,
    3 warm-up + 5 timed launches of AOP + RT), its FP64 roofline on the
    reference-algorithm flop model, parity against the oracle, and the oracle
    on the host cores (all cores, and one core on the first 128 columns)."""
    from aeroapps_gb300 import _lib, mie, synth
    from oracle import oracle
    ncol, km, N, ch = 1024, 72, 8, [550.0]
    cols = synth.make_columns(ncol, ch, seed=20261203, nlayers=km)
    tabs = mie.generate_tables(ch, nmom=2 * N)
    chem = mie.ChemMie(tabs)
    names = synth.tracer_names()
    qt = np.array([chem.query_idx(n)[0] for n in names], np.int32)
    qb = np.array([chem.query_idx(n)[1] for n in names], np.int32)
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    d = {k: dev(cols[k], np.float64) for k in ("ROT", "depol", "he", "albedo", "sza", "raa", "vza")}
    qm, rh = dev(cols["qm"], np.float32), dev(cols["rh"], np.float32)
    tau = torch.empty(km * ncol, dtype=torch.float32, device="cuda")
    ssa, g = torch.empty_like(tau), torch.empty_like(tau)
    pm = torch.empty(km * ncol * 2 * N, dtype=torch.float32, device="cuda")
    rad = torch.empty(ncol, dtype=torch.float64, device="cuda")
    refl, nf, st = torch.empty_like(rad), torch.empty(ncol, dtype=torch.int32, device="cuda"), \
        torch.empty(ncol, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ch32 = np.array(ch, np.float32)
    P = lambda t: t.data_ptr()
    # the library's own kernel choice for this batch size (1,024 solves: the
    # team kernel, one warp per solve); the shipped table's 8-stream FP64
    # entry was tuned on 8,192-column buckets
    L.aerort_set_kernel(N, _lib.PREC_FP64, _lib.KERNEL_AUTO)
    L.aerort_set_schedule(N, _lib.PREC_FP64, 32, 0)

    def run():
        rc = L.aerort_get_aop_vector_dev(chem.handle, km, ncol, 1, 20, _lib.ptr(ch32, _lib.P_f), _lib.ptr(qt, _lib.P_i),
                                         _lib.ptr(qb, _lib.P_i), P(qm), P(rh), 2 * N, 1, P(tau), P(ssa), P(g), P(pm),
                                         stream)
        assert rc == 0, _lib.last_error()
        rc = L.aerort_vlidort_scalar_lambert_batch_dev(km, 1, ncol, N, 0, 2 * N, None, P(d["ROT"]), P(d["depol"]),
                                                       None, None, None, P(tau), P(ssa), P(pm), P(d["he"]),
                                                       P(d["albedo"]), P(d["sza"]), P(d["raa"]), P(d["vza"]), MISSING,
                                                       P(rad), P(refl), P(nf), P(st), stream)
        assert rc == 0, _lib.last_error()
    for _ in range(3):
        run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    e0.record()
    for _ in range(reps):
        run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    grad = rad.cpu().numpy()
    gnf = nf.cpu().numpy()
    # the same launches with the term-parallel team solve (each column's
    # Fourier terms over the warps of a block), AERORT_KERNEL_TERMS
    L.aerort_set_kernel(N, _lib.PREC_FP64, _lib.KERNEL_TERMS)
    for _ in range(2):
        run()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(reps):
        run()
    t1.record()
    torch.cuda.synchronize()
    ms_terms = t0.elapsed_time(t1) / reps
    trad = rad.cpu().numpy()
    L.aerort_set_kernel(N, _lib.PREC_FP64, _lib.KERNEL_AUTO)
    okt = grad != MISSING
    kernel_ab = {"auto_ms": ms, "terms_ms": ms_terms, "terms_speedup": ms / ms_terms,
                 "terms_vs_auto_max_rel": float(np.max(np.abs(trad[okt] / grad[okt] - 1.0))),
                 "fourier_terms_identical": bool(np.array_equal(nf.cpu().numpy(), gnf))}
    flops = float(ftab[N][km, gnf].sum())
    ach = flops / (ms * 1e-3) / 1e12
    out = {"workload": "plain FP64 method: 1,024 columns x 72 layers, 550 nm, 8 streams, 16 moments, Lambertian; "
                       "AOP kernel + FP64 RT per launch",
           "value": ncol / (ms * 1e-3), "unit": "columns/s", "ms_per_launch": ms, "kernel_ab": kernel_ab,
           "roofline": {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                        "frac": ach / fp64_peak,
                        "note": "reference-algorithm flops (banded-LU BVP, nonsymmetric eigen-solve) summed over the "
                                "Fourier terms each column ran; peak = live DFMA probe, of measured"}}
    chem.destroy()
    if cpu:
        cols["nstreams"] = np.full(ncol, N)
        orad, _, dt = oracle_radiances(cols, ncol, ch)
        ok = np.isfinite(orad[:, 0]) & (orad[:, 0] != MISSING)
        mx, md, n = rel_err_stats(grad, orad[:, 0], ok)
        _, _, dt1 = oracle_radiances(cols, 128, ch, threads=1)
        out["parity_vs_oracle"] = {"max_rel_err": mx, "median_rel_err": md, "columns": n, "bar": 1e-9}
        out["cpu_baseline"] = {"value": ncol / dt, "unit": "columns/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": "the same 1,024 columns (oracle AOP + FP64 RT, OpenMP over pixels)",
                               "single_core": {"value": 128 / dt1, "unit": "columns/s", "cores": 1,
                                               "sample": "first 128 of the same columns"}}
    return out


def config3(torch, L, ncols, ocols=32, cpu=True):
    """The polarized configuration: NSTOKES = 3, 12 streams, 64 Greek
    coefficients of the six scattering-matrix elements (from the same
    Lorenz-Mie tables, mixed by the AOP kernel with nPol = 6), 72 layers, 8
    wavelengths (SERVE_CHANNELS), Lambertian albedo U(0.02, 0.40).  A bounded
    sample of the 65,536-column workload: `ncols` columns at every wavelength
    in one AOP + vector RT launch pair (FP32 optics straight into the FP64
    polarized solve), 1 warm-up + 1 timed launch with CUDA events.  I, Q, U
    of the first `ocols` columns against the polarized FP64 oracle (I
    relative; Q and U relative to I, as they pass through zero), and the
    oracle's own rate on the host cores."""
    from aeroapps_gb300 import _lib, mie, synth
    from oracle import oracle
    N, km, nmom, ch = 12, 72, 64, list(SERVE_CHANNELS)
    nch = len(ch)
    cols = synth.make_columns(ncols, ch, seed=SEED + 3, nlayers=km)
    cols["albedo"] = np.asfortranarray(np.random.default_rng(SEED + 33).uniform(0.02, 0.40, (ncols, nch)))
    tabs = mie.generate_tables(ch, nmom=nmom, npol=6)
    chem = mie.ChemMie(tabs)
    names = synth.tracer_names()
    qt = np.array([chem.query_idx(n)[0] for n in names], np.int32)
    qb = np.array([chem.query_idx(n)[1] for n in names], np.int32)
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    d = {k: dev(cols[k], np.float64) for k in ("ROT", "depol", "he", "albedo", "sza", "raa", "vza")}
    qm, rh = dev(cols["qm"], np.float32), dev(cols["rh"], np.float32)
    nl = km * nch * ncols
    tau = torch.empty(nl, dtype=torch.float32, device="cuda")
    ssa, g = torch.empty_like(tau), torch.empty_like(tau)
    pm = torch.empty(nl * nmom * 6, dtype=torch.float32, device="cuda")
    out = {k: torch.empty(ncols * nch, dtype=torch.float64, device="cuda") for k in ("rad", "refl", "q", "u")}
    nf = torch.empty(ncols * nch, dtype=torch.int32, device="cuda")
    st = torch.empty_like(nf)
    stream = torch.cuda.current_stream().cuda_stream
    ch32 = np.array(ch, np.float32)
    P = lambda t: t.data_ptr()

    def run():
        rc = L.aerort_get_aop_vector_dev(chem.handle, km, ncols, nch, 20, _lib.ptr(ch32, _lib.P_f),
                                         _lib.ptr(qt, _lib.P_i), _lib.ptr(qb, _lib.P_i), P(qm), P(rh), nmom, 6,
                                         P(tau), P(ssa), P(g), P(pm), stream)
        assert rc == 0, _lib.last_error()
        rc = L.aerort_vlidort_vector_lambert_batch_dev(km, nch, ncols, N, 0, nmom, None, P(d["ROT"]), P(d["depol"]),
                                                        None, None, None, None, P(tau), P(ssa), P(pm), P(d["he"]),
                                                        P(d["albedo"]), P(d["sza"]), P(d["raa"]), P(d["vza"]), None,
                                                        MISSING, P(out["rad"]), P(out["refl"]), P(out["q"]),
                                                        P(out["u"]), P(nf), P(st), stream)
        assert rc == 0, _lib.last_error()
    run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 1
    e0.record()
    for _ in range(reps):
        run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    res = {"workload": "polarized: NSTOKES=3, 12 streams, 64 Greek coefficients x 6 elements, 72 layers, 8 wavelengths "
                       "(340-2130 nm), Lambertian albedo U(0.02,0.40); AOP (nPol=6) + FP64 vector RT per launch",
           "columns": ncols, "solves": ncols * nch, "value": ncols * nch / (ms * 1e-3), "unit": "radiances/s",
           "ms_per_launch": ms, "sample": "%d of the workload's 65,536 columns, all 8 wavelengths" % ncols,
           "failed_solves": int((st.cpu().numpy() != 0).sum())}
    g_out = {k: v.cpu().numpy().reshape(ncols, nch, order="F") for k, v in out.items()}
    gnf = nf.cpu().numpy().reshape(ncols, nch, order="F")
    chem.destroy()
    if cpu:
        sub = subset(cols, np.arange(ocols))
        t0 = time.perf_counter()
        otau, ossa, _, opm, rc = oracle.get_aop_vector(tabs, km, ocols, nch, 20, ch32, qt, qb, sub["qm"], sub["rh"],
                                                       nmom, 6)
        F = lambda a: np.asfortranarray(a.astype(np.float64))
        orad, _, oq, ou, rc2, onf, ost = oracle.vector_lambert(km, nch, ocols, N, 0, nmom, sub["ROT"], sub["depol"],
                                                               None, F(otau), F(ossa), F(opm), sub["he"],
                                                               sub["albedo"], sub["sza"], sub["raa"], sub["vza"],
                                                               None, MISSING)
        dt = time.perf_counter() - t0
        ok = (orad != MISSING) & (ost == 0)
        gi, gq, gu = g_out["rad"][:ocols], g_out["q"][:ocols], g_out["u"][:ocols]
        ei = np.abs(gi[ok] / orad[ok] - 1.0)
        eq = np.abs(gq[ok] - oq[ok]) / orad[ok]
        eu = np.abs(gu[ok] - ou[ok]) / orad[ok]
        res["parity_vs_oracle"] = {"I_max_rel": float(ei.max()), "I_median_rel": float(np.median(ei)),
                                   "Q_max_rel_to_I": float(eq.max()), "U_max_rel_to_I": float(eu.max()),
                                   "fourier_terms_identical": bool(np.array_equal(onf, gnf[:ocols])),
                                   "solves": int(ok.sum()), "bar": 1e-9}
        res["cpu_baseline"] = {"value": ocols * nch / dt, "unit": "radiances/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": "the first %d columns x 8 wavelengths: oracle AOP (nPol=6) "
                                                         "+ polarized FP64 oracle, OpenMP over pixels; %.1f s"
                                                         % (ocols, dt)}
    return res


def e2e_host_abi(L, chem, groups, qt, qb, ch32, steps):
    """End to end through the host-pointer C ABI, as a Fortran caller would
    drive it: per stream-count group, aerort_get_aop_vector on host
    Fortran-order qm, rh (copy in, AOP kernel, copy out of the FP32 optics),
    the caller's dble() of the optics on the host (geo_vlidort.F90:598-601),
    then aerort_vlidort_scalar_lambert_mixed_batch on host arrays (copy in,
    mixed RT, copy out of radiance, reflectance, Fourier count, status).
    Returns (radiances/s, h2d bytes per step, d2h bytes per step, step times)."""
    from aeroapps_gb300 import _lib
    Pf = lambda a: _lib.ptr(a, _lib.P_f)
    Pd = lambda a: _lib.ptr(a, _lib.P_d)
    Pi = lambda a: _lib.ptr(a, _lib.P_i)
    nch = len(CHANNELS)
    h2d = d2h = 0
    for d in groups:
        h, km, n, nm = d["host"], d["km"], d["n"], d["nmom"]
        if "e2e" not in d:
            F = lambda shape, dt: np.zeros(shape, dt, order="F")
            d["e2e"] = {"tau": F((km, nch, n), np.float32), "ssa": F((km, nch, n), np.float32),
                        "g": F((km, nch, n), np.float32), "pmom": F((km, nch, n, nm, 1), np.float32),
                        "tau64": F((km, nch, n), np.float64), "ssa64": F((km, nch, n), np.float64),
                        "pmom64": F((km, nch, n, nm), np.float64), "rad": F((n, nch), np.float64),
                        "refl": F((n, nch), np.float64), "nf": F((n, nch), np.int32), "st": F((n, nch), np.int32),
                        "nl": np.ascontiguousarray(h["nlayers"], np.int32),
                        "ROT": np.asfortranarray(h["ROT"], np.float64), "he": np.asfortranarray(h["he"], np.float64),
                        "albedo": np.asfortranarray(h["albedo"], np.float64),
                        "sza": np.ascontiguousarray(h["sza"], np.float64),
                        "raa": np.ascontiguousarray(h["raa"], np.float64),
                        "vza": np.ascontiguousarray(h["vza"], np.float64),
                        "depol": np.ascontiguousarray(h["depol"], np.float64)}
        e = d["e2e"]
        h2d += h["qm"].nbytes + h["rh"].nbytes
        d2h += e["tau"].nbytes * 3 + e["pmom"].nbytes
        h2d += sum(e[k].nbytes for k in ("ROT", "depol", "tau64", "ssa64", "pmom64", "he", "albedo", "sza", "raa",
                                         "vza", "nl"))
        d2h += sum(e[k].nbytes for k in ("rad", "refl", "nf", "st"))

    def one_step():
        for d in groups:
            h, km, n, N, nm, e = d["host"], d["km"], d["n"], d["N"], d["nmom"], d["e2e"]
            rc = L.aerort_get_aop_vector(chem.handle, km, n, nch, 20, Pf(ch32), Pi(qt), Pi(qb), Pf(h["qm"]),
                                         Pf(h["rh"]), nm, 1, Pf(e["tau"]), Pf(e["ssa"]), Pf(e["g"]), Pf(e["pmom"]))
            assert rc == 0, _lib.last_error()
            np.copyto(e["tau64"], e["tau"])
            np.copyto(e["ssa64"], e["ssa"])
            np.copyto(e["pmom64"], e["pmom"][..., 0])
            rc = L.aerort_vlidort_scalar_lambert_mixed_batch(
                km, nch, n, N, 0, nm, Pi(e["nl"]), Pd(e["ROT"]), Pd(e["depol"]), Pd(e["tau64"]), Pd(e["ssa64"]),
                Pd(e["pmom64"]), Pd(e["he"]), Pd(e["albedo"]), Pd(e["sza"]), Pd(e["raa"]), Pd(e["vza"]), MISSING,
                Pd(e["rad"]), Pd(e["refl"]), Pi(e["nf"]), Pi(e["st"]))
            assert rc == 0, _lib.last_error()
        return sum(float(d["e2e"]["rad"][0, 0]) for d in groups)  # the host reads the step's results
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        got = one_step()
        times.append(time.perf_counter() - t)
        assert np.isfinite(got)
    solves = sum(d["n"] for d in groups) * nch
    return solves / (sum(times) / len(times)), h2d, d2h, times


def serving_run(args, tabs):
    """Config 4: Poisson swaths of 64-16,384 columns (log-uniform), 1-8
    wavelengths, streams {4..16}, layers 20-72, 120 GB HBM budget; p50/p95/p99
    at the configured rate and at half the measured offline capacity, and the
    offline batch of the same mix."""
    from aeroapps_gb300 import serve
    rng = np.random.default_rng(4)
    nreq = args.serve_requests
    sizes = np.exp(rng.uniform(np.log(64), np.log(args.serve_max_cols), nreq)).astype(int)
    nchs = rng.integers(1, len(SERVE_CHANNELS) + 1, nreq)
    firsts = [rng.integers(0, len(SERVE_CHANNELS) - k + 1) for k in nchs]
    base = [serve.make_swath(i, int(sizes[i]), list(SERVE_CHANNELS[f:f + k]), seed=5000 + i)
            for i, (f, k) in enumerate(zip(firsts, nchs))]
    fresh = lambda: [serve.Swath(rid=s.rid, cols=s.cols, nstreams=s.nstreams, channels=s.channels) for s in base]
    srv = serve.Server(tabs, nslots=2, precision="mixed", hbm_budget_gb=120.0, max_batch_cols=65536)
    srv.submit(serve.make_swath(999, 256, list(SERVE_CHANNELS), seed=1))
    srv.drain()
    srv.done.clear()
    done, wall = serve.run_poisson(srv, fresh(), args.serve_rate, seed=9)
    stats = serve.latency_stats(done)
    rads = sum(s.radiances for s in done)
    sw2 = fresh()
    srv.done.clear()
    t = time.perf_counter()
    for s in sw2:
        srv.submit(s)
    srv.drain()
    offline = sum(s.radiances for s in sw2) / (time.perf_counter() - t)
    mean_rads = sum(s.radiances for s in sw2) / len(sw2)
    half_rate = 0.5 * offline / mean_rads
    srv.done.clear()
    done3, wall3 = serve.run_poisson(srv, fresh(), half_rate, seed=11)
    stats3 = serve.latency_stats(done3)
    stats3.update({"arrival_rate_per_s": half_rate,
                   "sustained_radiances_per_s": sum(s.radiances for s in done3) / wall3})
    srv.close()
    out = dict(stats)
    out.update({"arrival_rate_per_s": args.serve_rate, "sustained_radiances_per_s": rads / wall,
                "offline_batch_radiances_per_s": offline, "sustained_over_offline": rads / wall / offline,
                "batch_lanes": 2, "max_batch_cols": 65536, "precision": "mixed",
                "swath_columns": "log-uniform %d..%d" % (64, args.serve_max_cols),
                "wavelengths_per_request": "1-8 of %s nm" % list(SERVE_CHANNELS), "hbm_budget_gb": 120.0,
                "note": "at the configured rate the GPU is saturated, so latency is queueing; at_half_capacity "
                        "repeats the mix at half the measured offline throughput",
                "at_half_capacity": stats3})
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from aeroapps_gb300 import _lib, autotune, mie, synth
    L = _lib.lib()
    run_contraction = _lib.CONTRACT_TF32X3 if args.contraction == "tf32x3" else _lib.CONTRACT_FMA
    assert L.aerort_set_moment_contraction(run_contraction) == 0
    stream = torch.cuda.current_stream().cuda_stream
    dev_name = torch.cuda.get_device_name(local)
    tuned_src = autotune.apply_defaults(dev_name)
    tabs = mie.generate_tables(list(CHANNELS), nmom=32)
    chem = mie.ChemMie(tabs)
    names = synth.tracer_names()
    qt = np.array([chem.query_idx(n)[0] for n in names], np.int32)
    qb = np.array([chem.query_idx(n)[1] for n in names], np.int32)
    ch32 = np.array(CHANNELS, np.float32)
    # weak scaling: every rank generates and solves its own batch of cols
    # columns (seed + rank); no data-path collective
    batch = make_batch(args.cols, seed=SEED + 7919 * rank)
    my_cols = batch["ncol"]
    nch = len(CHANNELS)
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    # one launch group per (stream count, layer bucket): its arrays are
    # dimensioned by the bucket's deepest column, and the autotuner's schedule
    # for that (layers, streams) bucket is applied to its launches
    buckets = [int(x) for x in args.buckets.split(",")]
    groups = []
    for N in STREAMS:
        lo = 0
        for hi in buckets:
            idx = np.nonzero((batch["nstreams"] == N) & (batch["nlayers"] > lo) & (batch["nlayers"] <= hi))[0]
            lo = hi
            if len(idx) == 0:
                continue
            idx = idx[np.argsort(-batch["nlayers"][idx], kind="stable")]  # similar layer counts share a warp
            groups.append((N, idx))
    groups.sort(key=lambda t: -t[0] ** 3 * len(t[1]))  # costliest first
    glist, groups = groups, []

    def build_group(N, g, idx):
        km, n = g["km"], g["ncol"]
        d = {"N": N, "km": km, "n": n, "nmom": 2 * N, "host": g, "idx": idx,
             "qm": dev(g["qm"], np.float32), "rh": dev(g["rh"], np.float32), "ROT": dev(g["ROT"], np.float64),
             "depol": dev(g["depol"], np.float64), "he": dev(g["he"], np.float64),
             "albedo": dev(g["albedo"], np.float64), "sza": dev(g["sza"], np.float64),
             "raa": dev(g["raa"], np.float64), "vza": dev(g["vza"], np.float64), "nlay": dev(g["nlayers"], np.int32)}
        d["tau"] = torch.zeros(km * nch * n, dtype=torch.float32, device="cuda")
        d["ssa"] = torch.zeros_like(d["tau"])
        d["g"] = torch.zeros_like(d["tau"])
        d["pmom"] = torch.zeros(km * nch * n * 2 * N, dtype=torch.float32, device="cuda")
        for p in ("m", "d"):
            d["rad" + p] = torch.zeros(n * nch, dtype=torch.float64, device="cuda")
            d["refl" + p] = torch.zeros_like(d["rad" + p])
            d["nf" + p] = torch.zeros(n * nch, dtype=torch.int32, device="cuda")
            d["st" + p] = torch.zeros_like(d["nf" + p])
        return d
    for N, idx in glist:
        groups.append(build_group(N, subset(batch, idx), idx))
    P = lambda t: t.data_ptr()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def run_group(d, prec, s, tuned_schedule=True):
        p = "m" if prec == _lib.PREC_MIXED else "d"
        if tuned_schedule:
            autotune.apply_for(d["N"], d["km"], prec)
        fn = (L.aerort_vlidort_scalar_lambert_mixed_batch_dev if prec == _lib.PREC_MIXED
              else L.aerort_vlidort_scalar_lambert_batch_dev)
        rc = fn(d["km"], nch, d["n"], d["N"], 0, d["nmom"], P(d["nlay"]), P(d["ROT"]), P(d["depol"]), None, None, None,
                P(d["tau"]), P(d["ssa"]), P(d["pmom"]), P(d["he"]), P(d["albedo"]), P(d["sza"]), P(d["raa"]),
                P(d["vza"]), MISSING, P(d["rad" + p]), P(d["refl" + p]), P(d["nf" + p]), P(d["st" + p]), s)
        assert rc == 0, _lib.last_error()

    # every launch group on its own CUDA stream (the library keeps one scratch
    # pad per stream, for up to 16 streams), so the groups' launches overlap
    side = [torch.cuda.Stream() for _ in groups] if not args.serial else None

    def group_work(d, prec, s):
        rc = L.aerort_get_aop_vector_dev(chem.handle, d["km"], d["n"], nch, 20, _lib.ptr(ch32, _lib.P_f),
                                         _lib.ptr(qt, _lib.P_i), _lib.ptr(qb, _lib.P_i), P(d["qm"]), P(d["rh"]),
                                         d["nmom"], 1, P(d["tau"]), P(d["ssa"]), P(d["g"]), P(d["pmom"]), s)
        assert rc == 0, _lib.last_error()
        run_group(d, prec, s)

    def step(prec):
        main_s = torch.cuda.current_stream()
        if side is None:
            for d in groups:
                group_work(d, prec, main_s.cuda_stream)
            return
        for d, ss in zip(groups, side):
            ss.wait_stream(main_s)
            with torch.cuda.stream(ss):
                group_work(d, prec, ss.cuda_stream)
        for ss in side:
            main_s.wait_stream(ss)

    def timed_step(prec):
        e0, e1 = ev(), ev()
        e0.record()
        step(prec)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    tuned = None
    if args.tune:
        # each (layers, streams) bucket is tuned on its first 8,192 columns
        # (32,768 solves, several warps of 32 solves per SM for the thread kernel)
        tuned = {}
        for d in groups:
            ds = build_group(d["N"], subset(d["host"], np.arange(min(d["n"], 8192))), None)
            group_work(ds, _lib.PREC_MIXED, stream)  # the AOP optics the RT launches read
            torch.cuda.synchronize()
            for prec in (_lib.PREC_MIXED, _lib.PREC_FP64):
                r = autotune.tune(lambda: run_group(ds, prec, stream, tuned_schedule=False), ds["N"], ds["km"],
                                  prec, dev_name, budget_s=10.0 if prec == _lib.PREC_MIXED else 20.0)
                tuned["%s N%d L%d" % ("mixed" if prec else "fp64", ds["N"], ds["km"])] = r["all"]
            del ds
    else:
        tuned = {"source": tuned_src, "table": autotune.table_summary(dev_name)}

    # ---------------------------------------------------------------- mixed (headline)
    for _ in range(args.warmup):
        step(_lib.PREC_MIXED)
    torch.cuda.synchronize()
    lc0 = L.aerort_launch_count()
    rt_ms_m = timed_step(_lib.PREC_MIXED)  # one eager step: per-step kernel span and launch count
    launches_per_step = L.aerort_launch_count() - lc0
    graph, graph_note = None, "eager launches"
    if not args.eager:
        # the whole step (AOP + RT launches of every stream group) as one CUDA
        # graph; the warm-up above sized every buffer, so nothing allocates here
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, capture_error_mode="thread_local"):
            step(_lib.PREC_MIXED)
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        graph_note = "CUDA graph replay of the captured step (%d kernel launches per step)" % launches_per_step
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    t0, t1 = ev(), ev()
    torch.cuda.synchronize()
    t0.record()
    for _ in range(args.steps):
        if graph is not None:
            graph.replay()
        else:
            step(_lib.PREC_MIXED)
    t1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = launches_per_step * args.steps
    ms = t0.elapsed_time(t1) / args.steps
    if world > 1:
        tt = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms = float(tt.item())
    solves = my_cols * nch
    total_solves = solves * world
    value = total_solves / (ms * 1e-3)

    # ---------------------------------------------------------------- plain FP64 on the same batch
    # (first-launch costs of the FP64 kernels are included: < 0.1% of a step)
    rt_ms_d = 0.0
    for _ in range(args.plain_steps):
        rt_ms_d += timed_step(_lib.PREC_FP64) / args.plain_steps
    plain_value = total_solves / (rt_ms_d * 1e-3)

    # ---------------------------------------------------------------- the dominant kernel
    # every group's mixed RT launches alone on the main stream (serial, CUDA
    # events), for the roofline of the costliest one
    group_ms = []
    for d in groups:
        g0, g1 = ev(), ev()
        g0.record()
        run_group(d, _lib.PREC_MIXED, stream)
        g1.record()
        torch.cuda.synchronize()
        group_ms.append(g0.elapsed_time(g1))
    dom = int(np.argmax(group_ms))

    # ---------------------------------------------------------------- tensor-core contraction A/B
    # the dominant group's mixed RT launches with the layer-matrix moment
    # contraction on the tensor cores (3xTF32 mma.sync) and on the CUDA cores,
    # the run's own choice last (so the group's results below are its own)
    contraction_ab = None
    dgab = groups[dom]
    if dgab["N"] >= 8 and args.plain_steps > 0:
        ab = {}
        modes = [(_lib.CONTRACT_TF32X3, "tf32x3"), (_lib.CONTRACT_FMA, "fma")]
        if run_contraction == _lib.CONTRACT_TF32X3:
            modes = modes[::-1]
        for mode, name in modes:
            assert L.aerort_set_moment_contraction(mode) == 0
            run_group(dgab, _lib.PREC_MIXED, stream)
            torch.cuda.synchronize()
            best = None
            for _ in range(2):
                g0, g1 = ev(), ev()
                g0.record()
                run_group(dgab, _lib.PREC_MIXED, stream)
                g1.record()
                torch.cuda.synchronize()
                best = min(best or 1e30, g0.elapsed_time(g1))
            cnt = ctypes.c_int(0)
            L.aerort_refined_count(ctypes.c_void_p(stream), ctypes.byref(cnt))
            rm, rd = dgab["radm"].cpu().numpy(), dgab["radd"].cpu().numpy()
            ok = (rd != MISSING) & (dgab["stm"].cpu().numpy() == 0)
            e = np.abs(rm[ok] / rd[ok] - 1.0)
            ab[name] = {"ms": best, "max_rel_err_vs_fp64": float(e.max()), "median_rel_err_vs_fp64": float(np.median(e)),
                        "refined": int(cnt.value)}
        L.aerort_set_moment_contraction(run_contraction)
        contraction_ab = {"group": "N%d|L%d" % (dgab["N"], dgab["km"]), "solves": int(dgab["n"]) * nch,
                          "speedup_tf32x3": ab["fma"]["ms"] / ab["tf32x3"]["ms"], **ab,
                          "time": "the group's mixed RT launches alone on one stream, best of 2, CUDA events"}

    # ---------------------------------------------------------------- results, flops
    rad_m = np.zeros((my_cols, nch))
    rad_d = np.zeros((my_cols, nch))
    nf_d = np.zeros((my_cols, nch), np.int32)
    bad, flops = 0, 0.0
    for d in groups:
        n = d["n"]
        rad_m[d["idx"]] = d["radm"].cpu().numpy().reshape(n, nch, order="F")
        rad_d[d["idx"]] = d["radd"].cpu().numpy().reshape(n, nch, order="F")
        nf_d[d["idx"]] = d["nfd"].cpu().numpy().reshape(n, nch, order="F")
        bad += int((d["stm"].cpu().numpy() != 0).sum() + (d["std"].cpu().numpy() != 0).sum())
    ftab = flops_table()
    for N in STREAMS:
        sel = batch["nstreams"] == N
        flops += float(ftab[N][batch["nlayers"][sel][:, None], np.clip(nf_d[sel], 0, 63)].sum())
    okall = (rad_d != MISSING)
    dev_err = np.abs(rad_m[okall] / rad_d[okall] - 1.0)
    # the solves furthest from the FP64 result: column, wavelength, streams,
    # layers, error, Fourier terms (the batch is seeded, so each can be
    # re-solved on the host)
    err_full = np.zeros_like(rad_d)
    err_full[okall] = dev_err
    worst = []
    for flat in np.argsort(err_full, axis=None)[::-1][:8]:
        ci, wi = np.unravel_index(flat, err_full.shape)
        worst.append({"col": int(ci), "nm": CHANNELS[wi], "N": int(batch["nstreams"][ci]),
                      "L": int(batch["nlayers"][ci]), "err": float(err_full[ci, wi]), "nf": int(nf_d[ci, wi])})
    fp64_peak, fp32_peak, dgemm = pipe_peaks(torch, L, stream)
    ach_m = flops / (rt_ms_m * 1e-3) / 1e12
    ach_d = flops / (rt_ms_d * 1e-3) / 1e12
    dg = groups[dom]
    dom_nf = dg["nfm"].cpu().numpy().reshape(dg["n"], nch, order="F")
    dom_flops = float(ftab[dg["N"]][dg["host"]["nlayers"][:, None], np.clip(dom_nf, 0, 63)].sum())
    dom_solves = int((dom_nf >= 0).sum())
    ach_dom = dom_flops / (group_ms[dom] * 1e-3) / 1e12
    # algorithmic bytes per solve-layer of the series: FP32 tau, ssa and 2N = 32
    # moments (136 B), FP64 ROT and level height (16 B)
    traffic = None
    if dg["N"] == 16:
        traffic = TEAM16_DRAM_BYTES_PER_SOLVE_LAYER * float((dg["host"]["nlayers"][:, None] * (dom_nf >= 0)).sum())
    roofline = {"bound": "fp32", "achieved": ach_dom, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": ach_dom / fp32_peak, "traffic": traffic,
                "kernel": "k_team_setup + k_team_series<%d, float> (+ the FP64 refinement launch) of the %d-stream "
                          "group with %d-%d layers" % (dg["N"], dg["N"], int(dg["host"]["nlayers"].min()),
                                                        int(dg["host"]["nlayers"].max())),
                "kernel_ms": group_ms[dom], "solves": dom_solves,
                "kernel_time": "the group's RT launches alone on one stream, CUDA events",
                "traffic_source": "DRAM bytes per solve-layer of k_team_series<16, float> from one ncu capture "
                                  "(profiles/k_team_series_16_float_cols8192.md) x the group's solve-layers",
                "traffic_algorithmic": 152.0 * float((dg["host"]["nlayers"][:, None] * (dom_nf >= 0)).sum()),
                "peak_source": "measured live: FFMA issue-rate probe (8 FMA chains/thread), of measured",
                "note": "achieved = reference-algorithm flops (banded-LU BVP, nonsymmetric eigen-solve) of the solves "
                        "/ kernel time; the kernel executes a different, mostly FP32 operation mix",
                "whole_step": {"achieved": ach_m, "frac": ach_m / fp32_peak, "kernel_ms_per_step": rt_ms_m,
                               "group_ms": {"N%d|L%d" % (d["N"], d["km"]): ms for d, ms in zip(groups, group_ms)}}}
    roofline_plain = {"bound": "fp64", "achieved": ach_d, "peak": fp64_peak, "unit": "TFLOP/s",
                      "frac": ach_d / fp64_peak, "kernel": "k_team_series<NS, double> / k_scalar_lambert<NS, double>",
                      "kernel_ms_per_step": rt_ms_d,
                      "peak_source": "measured live: DFMA issue-rate probe, of measured; cuBLAS DGEMM %.3f TFLOP/s"
                                     % dgemm,
                      "note": "reference-algorithm flops; the kernel executes fewer (block BVP sweep, symmetric "
                              "eigen-reduction), so frac can exceed 1"}

    # ---------------------------------------------------------------- end to end through the host C ABI
    e2e = None
    if args.e2e_steps > 0:
        e2e_val, h2d, d2h, times = e2e_host_abi(L, chem, groups, qt, qb, ch32, args.e2e_steps)
        e2e = {"value": e2e_val, "unit": "radiances/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "steps": args.e2e_steps, "s_per_step": times,
               "path": "host Fortran-order arrays -> aerort_get_aop_vector (copies in, AOP kernel, FP32 optics out) "
                       "-> host dble() -> aerort_vlidort_scalar_lambert_mixed_batch (copies in, mixed RT, results "
                       "out), per stream group; host wall clock; the host reads the results"}

    # ---------------------------------------------------------------- CPU oracle: baseline and parity at scale
    cpu = acc = stress = None
    if rank == 0 and world == 1 and not args.no_cpu:
        ncs = min(args.cpu_cols or 4096, my_cols)
        orad, onf, dt = oracle_radiances(batch, ncs, CHANNELS)
        _, _, dt1 = oracle_radiances(batch, min(128, my_cols), CHANNELS, threads=1)
        cpu = {"value": ncs * nch / dt, "unit": "radiances/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "first %d columns x 4 wavelengths of the same batch: C++ oracle restating Chem_MieQuery "
                         "(FP32) + VLIDORT 2.8.3 (FP64), OpenMP over pixels, %d threads; %.1f s"
                         % (ncs, os.cpu_count(), dt),
               "single_core": {"value": 128 * nch / dt1, "unit": "radiances/s", "cores": 1,
                               "sample": "first 128 columns of the same batch, one thread; %.1f s" % dt1}}
        ok = np.isfinite(orad) & (orad != MISSING)
        per = []
        for i in range(nch):
            mx, md, n = rel_err_stats(rad_m[:ncs, i], orad[:, i], ok[:, i])
            pmx, pmd, _ = rel_err_stats(rad_d[:ncs, i], orad[:, i], ok[:, i])
            per.append({"nm": CHANNELS[i], "mixed_max": mx, "mixed_median": md, "fp64_max": pmx, "n": n})
        acc = {"vs": "FP64 oracle", "columns": ncs, "per_wavelength": per,
               "fourier_terms_identical": bool(np.array_equal(onf, nf_d[:ncs]))}
        # near-conservative stress set: aerosol SSA in [0.999, 1) on 96 columns per stream count
        pick = np.sort(np.concatenate([np.nonzero(batch["nstreams"] == N)[0][:args.stress_cols] for N in STREAMS]))
        sb = subset(batch, pick)
        ov = lambda N, s: np.asfortranarray(
            (0.999 + 0.001 * np.random.default_rng(31 + N).random(s.shape)).astype(np.float32))
        orad_s, _, _ = oracle_radiances(sb, sb["ncol"], CHANNELS, ssa_override=ov)
        stress = stress_gpu(L, sb, chem, qt, qb, ch32, ov, orad_s)

    # ---------------------------------------------------------------- config 0 (plain method)
    c0 = None
    if rank == 0 and not args.no_config0:
        c0 = config0(torch, L, fp64_peak, ftab, cpu=(world == 1 and not args.no_cpu))

    # ---------------------------------------------------------------- config 3 (polarized)
    c3 = None
    if rank == 0 and args.config3_cols > 0:
        c3 = config3(torch, L, args.config3_cols, cpu=(world == 1 and not args.no_cpu))

    # ---------------------------------------------------------------- front end kernels (ROT, edge, AOP)
    rot_line = edge_line = aop_line = None
    if rank == 0:
        rot_line, edge_line, aop_line = front_end_rooflines(torch, L, batch, stream, chem=chem, qt=qt, qb=qb)

    # ---------------------------------------------------------------- serving (config 4)
    serving = None
    if not args.no_serve and rank == 0 and args.serve_requests > 0:
        serving = serving_run(args, mie.generate_tables(list(SERVE_CHANNELS), nmom=32))

    cfg = bench_config(args)
    cfg.update({"failed_solves": bad, "tuned_schedules": tuned, "launch": graph_note, "contraction": args.contraction,
                "groups": ("%d launch groups (stream count x layer bucket <= %s), concurrent on one CUDA stream each"
                           % (len(groups), args.buckets)) if side else "serial, one CUDA stream"})
    line = {
        "metric": METRIC, "value": value, "unit": "radiances/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 (mixed: FP64 set-up and single scatter, FP32 Fourier series)", "data": "synthetic",
        "config": cfg, "gpu_launches": launches, "clocks": clk, "roofline": roofline, "cpu_baseline": cpu,
        "e2e": e2e, "rot_calc": rot_line, "edge_vars": edge_line, "aop": aop_line, "serving": serving,
        "config3_polarized": c3, "config0_plain_fp64": c0, "roofline_plain": roofline_plain,
        "contraction_ab": contraction_ab, "accuracy": acc, "accuracy_ssa_stress": stress,
        "plain_fp64": {"value": plain_value, "unit": "radiances/s", "ms_per_step": rt_ms_d, "steps": args.plain_steps,
                       "mixed_over_plain": value / plain_value,
                       "mixed_vs_fp64_gpu_max": float(dev_err.max()),
                       "mixed_vs_fp64_gpu_median": float(np.median(dev_err)), "radiances": int(dev_err.size),
                       "mixed_over_1e-4": int((dev_err > 1e-4).sum()), "worst": worst},
    }
    if rank == 0:
        print(json.dumps(line))
    chem.destroy()
    if world > 1:
        torch.distributed.destroy_process_group()


def stress_gpu(L, sb, chem, qt, qb, ch32, ov, orad_s):
    """Mixed and FP64 GPU solves of the stress set (the same overridden SSA as
    the oracle got) through the host-pointer batched entry points; max/median
    relative error per wavelength against the oracle."""
    from aeroapps_gb300 import _lib, vlidort
    nch = len(CHANNELS)
    rad_m = np.full((sb["ncol"], nch), np.nan)
    rad_d = np.full((sb["ncol"], nch), np.nan)
    for N in STREAMS:
        idx = np.nonzero(sb["nstreams"] == N)[0]
        if len(idx) == 0:
            continue
        g = subset(sb, idx)
        km, n = g["km"], g["ncol"]
        tau = np.zeros((km, nch, n), np.float32, order="F")
        ssa, gg = np.zeros_like(tau), np.zeros_like(tau)
        pm = np.zeros((km, nch, n, 2 * N, 1), np.float32, order="F")
        Pf = lambda a: _lib.ptr(a, _lib.P_f)
        rc = L.aerort_get_aop_vector(chem.handle, km, n, nch, 20, Pf(ch32), _lib.ptr(qt, _lib.P_i),
                                     _lib.ptr(qb, _lib.P_i), Pf(g["qm"]), Pf(g["rh"]), 2 * N, 1, Pf(tau), Pf(ssa),
                                     Pf(gg), Pf(pm))
        assert rc == 0, _lib.last_error()
        ssa = ov(N, ssa)
        for prec, out in (("mixed", rad_m), ("fp64", rad_d)):
            r, _, rc, _, st = vlidort.vlidort_scalar_lambert_batch(
                km, nch, n, N, 2 * N, g["nlayers"], g["ROT"], g["depol"], tau.astype(np.float64),
                ssa.astype(np.float64), pm[..., 0].astype(np.float64), g["he"], g["albedo"], g["sza"], g["raa"],
                g["vza"], MISSING=MISSING, precision=prec)
            assert rc == 0
            out[idx] = r
    ok = np.isfinite(orad_s) & (orad_s != MISSING)
    per = []
    for i in range(nch):
        mx, md, n = rel_err_stats(rad_m[:, i], orad_s[:, i], ok[:, i])
        pmx, _, _ = rel_err_stats(rad_d[:, i], orad_s[:, i], ok[:, i])
        per.append({"nm": CHANNELS[i], "mixed_max": mx, "mixed_median": md, "fp64_max": pmx, "n": n})
    return {"vs": "FP64 oracle", "set": "aerosol SSA in [0.999, 1) on %d columns of the batch (equal shares of the "
                                        "stream counts)" % sb["ncol"], "per_wavelength": per}


if __name__ == "__main__":
    main()

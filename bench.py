"""Benchmark: TOA radiances/s of the aerosol-optics + VLIDORT path on GB300.

Metric: TOA radiances per second of the mixed-precision GPU solve, whose
error against the FP64 solve is measured on every radiance of the batch and
must stay <= 1e-4, reported beside the plain FP64 GPU solve of the same
batch, with serving p50/p95/p99 latency.

Workload (one step): one batch of synthetic columns of the 262,144-column
batching configuration -- 4 wavelengths (470, 550, 670, 865 nm), per-column
layer count uniform in 20..72, half-space streams drawn from {4,6,8,12,16},
2 x streams Legendre moments.  A step runs, for every stream-count group, the
Mie-table AOP kernel (FP32) and the RT kernel on device-resident inputs.  The
optics and scratch of a step are hundreds of MB, more than the 129 MB L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
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
METRIC = ("TOA radiances/sec at <=1e-4 rel err vs FP64 (mixed-precision GPU solve; plain FP64 GPU solve and "
          "serving p50/p99 latency reported beside it)")
WORKLOAD = ("batching config: columns of the 262,144-column configuration, 20-72 layers, streams {4,6,8,12,16} "
            "(moments 2x streams), 4 wavelengths; Mie AOP (FP32) + scalar Lambertian RT per stream group")


# per stream-count group: the column inputs copied host->device and the
# outputs copied device->host in every end-to-end step
E2E_IN = ("qm", "rh", "ROT", "depol", "he", "albedo", "sza", "raa", "vza", "nlay")
E2E_OUT = ("rad", "refl", "nf", "st")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cols", type=int, default=16384, help="columns per step per GPU (x4 wavelengths = solves)")
    ap.add_argument("--plain-steps", type=int, default=1, help="timed steps of the plain FP64 solve")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--cpu-cols", type=int, default=0, help="CPU-baseline sample columns (0 = 4096, or 512 per step "
                    "of --impl reference)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=32)
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="Poisson arrival rate [requests/s]")
    ap.add_argument("--serve-max-cols", type=int, default=4096, help="largest swath of the serving run")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--tune", action="store_true", help="autotune the RT schedules before timing")
    ap.add_argument("--graph", action="store_true", help="replay the mixed step from a captured CUDA graph")
    ap.add_argument("--serial", action="store_true", help="run the stream-count groups one after another on one "
                    "CUDA stream instead of concurrently on one stream each")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


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


def table_index(tabs):
    qidx = {}
    for ti, t in enumerate(tabs.tables):
        for b in range(t.bext.shape[2]):
            qidx["%s%03d" % (t.name, b + 1)] = (ti, b)
    return qidx


def cpu_baseline(batch, ncols_sample, threads=0):
    """The oracle (C++ restatement of the reference path, OpenMP over all host
    cores, or over `threads` of them) on the first columns."""
    from oracle import oracle
    from aeroapps_gb300 import mie, synth
    sub = subset(batch, np.arange(ncols_sample))
    cores = threads or os.cpu_count() or 1
    oracle.set_threads(threads)
    tabs = mie.generate_tables(list(CHANNELS), nmom=32)
    qidx = table_index(tabs)
    qt, qb = zip(*[qidx[n] for n in synth.tracer_names()])
    t0 = time.perf_counter()
    nsolve = 0
    for N in STREAMS:
        idx = np.nonzero(sub["nstreams"] == N)[0]
        if len(idx) == 0:
            continue
        g = subset(sub, idx)
        km, n, nch = g["km"], g["ncol"], len(CHANNELS)
        tau, ssa, gg, pm, rc = oracle.get_aop_vector(tabs, km, n, nch, 20, np.float32(CHANNELS), qt, qb, g["qm"],
                                                     g["rh"], 2 * N, 1)
        oracle.scalar_lambert(km, nch, n, np.array(CHANNELS), N, 0, 2 * N, 1, g["ROT"], g["depol"], tau, ssa, gg, pm,
                              g["pe"], g["he"], g["te"], g["albedo"], g["sza"], g["raa"], g["vza"], -1.0e15,
                              nlay=g["nlayers"])
        nsolve += n * nch
    dt = time.perf_counter() - t0
    oracle.set_threads(0)
    return {"value": nsolve / dt, "unit": "radiances/s", "cores": cores, "kind": "port",
            "sample": "%d columns x %d wavelengths of the same batch (4-16 streams, 20-72 layers): C++ oracle restating "
                      "VLIDORT 2.8.3 + Chem_MieQuery (FP64), OpenMP over pixels, %d host threads; %.1f s"
                      % (ncols_sample, len(CHANNELS), cores, dt)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    batch = make_batch(max(args.cpu_cols or 512, 8), seed=20261204)  # about 2-5 s per step on 8-16 cores
    ncols = batch["ncol"]
    times = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(batch, ncols)
        if i >= args.warmup:
            times.append(ncols * len(CHANNELS) / r["value"])
    v = ncols * len(CHANNELS) * len(times) / sum(times)
    line = {"metric": METRIC, "value": v, "unit": "radiances/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "columns_per_step": ncols, "wavelengths": list(CHANNELS)},
            "cpu_baseline": {"value": v, "unit": "radiances/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "%d columns x 4 wavelengths per step; the reference Fortran cannot be built "
                                       "here or on the GPU host (no Fortran compiler), so its C++ restatement runs "
                                       "(FP64, OpenMP over pixels)" % ncols},
            "e2e": {"value": v, "unit": "radiances/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _hbm_peak():
    try:
        peak = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")))["hbm_gbs"]
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
    my_cols = batch["ncol"]
    nch = len(CHANNELS)
    peak, src = _hbm_peak()
    # Fortran (k, columns) = C (columns, k), tiled to ncr columns
    tile = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).T)).cuda().repeat(
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
                "limiter": "FP64 issue: two correctly rounded FP64 divisions per layer edge and pixel (bit "
                           "identity with the reference rules out reciprocal products); GB300 runs FP64 at "
                           "about 1 TFLOP/s",
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
        ua = synth.make_columns(min(batch["ncol"], 4096), list(CHANNELS), seed=5, nlayers=km)
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
    stream = torch.cuda.current_stream().cuda_stream
    dev_name = torch.cuda.get_device_name(local)
    autotune.apply_cached(dev_name)
    tabs = mie.generate_tables(list(CHANNELS), nmom=32)
    chem = mie.ChemMie(tabs)
    names = synth.tracer_names()
    qt = np.array([chem.query_idx(n)[0] for n in names], np.int32)
    qb = np.array([chem.query_idx(n)[1] for n in names], np.int32)
    ch32 = np.array(CHANNELS, np.float32)
    # weak scaling: a global batch of cols x world columns, each rank solving its
    # cost-balanced contiguous share (aeroapps_gb300.shard); no data-path collective
    from aeroapps_gb300 import shard
    full = make_batch(args.cols * world, seed=20261204)
    if world > 1:
        batch = subset(full, shard.my_columns(full["nstreams"], full["nlayers"], rank, world))
    else:
        batch = full
    my_cols = batch["ncol"]
    nch = len(CHANNELS)
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).cuda()
    groups = []
    for N in STREAMS:
        idx = np.nonzero(batch["nstreams"] == N)[0]
        if len(idx) == 0:
            continue
        idx = idx[np.argsort(-batch["nlayers"][idx], kind="stable")]  # similar layer counts share a warp
        g = subset(batch, idx)
        km, n = g["km"], g["ncol"]
        d = {"N": N, "km": km, "n": n, "nmom": 2 * N, "host": g,
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
        # pinned host copies of the step's inputs and outputs (end-to-end timing)
        for k in E2E_IN:
            d["pin_" + k] = d[k].cpu().pin_memory()
        for k in E2E_OUT:
            d["pin_" + k] = torch.empty_like(d[k + "m"], device="cpu").pin_memory()
        groups.append(d)
    P = lambda t: t.data_ptr()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def run_group(d, prec, stream=None):
        stream = stream or torch.cuda.current_stream().cuda_stream
        p = "m" if prec == _lib.PREC_MIXED else "d"
        fn = (L.aerort_vlidort_scalar_lambert_mixed_batch_dev if prec == _lib.PREC_MIXED
              else L.aerort_vlidort_scalar_lambert_batch_dev)
        rc = fn(d["km"], nch, d["n"], d["N"], 0, d["nmom"], P(d["nlay"]), P(d["ROT"]), P(d["depol"]), None, None, None,
                P(d["tau"]), P(d["ssa"]), P(d["pmom"]), P(d["he"]), P(d["albedo"]), P(d["sza"]), P(d["raa"]),
                P(d["vza"]), -1.0e15, P(d["rad" + p]), P(d["refl" + p]), P(d["nf" + p]), P(d["st" + p]), stream)
        assert rc == 0, _lib.last_error()

    # every stream-count group on its own CUDA stream (the library keeps one
    # scratch pad per stream), so the groups' launches overlap on the GPU
    side = [torch.cuda.Stream() for _ in groups] if not args.serial else None

    def group_work(d, prec, s, e2e=False):
        if e2e:
            for k in E2E_IN:
                d[k].copy_(d["pin_" + k], non_blocking=True)
        rc = L.aerort_get_aop_vector_dev(chem.handle, d["km"], d["n"], nch, 20, _lib.ptr(ch32, _lib.P_f),
                                         _lib.ptr(qt, _lib.P_i), _lib.ptr(qb, _lib.P_i), P(d["qm"]), P(d["rh"]),
                                         d["nmom"], 1, P(d["tau"]), P(d["ssa"]), P(d["g"]), P(d["pmom"]), s)
        assert rc == 0, _lib.last_error()
        run_group(d, prec, s)
        if e2e:
            for k in E2E_OUT:
                d["pin_" + k].copy_(d[k + "m"], non_blocking=True)

    def step(prec, rt_events=None, e2e=False):
        main = torch.cuda.current_stream()
        if rt_events is not None:
            e0, e1 = ev(), ev()
            e0.record()
        if side is None:
            for d in groups:
                group_work(d, prec, main.cuda_stream, e2e)
        else:
            for d, ss in zip(groups, side):
                ss.wait_stream(main)
                with torch.cuda.stream(ss):
                    group_work(d, prec, ss.cuda_stream, e2e)
            for ss in side:
                main.wait_stream(ss)
        if rt_events is not None:
            e1.record()
            rt_events.append((0, e0, e1))

    tuned = {}
    if args.tune:
        for d in groups:
            for prec in (_lib.PREC_MIXED, _lib.PREC_FP64):
                r = autotune.tune(lambda: run_group(d, prec), d["N"], prec, dev_name,
                                  budget_s=20.0 if prec == _lib.PREC_MIXED else 40.0)
                tuned["%s N%d" % ("mixed" if prec else "fp64", d["N"])] = (
                    "team" if r["kernel"] == _lib.KERNEL_TEAM else "thread", r["threads"], r["blocks_per_sm"])

    # Concurrent groups are launched in stream-count order; each group's
    # persistent kernel takes the SMs it can get, and the next groups' blocks
    # fill them as it drains.  (Measured on GB300: capping each group's resident
    # blocks to a cost-proportional share of the SMs was 25% slower, since SMs
    # freed by a group that finishes early stay idle; launching the costliest
    # group first was no faster.)

    # ---------------------------------------------------------------- mixed (headline)
    for _ in range(args.warmup):
        step(_lib.PREC_MIXED)
    torch.cuda.synchronize()
    graph, graph_note = None, "eager launches"
    if args.graph:
        # the whole step (AOP + RT launches of every stream group) as one CUDA
        # graph; the warm-up above sized every buffer, so nothing allocates here
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            step(_lib.PREC_MIXED)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        graph, graph_note = g, "CUDA graph replay of the captured step"
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    t0, t1 = ev(), ev()
    rt_m = []
    torch.cuda.synchronize()
    lc0 = L.aerort_launch_count()
    t0.record()
    for _ in range(args.steps):
        if graph is not None:
            graph.replay()
        else:
            step(_lib.PREC_MIXED, rt_m)
    t1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = L.aerort_launch_count() - lc0  # the library's kernel launches in the timed region
    if graph is not None:  # per-kernel times from one eager step; a replay launches that step's kernels
        lc0 = L.aerort_launch_count()
        step(_lib.PREC_MIXED, rt_m)
        torch.cuda.synchronize()
        launches = (L.aerort_launch_count() - lc0) * args.steps
    ms = t0.elapsed_time(t1) / args.steps
    if world > 1:
        tt = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms = float(tt.item())
    solves = my_cols * nch
    total_solves = solves
    if world > 1:
        ts = torch.tensor([float(solves)], device="cuda")
        torch.distributed.all_reduce(ts, op=torch.distributed.ReduceOp.SUM)
        total_solves = float(ts.item())
    value = total_solves / (ms * 1e-3)
    rt_ms_m = sum(e0.elapsed_time(e1) for (_, e0, e1) in rt_m) / (1 if graph is not None else args.steps)

    # ---------------------------------------------------------------- plain FP64 on the same batch
    step(_lib.PREC_FP64)
    torch.cuda.synchronize()
    rt_d = []
    p0, p1 = ev(), ev()
    p0.record()
    for _ in range(args.plain_steps):
        step(_lib.PREC_FP64, rt_d)
    p1.record()
    torch.cuda.synchronize()
    ms_plain = p0.elapsed_time(p1) / args.plain_steps
    rt_ms_d = sum(e0.elapsed_time(e1) for (_, e0, e1) in rt_d) / args.plain_steps
    plain_value = total_solves / (ms_plain * 1e-3)

    # ---------------------------------------------------------------- accuracy of mixed vs FP64, flops
    errs, bad, flops = [], 0, 0.0
    for d in groups:
        rm, rd = d["radm"].cpu().numpy(), d["radd"].cpu().numpy()
        stm, std_ = d["stm"].cpu().numpy(), d["std"].cpu().numpy()
        bad += int((stm != 0).sum() + (std_ != 0).sum())
        ok = (rd != -1.0e15) & (stm == 0) & (std_ == 0)
        errs.append(np.abs(rm[ok] / rd[ok] - 1.0))
        nf = d["nfd"].cpu().numpy().reshape(d["n"], nch, order="F")
        nl = d["host"]["nlayers"]
        for j in range(d["n"]):
            for i in range(nch):
                flops += alg_flops(d["N"], int(nl[j]), int(nf[j, i]))
    err = np.concatenate(errs)
    fp64_peak, fp32_peak, dgemm = pipe_peaks(torch, L, stream)
    ach_m = flops / (rt_ms_m * 1e-3) / 1e12
    ach_d = flops / (rt_ms_d * 1e-3) / 1e12
    roofline = {"bound": "fp32", "achieved": ach_m, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach_m / fp32_peak,
                "traffic": None, "kernel": "k_scalar_lambert<NS, float> (mixed; all stream counts)",
                "kernel_ms_per_step": rt_ms_m,
                "kernel_time": "span of the step's launches (all stream groups, AOP kernels included at <1%)",
                "peak_source": "measured live: FFMA issue-rate probe (8 FMA chains/thread), of measured",
                "note": "achieved = reference-algorithm flops (banded-LU BVP, nonsymmetric eigen-solve) of the solves "
                        "/ kernel time; the kernel executes a different, mostly FP32 operation mix"}
    roofline_plain = {"bound": "fp64", "achieved": ach_d, "peak": fp64_peak, "unit": "TFLOP/s",
                      "frac": ach_d / fp64_peak, "kernel": "k_scalar_lambert<NS, double> (plain FP64)",
                      "kernel_ms_per_step": rt_ms_d,
                      "peak_source": "measured live: DFMA issue-rate probe, of measured; cuBLAS DGEMM %.3f TFLOP/s"
                                     % dgemm,
                      "note": "reference-algorithm flops; the kernel executes fewer (block BVP sweep, symmetric "
                              "eigen-reduction), so frac can exceed 1"}

    # ---------------------------------------------------------------- end to end from pinned host memory
    # per group and step: host->device copy of the column inputs, the AOP and
    # mixed RT entry points of the C ABI, device->host copy of radiance,
    # reflectance, Fourier count and status; the host reads the results
    e2e_val, h2d, d2h = None, 0, 0
    if args.e2e_steps > 0:
        h2d = sum(d["pin_" + k].numel() * d["pin_" + k].element_size() for d in groups for k in E2E_IN)
        d2h = sum(d["pin_" + k].numel() * d["pin_" + k].element_size() for d in groups for k in E2E_OUT)
        step(_lib.PREC_MIXED, e2e=True)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(args.e2e_steps):
            step(_lib.PREC_MIXED, e2e=True)
            torch.cuda.synchronize()
            got = sum(float(d["pin_rad"][0]) for d in groups)  # the host reads the step's results
        e2e_val = solves / ((time.perf_counter() - t) / args.e2e_steps)
        assert np.isfinite(got)

    # ---------------------------------------------------------------- front end kernels (ROT, edge profiles)
    rot_line = edge_line = aop_line = None
    if rank == 0:
        rot_line, edge_line, aop_line = front_end_rooflines(torch, L, batch, stream, chem=chem, qt=qt, qb=qb)

    # ---------------------------------------------------------------- serving
    serving = None
    if not args.no_serve and rank == 0 and args.serve_requests > 0:
        from aeroapps_gb300 import serve
        rng = np.random.default_rng(4)
        sizes = np.exp(rng.uniform(np.log(64), np.log(args.serve_max_cols), args.serve_requests)).astype(int)
        nchs = rng.integers(1, 5, args.serve_requests)
        mk = lambda: [serve.make_swath(i, int(sizes[i]), list(CHANNELS[: nchs[i]]), seed=5000 + i)
                      for i in range(args.serve_requests)]
        srv = serve.Server(tabs, nslots=4, precision="mixed", hbm_budget_gb=120.0)
        warm = serve.make_swath(999, 64, list(CHANNELS), seed=1)
        srv.submit(warm)
        srv.drain()
        srv.done.clear()
        sw = mk()
        done, wall = serve.run_poisson(srv, sw, args.serve_rate, seed=9)
        stats = serve.latency_stats(done)
        rads = sum(s.radiances for s in done)
        # the same mix as one offline batch (all submitted at once)
        sw2 = mk()
        srv.done.clear()
        t = time.perf_counter()
        for s in sw2:
            srv.submit(s)
        srv.drain()
        offline = sum(s.radiances for s in sw2) / (time.perf_counter() - t)
        # the same request mix at half the measured capacity: latency of the
        # pipeline itself rather than of the queue
        mean_rads = sum(s.radiances for s in sw2) / len(sw2)
        half_rate = 0.5 * offline / mean_rads
        sw3 = mk()
        srv.done.clear()
        done3, wall3 = serve.run_poisson(srv, sw3, half_rate, seed=11)
        stats3 = serve.latency_stats(done3)
        stats3.update({"arrival_rate_per_s": half_rate,
                       "sustained_radiances_per_s": sum(s.radiances for s in done3) / wall3})
        srv.close()
        serving = dict(stats)
        serving.update({"arrival_rate_per_s": args.serve_rate, "sustained_radiances_per_s": rads / wall,
                        "offline_batch_radiances_per_s": offline, "slots": 4, "precision": "mixed",
                        "swath_columns": "log-uniform %d..%d" % (64, args.serve_max_cols),
                        "wavelengths_per_request": "1-4", "hbm_budget_gb": 120.0,
                        "note": "at the configured rate the GPU is saturated, so latency is queueing; "
                                "at_half_capacity repeats the mix at half the measured offline throughput",
                        "at_half_capacity": stats3})

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(batch, min(args.cpu_cols or 4096, my_cols))  # about 10 s on a 16-core host
        one = cpu_baseline(batch, min(128, my_cols), threads=1)  # about 5 s on one core
        cpu["single_core"] = {"value": one["value"], "unit": one["unit"], "cores": 1, "sample": one["sample"]}
    line = {
        "metric": METRIC, "value": value, "unit": "radiances/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 (mixed: FP64 set-up and single scatter, FP32 Fourier series)", "data": "synthetic",
        "config": {"workload": WORKLOAD + "; one step = %d columns x 4 wavelengths per GPU" % args.cols,
                   "columns_per_step": args.cols, "solves_per_step": solves, "wavelengths": list(CHANNELS),
                   "l2": "inputs larger than L2 (optics + scratch of a step: hundreds of MB)",
                   "failed_solves": bad, "tuned_schedules": tuned or None, "launch": graph_note,
                   "groups": "concurrent, one CUDA stream per stream count" if side else "serial, one CUDA stream"},
        "accuracy": {"max_rel_err_vs_fp64": float(err.max()), "median_rel_err_vs_fp64": float(np.median(err)),
                     "radiances_compared": int(err.size), "bar": 1e-4},
        "plain_fp64": {"value": plain_value, "unit": "radiances/s", "ms_per_step": ms_plain,
                       "steps": args.plain_steps, "mixed_over_plain": value / plain_value},
        "roofline": roofline, "roofline_plain": roofline_plain, "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": "radiances/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "pinned host inputs -> device copies, aerort_get_aop_vector_dev + "
                        "aerort_vlidort_scalar_lambert_mixed_batch_dev per stream group (%s), device -> pinned host "
                        "outputs, host read" % ("one CUDA stream per group" if side else "one stream")},
        "serving": serving, "gpu_launches": launches, "clocks": clk, "rot_calc": rot_line, "edge_vars": edge_line, "aop": aop_line,
    }
    if rank == 0:
        print(json.dumps(line))
    chem.destroy()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""Serving loop: continuous batching of retrieval / simulator swaths on one GPU.

A request is a swath of columns (each with its own stream count and layer
count) at 1-8 wavelengths.  The server keeps the Mie tables resident on the
device and owns a fixed set of slots.  Each slot has a CUDA stream and a
caller-owned RT workspace (aerort_workspace), so that slots run concurrently
without sharing scratch.  A request is admitted as soon as a slot is free and
its device-memory estimate fits both the configured HBM budget (the device
memory the server may hold for requests in flight) and the free device memory
the CUDA driver reports.  Requests that arrive while others are on the GPU are
admitted as slots free up, and their kernels overlap on the device.  A request
completes when the event recorded after its last device->host copy fires;
latency is completion minus arrival.

Per request, for every stream-count group of its columns, on the slot's stream:
host->device copy of the column inputs (pinned), VLIDORT_getAOPvector
(aerort_get_aop_vector_dev, FP32), the RT solve (aerort_vlidort_scalar_lambert_ws_dev,
mixed or FP64), device->host copy of radiance / reflectance / Fourier count /
status.  Every solve's result depends on its own inputs only (whichever thread
or warp runs it), so a request's result is the same alone and in the mix.
(One stream and workspace per stream-count group in each slot, so that a
request's groups run concurrently, was measured on GB300: same latency at half
capacity, 35% lower offline throughput.)
"""
import collections
import ctypes
import dataclasses
import threading
import time

import numpy as np

from . import _lib, mie, synth

MISSING = -1.0e15
STREAMS = (4, 6, 8, 12, 16)


@dataclasses.dataclass
class Swath:
    """One request: columns (synth.make_columns layout) at `channels` [nm]."""
    rid: int
    cols: dict
    nstreams: np.ndarray          # (ncol,) half-space streams per column
    channels: list
    t_arrival: float = 0.0        # seconds on the server clock
    t_admit: float = 0.0
    t_done: float = 0.0
    radiance: np.ndarray = None   # (ncol, nch)
    reflectance: np.ndarray = None
    nfourier: np.ndarray = None
    status: np.ndarray = None

    @property
    def ncol(self):
        return self.cols["ncol"]

    @property
    def radiances(self):
        return self.ncol * len(self.channels)


def _group(cols, idx):
    """Columns idx of a make_columns dict, with km trimmed to their deepest column."""
    out = {"ncol": len(idx)}
    nl = cols["nlayers"][idx]
    km = int(nl.max())
    out["km"] = km
    out["nlayers"] = np.ascontiguousarray(nl, np.int32)
    F = np.asfortranarray
    out["qm"] = F(cols["qm"][:km, :, idx])
    out["rh"] = F(cols["rh"][:km, idx])
    out["ROT"] = F(cols["ROT"][:km, idx, :])
    out["he"] = F(cols["he"][: km + 1, idx])
    out["albedo"] = F(cols["albedo"][idx, :])
    for k in ("sza", "raa", "vza"):
        out[k] = np.ascontiguousarray(cols[k][idx])
    out["depol"] = cols["depol"]
    return out


def request_bytes(swath, precision, ws_bytes):
    """Device memory a request holds while in flight (inputs, optics, outputs);
    the slot workspace is preallocated and not counted."""
    nch = len(swath.channels)
    tot = 0
    for N in STREAMS:
        n = int((swath.nstreams == N).sum())
        if n == 0:
            continue
        km = int(swath.cols["nlayers"][swath.nstreams == N].max())
        tot += km * n * (20 + 1) * 4                       # qm, rh
        tot += km * n * nch * 8 + (km + 1) * n * 8 + n * nch * 8 + 3 * n * 8 + n * 4 + nch * 8
        tot += km * n * nch * (3 + 2 * N) * 4              # tau, ssa, g, pmom (FP32)
        tot += n * nch * (8 + 8 + 4 + 4)                   # outputs
    return tot


def can_admit(request_bytes_, inflight_bytes, budget_bytes, free_bytes, reserve_bytes):
    """Admission by device memory: the request must fit in the budget next to
    the requests already in flight, and in the free device memory minus a
    reserve."""
    return (inflight_bytes + request_bytes_ <= budget_bytes) and (request_bytes_ <= free_bytes - reserve_bytes)


class Server:
    def __init__(self, tables, nslots=4, precision="mixed", hbm_budget_gb=120.0, slot_fraction=None,
                 reserve_gb=2.0):
        import torch
        self.torch = torch
        self.L = _lib.lib()
        self.prec = _lib.PREC_MIXED if precision == "mixed" else _lib.PREC_FP64
        self.tables = tables
        self.table_nm = [float(x) for x in np.asarray(tables.channels_m) * 1e9]
        self.chem = mie.ChemMie(tables)
        names = synth.tracer_names()
        self.qt = np.array([self.chem.query_idx(x)[0] for x in names], np.int32)
        self.qb = np.array([self.chem.query_idx(x)[1] for x in names], np.int32)
        self.budget = int(hbm_budget_gb * (1 << 30))
        self.reserve = int(reserve_gb * (1 << 30))
        props = torch.cuda.get_device_properties(torch.cuda.current_device())
        # each slot's workspace holds 1/nslots of the threads the GPU keeps resident
        frac = slot_fraction if slot_fraction is not None else 1.0 / nslots
        threads = max(64, int(props.multi_processor_count * 256 * frac) // 64 * 64)
        per_thread = self.L.aerort_workspace_bytes_per_thread(72, 16, self.prec)
        self.ws_bytes = per_thread * threads
        self.slots = []
        for _ in range(nslots):
            ws = ctypes.c_void_p()
            rc = self.L.aerort_workspace_create(self.ws_bytes, ctypes.byref(ws))
            if rc != 0:
                raise RuntimeError("workspace_create rc=%d: %s" % (rc, _lib.last_error()))
            self.slots.append({"stream": torch.cuda.Stream(), "ws": ws, "busy": None})
        self.queue = collections.deque()
        self.lock = threading.Lock()
        self.inflight_bytes = 0
        self.done = []
        self.t0 = time.perf_counter()

    def now(self):
        return time.perf_counter() - self.t0

    def close(self):
        for s in self.slots:
            s["stream"].synchronize()
            self.L.aerort_workspace_destroy(s["ws"])
        self.slots = []
        self.chem.destroy()

    # ------------------------------------------------------------------ request path
    def submit(self, swath):
        swath.t_arrival = self.now()
        with self.lock:
            self.queue.append(swath)

    def _issue(self, slot, sw):
        torch = self.torch
        L = self.L
        nch = len(sw.channels)
        ch32 = np.array(sw.channels, np.float32)
        keep = []
        outs = []
        with torch.cuda.stream(slot["stream"]):
            st = slot["stream"].cuda_stream
            for N in STREAMS:
                idx = np.nonzero(sw.nstreams == N)[0]
                if len(idx) == 0:
                    continue
                g = _group(sw.cols, idx)
                km, n = g["km"], g["ncol"]

                def dev(a, dt):
                    h = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).pin_memory()
                    d = torch.empty(h.shape, dtype=h.dtype, device="cuda")
                    d.copy_(h, non_blocking=True)
                    keep.append(h)
                    return d
                qm, rh = dev(g["qm"], np.float32), dev(g["rh"], np.float32)
                rot, depol, he = dev(g["ROT"], np.float64), dev(g["depol"], np.float64), dev(g["he"], np.float64)
                alb, sza = dev(g["albedo"], np.float64), dev(g["sza"], np.float64)
                raa, vza, nl = dev(g["raa"], np.float64), dev(g["vza"], np.float64), dev(g["nlayers"], np.int32)
                tau = torch.empty(km * nch * n, dtype=torch.float32, device="cuda")
                ssa, gg = torch.empty_like(tau), torch.empty_like(tau)
                pm = torch.empty(km * nch * n * 2 * N, dtype=torch.float32, device="cuda")
                rc = L.aerort_get_aop_vector_dev(self.chem.handle, km, n, nch, 20, _lib.ptr(ch32, _lib.P_f),
                                                 _lib.ptr(self.qt, _lib.P_i), _lib.ptr(self.qb, _lib.P_i),
                                                 qm.data_ptr(), rh.data_ptr(), 2 * N, 1, tau.data_ptr(),
                                                 ssa.data_ptr(), gg.data_ptr(), pm.data_ptr(), st)
                if rc != 0:
                    raise RuntimeError("aop rc=%d: %s" % (rc, _lib.last_error()))
                rad = torch.empty(n * nch, dtype=torch.float64, device="cuda")
                refl = torch.empty_like(rad)
                nf = torch.empty(n * nch, dtype=torch.int32, device="cuda")
                sts = torch.empty_like(nf)
                rc = L.aerort_vlidort_scalar_lambert_ws_dev(
                    slot["ws"], self.prec, km, nch, n, N, 0, 2 * N, nl.data_ptr(), rot.data_ptr(), depol.data_ptr(),
                    None, None, None, tau.data_ptr(), ssa.data_ptr(), pm.data_ptr(), he.data_ptr(), alb.data_ptr(),
                    sza.data_ptr(), raa.data_ptr(), vza.data_ptr(), MISSING, rad.data_ptr(), refl.data_ptr(),
                    nf.data_ptr(), sts.data_ptr(), st)
                if rc != 0:
                    raise RuntimeError("rt rc=%d: %s" % (rc, _lib.last_error()))
                hrad = torch.empty(rad.shape, dtype=rad.dtype, pin_memory=True)
                hrefl = torch.empty(refl.shape, dtype=refl.dtype, pin_memory=True)
                hnf = torch.empty(nf.shape, dtype=nf.dtype, pin_memory=True)
                hst = torch.empty(sts.shape, dtype=sts.dtype, pin_memory=True)
                hrad.copy_(rad, non_blocking=True)
                hrefl.copy_(refl, non_blocking=True)
                hnf.copy_(nf, non_blocking=True)
                hst.copy_(sts, non_blocking=True)
                keep += [qm, rh, rot, depol, he, alb, sza, raa, vza, nl, tau, ssa, gg, pm, rad, refl, nf, sts]
                outs.append((idx, hrad, hrefl, hnf, hst, n))
            ev = torch.cuda.Event()
            ev.record(slot["stream"])
        return ev, keep, outs

    def _finish(self, sw, outs):
        nch = len(sw.channels)
        sw.radiance = np.zeros((sw.ncol, nch))
        sw.reflectance = np.zeros((sw.ncol, nch))
        sw.nfourier = np.zeros((sw.ncol, nch), np.int32)
        sw.status = np.zeros((sw.ncol, nch), np.int32)
        for idx, hrad, hrefl, hnf, hst, n in outs:
            sw.radiance[idx] = hrad.numpy().reshape(n, nch, order="F")
            sw.reflectance[idx] = hrefl.numpy().reshape(n, nch, order="F")
            sw.nfourier[idx] = hnf.numpy().reshape(n, nch, order="F")
            sw.status[idx] = hst.numpy().reshape(n, nch, order="F")

    def step(self):
        """Complete finished requests and admit waiting ones; returns True if anything is pending."""
        torch = self.torch
        for slot in self.slots:
            b = slot["busy"]
            if b is not None and b["event"].query():
                sw = b["swath"]
                self._finish(sw, b["outs"])
                sw.t_done = self.now()
                self.inflight_bytes -= b["bytes"]
                slot["busy"] = None
                self.done.append(sw)
        for slot in self.slots:
            if slot["busy"] is not None:
                continue
            with self.lock:
                if not self.queue:
                    break
                sw = self.queue[0]
            need = request_bytes(sw, self.prec, self.ws_bytes)
            free, _ = torch.cuda.mem_get_info()
            if not can_admit(need, self.inflight_bytes, self.budget, free, self.reserve):
                break
            with self.lock:
                self.queue.popleft()
            sw.t_admit = self.now()
            ev, keep, outs = self._issue(slot, sw)
            self.inflight_bytes += need
            slot["busy"] = {"swath": sw, "event": ev, "keep": keep, "outs": outs, "bytes": need}
        with self.lock:
            pending = bool(self.queue)
        return pending or any(s["busy"] is not None for s in self.slots)

    def drain(self):
        while self.step():
            time.sleep(0.0002)


def make_swath(rid, ncol, channels, seed, streams=STREAMS, layers=(20, 72)):
    """A request with config-1/4 distributions: per-column streams and layer counts."""
    rng = np.random.default_rng(seed)
    nl = rng.integers(layers[0], layers[1] + 1, ncol)
    ns = rng.choice(np.array(streams), ncol)
    cols = synth.make_columns(ncol, list(channels), seed=seed + 1, nlayers=nl)
    return Swath(rid=rid, cols=cols, nstreams=ns, channels=list(channels))


def run_poisson(server, swaths, rate_per_s, seed=0):
    """Submit swaths at Poisson arrival times (rate_per_s) while serving; returns
    the completed swaths and the wall time from the first arrival to the last completion."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, len(swaths))
    t_start = server.now()
    arrivals = t_start + np.cumsum(gaps) - gaps[0]
    i = 0
    while i < len(swaths) or server.step():
        now = server.now()
        while i < len(swaths) and arrivals[i] <= now:
            server.submit(swaths[i])
            i += 1
        server.step()
        if i < len(swaths):
            time.sleep(min(0.0002, max(0.0, arrivals[i] - server.now())))
    return server.done, server.now() - t_start


def latency_stats(swaths):
    lat = np.array([s.t_done - s.t_arrival for s in swaths])
    return {"p50_ms": 1e3 * float(np.percentile(lat, 50)), "p95_ms": 1e3 * float(np.percentile(lat, 95)),
            "p99_ms": 1e3 * float(np.percentile(lat, 99)), "mean_ms": 1e3 * float(lat.mean()), "requests": len(lat)}

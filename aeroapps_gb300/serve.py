"""Serving loop: continuous batching of retrieval / simulator swaths on one GPU.

A request is a swath of columns (each with its own stream count and layer
count) at 1-8 wavelengths.  The server keeps the Mie tables resident on the
device.  Whenever one of its `nslots` batch lanes is free and requests are
waiting, it merges the waiting requests, in arrival order, into one batch
(up to `max_batch_cols` columns, and only as far as the batch's
device-memory estimate fits the configured HBM budget next to the batches in
flight and the free device memory the CUDA driver reports).  A batch is
solved as one launch group per stream count, each on its own CUDA stream
(the library keeps one scratch pad per stream), over the union of the
batch's wavelengths: a column's wavelengths that its request did not ask for
get a MISSING albedo, which the solver skips at set-up.  A batch lane's
groups overlap on the device with each other and with the other lane's
batch, while the host merges the next batch.  A request completes when the
event recorded after its batch's last device->host copy fires; latency is
completion minus arrival.

Per launch group, on its stream: host->device copy of the merged column
inputs (pinned), VLIDORT_getAOPvector (aerort_get_aop_vector_dev, FP32), the
RT solve (aerort_vlidort_scalar_lambert_mixed_batch_dev or _batch_dev), and
device->host copy of radiance / reflectance / Fourier count / status.
Every solve's result depends on its own inputs only, and the server fixes the
kernel of each stream count (thread or team) for its lifetime, so a
request's result is the same alone and in any mix.
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


def request_bytes(swath, precision=None, ws_bytes=0):
    """Device memory a request alone holds while in flight (inputs, optics,
    outputs); the library's per-stream scratch is not counted."""
    return batch_bytes([swath], len(swath.channels))


def can_admit(request_bytes_, inflight_bytes, budget_bytes, free_bytes, reserve_bytes):
    """Admission by device memory: the request must fit in the budget next to
    the requests already in flight, and in the free device memory minus a
    reserve."""
    return (inflight_bytes + request_bytes_ <= budget_bytes) and (request_bytes_ <= free_bytes - reserve_bytes)


def _take(a, km, idx, axis):
    """a[:km, ..., idx, ...] along `axis` (the column axis), zero-padded to km
    rows when a holds fewer (its request's deepest column is shallower)."""
    sl = [slice(None)] * a.ndim
    sl[0] = slice(0, min(km, a.shape[0]))
    sl[axis] = idx
    out = a[tuple(sl)]
    if out.shape[0] < km:
        pad = [(0, km - out.shape[0])] + [(0, 0)] * (a.ndim - 1)
        out = np.pad(out, pad)
    return out


def batch_bytes(swaths, nch):
    """Device memory of one merged batch over nch wavelengths (inputs, optics,
    outputs); the library's per-stream scratch is not counted."""
    tot = 0
    for N in STREAMS:
        n, km = 0, 0
        for sw in swaths:
            sel = sw.nstreams == N
            if sel.any():
                n += int(sel.sum())
                km = max(km, int(sw.cols["nlayers"][sel].max()))
        if n == 0:
            continue
        tot += km * n * (20 + 1) * 4
        tot += km * n * nch * 8 + (km + 1) * n * 8 + n * nch * 8 + 3 * n * 8 + n * 4 + nch * 8
        tot += km * n * nch * (3 + 2 * N) * 4
        tot += n * nch * (8 + 8 + 4 + 4)
    return tot


def merge_group(batch, N, chans):
    """The columns with N streams of every request of `batch`, in request
    order, over the wavelengths `chans`: the RT and AOP inputs of one launch
    (Fortran order, km = the deepest column), with albedo MISSING at the
    wavelengths a column's request did not ask for, and `rows`: per request
    (swath, its column indices, their rows in the launch, the launch
    wavelength index of each of its channels).  None if no column has N
    streams."""
    parts = [(sw, np.nonzero(sw.nstreams == N)[0]) for sw in batch]
    parts = [(sw, idx) for sw, idx in parts if len(idx)]
    if not parts:
        return None
    nch = len(chans)
    n = sum(len(idx) for _, idx in parts)
    km = max(int(sw.cols["nlayers"][idx].max()) for sw, idx in parts)
    F = np.asfortranarray
    g = {"km": km, "n": n}
    g["qm"] = F(np.concatenate([_take(sw.cols["qm"], km, idx, 2) for sw, idx in parts], axis=2))
    g["rh"] = F(np.concatenate([_take(sw.cols["rh"], km, idx, 1) for sw, idx in parts], axis=1))
    g["he"] = F(np.concatenate([_take(sw.cols["he"], km + 1, idx, 1) for sw, idx in parts], axis=1))
    g["nlayers"] = np.concatenate([sw.cols["nlayers"][idx] for sw, idx in parts]).astype(np.int32)
    for k in ("sza", "raa", "vza"):
        g[k] = np.concatenate([sw.cols[k][idx] for sw, idx in parts])
    rot = np.zeros((km, n, nch), order="F")
    alb = np.full((n, nch), MISSING, order="F")
    depol = np.zeros(nch)
    rows, o = [], 0
    for sw, idx in parts:
        pos = [chans.index(float(c)) for c in sw.channels]
        r = _take(sw.cols["ROT"], km, idx, 1)
        for j, p in enumerate(pos):
            rot[:, o:o + len(idx), p] = r[:, :, j]
            alb[o:o + len(idx), p] = sw.cols["albedo"][idx, j]
            depol[p] = sw.cols["depol"][j]
        rows.append((sw, idx, np.arange(o, o + len(idx)), pos))
        o += len(idx)
    g.update(ROT=rot, albedo=alb, depol=depol, rows=rows)
    return g


class Server:
    def __init__(self, tables, nslots=2, precision="mixed", hbm_budget_gb=120.0, max_batch_cols=65536,
                 reserve_gb=2.0):
        import torch
        from . import autotune
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
        self.max_batch_cols = int(max_batch_cols)
        # one kernel per stream count for the server's lifetime (the shipped
        # schedule of the 72-layer bucket, else team from 12 streams up), for
        # the mixed series and for the FP64 re-solves, so that results do not
        # depend on the batch a request lands in
        autotune.apply_defaults(torch.cuda.get_device_name(torch.cuda.current_device()))
        self._saved = []  # the library's settings before the server's, put back by close()
        for N in STREAMS:
            for prec in {self.prec, _lib.PREC_FP64}:
                tpb, bps = ctypes.c_int(), ctypes.c_int()
                self.L.aerort_get_schedule(N, prec, ctypes.byref(tpb), ctypes.byref(bps))
                self._saved.append((N, prec, self.L.aerort_get_kernel(N, prec), tpb.value, bps.value))
                ent = autotune._active.get(autotune._key(N, 72, prec))
                if ent is not None:
                    autotune._set(N, prec, ent["kernel"], ent["threads"], ent["blocks_per_sm"])
                else:
                    autotune._set(N, prec, _lib.KERNEL_TEAM if N >= 12 else _lib.KERNEL_THREAD, 32, 0)
        self.slots = [{"streams": [torch.cuda.Stream() for _ in STREAMS], "busy": None} for _ in range(nslots)]
        self.queue = collections.deque()
        self.lock = threading.Lock()
        self.inflight_bytes = 0
        self.done = []
        self.t0 = time.perf_counter()

    def now(self):
        return time.perf_counter() - self.t0

    def close(self):
        from . import autotune
        for s in self.slots:
            for st in s["streams"]:
                st.synchronize()
        self.slots = []
        self.chem.destroy()
        for N, prec, kern, tpb, bps in self._saved:
            autotune._set(N, prec, kern, tpb, bps)

    # ------------------------------------------------------------------ request path
    def submit(self, swath):
        swath.t_arrival = self.now()
        with self.lock:
            self.queue.append(swath)

    def _issue(self, slot, batch):
        """Merge `batch` per stream count over the union of its wavelengths and
        enqueue every group on its own stream of the slot."""
        torch = self.torch
        L = self.L
        chans = sorted({float(c) for sw in batch for c in sw.channels})
        nch = len(chans)
        ch32 = np.array(chans, np.float32)
        keep, outs, events = [], [], []
        for gi, N in enumerate(STREAMS):
            g = merge_group(batch, N, chans)
            if g is None:
                continue
            km, n, rows = g["km"], g["n"], g["rows"]
            stream = slot["streams"][gi]
            with torch.cuda.stream(stream):
                st = stream.cuda_stream

                def dev(a, dt):
                    h = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dt).ravel(order="F"))).pin_memory()
                    d = torch.empty(h.shape, dtype=h.dtype, device="cuda")
                    d.copy_(h, non_blocking=True)
                    keep.append(h)
                    return d
                d_qm, d_rh = dev(g["qm"], np.float32), dev(g["rh"], np.float32)
                d_rot, d_dep, d_he = dev(g["ROT"], np.float64), dev(g["depol"], np.float64), dev(g["he"], np.float64)
                d_alb, d_sza = dev(g["albedo"], np.float64), dev(g["sza"], np.float64)
                d_raa, d_vza, d_nl = dev(g["raa"], np.float64), dev(g["vza"], np.float64), dev(g["nlayers"], np.int32)
                tau = torch.empty(km * nch * n, dtype=torch.float32, device="cuda")
                ssa, gg = torch.empty_like(tau), torch.empty_like(tau)
                pm = torch.empty(km * nch * n * 2 * N, dtype=torch.float32, device="cuda")
                rc = L.aerort_get_aop_vector_dev(self.chem.handle, km, n, nch, 20, _lib.ptr(ch32, _lib.P_f),
                                                 _lib.ptr(self.qt, _lib.P_i), _lib.ptr(self.qb, _lib.P_i),
                                                 d_qm.data_ptr(), d_rh.data_ptr(), 2 * N, 1, tau.data_ptr(),
                                                 ssa.data_ptr(), gg.data_ptr(), pm.data_ptr(), st)
                if rc != 0:
                    raise RuntimeError("aop rc=%d: %s" % (rc, _lib.last_error()))
                rad = torch.empty(n * nch, dtype=torch.float64, device="cuda")
                refl = torch.empty_like(rad)
                nf = torch.empty(n * nch, dtype=torch.int32, device="cuda")
                sts = torch.empty_like(nf)
                fn = (L.aerort_vlidort_scalar_lambert_mixed_batch_dev if self.prec == _lib.PREC_MIXED
                      else L.aerort_vlidort_scalar_lambert_batch_dev)
                rc = fn(km, nch, n, N, 0, 2 * N, d_nl.data_ptr(), d_rot.data_ptr(), d_dep.data_ptr(), None, None,
                        None, tau.data_ptr(), ssa.data_ptr(), pm.data_ptr(), d_he.data_ptr(), d_alb.data_ptr(),
                        d_sza.data_ptr(), d_raa.data_ptr(), d_vza.data_ptr(), MISSING, rad.data_ptr(),
                        refl.data_ptr(), nf.data_ptr(), sts.data_ptr(), st)
                if rc != 0:
                    raise RuntimeError("rt rc=%d: %s" % (rc, _lib.last_error()))
                host = [torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in (rad, refl, nf, sts)]
                for h, t in zip(host, (rad, refl, nf, sts)):
                    h.copy_(t, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(stream)
                events.append(ev)
                keep += [d_qm, d_rh, d_rot, d_dep, d_he, d_alb, d_sza, d_raa, d_vza, d_nl, tau, ssa, gg, pm, rad,
                         refl, nf, sts]
                outs.append((rows, host, n, nch))
        return events, keep, outs

    @staticmethod
    def _finish(batch, outs):
        for sw in batch:
            nch = len(sw.channels)
            sw.radiance = np.zeros((sw.ncol, nch))
            sw.reflectance = np.zeros((sw.ncol, nch))
            sw.nfourier = np.zeros((sw.ncol, nch), np.int32)
            sw.status = np.zeros((sw.ncol, nch), np.int32)
        for rows, (hrad, hrefl, hnf, hst), n, nch in outs:
            arr = [h.numpy().reshape(n, nch, order="F") for h in (hrad, hrefl, hnf, hst)]
            for sw, idx, r, pos in rows:
                sub = np.ix_(r, pos)
                sw.radiance[idx] = arr[0][sub]
                sw.reflectance[idx] = arr[1][sub]
                sw.nfourier[idx] = arr[2][sub]
                sw.status[idx] = arr[3][sub]

    def step(self):
        """Complete finished batches and merge waiting requests into a free
        lane; returns True if anything is pending."""
        torch = self.torch
        for slot in self.slots:
            b = slot["busy"]
            if b is not None and all(e.query() for e in b["events"]):
                self._finish(b["batch"], b["outs"])
                t = self.now()
                for sw in b["batch"]:
                    sw.t_done = t
                    self.done.append(sw)
                self.inflight_bytes -= b["bytes"]
                slot["busy"] = None
        for slot in self.slots:
            if slot["busy"] is not None:
                continue
            free = None
            batch, cols, need = [], 0, 0
            with self.lock:
                while self.queue:
                    sw = self.queue[0]
                    if batch and cols + sw.ncol > self.max_batch_cols:
                        break
                    nch = len({float(c) for x in batch + [sw] for c in x.channels})
                    nb = batch_bytes(batch + [sw], nch)
                    if free is None:
                        free, _ = torch.cuda.mem_get_info()
                    if not can_admit(nb, self.inflight_bytes, self.budget, free, self.reserve):
                        break
                    batch.append(self.queue.popleft())
                    cols += sw.ncol
                    need = nb
            if not batch:
                break
            t = self.now()
            for sw in batch:
                sw.t_admit = t
            events, keep, outs = self._issue(slot, batch)
            self.inflight_bytes += need
            slot["busy"] = {"batch": batch, "events": events, "keep": keep, "outs": outs, "bytes": need}
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

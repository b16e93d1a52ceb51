// aerort: CUDA implementation of the C ABI declared in include/aerort.h.
//
// Kernels
//   k_aop<MC>         Mie-table RH interpolation + species mixing (FP32, one
//                     thread per output (layer, channel, pixel); HBM/L2-gather bound)
//   k_nadir_first     sticky nadir-FO flag of the reference wrapper, as a device atomicMin
//   k_scalar_lambert  FP64 scalar RT, one thread per (pixel, channel) solve,
//                     warp-granular dynamic scheduling over a persistent grid
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "aerort_internal.cuh"

using namespace aerort;
using namespace aerort_internal;

namespace aerort_internal {

thread_local std::string g_last_error;

int set_error(int rc, const std::string& msg) {
  g_last_error = msg;
  return rc;
}

int DevBuf::ensure(size_t n) {
  if (n <= bytes) return 0;
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
  size_t want = n + n / 8;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    p = nullptr;
    return set_error(AERORT_RC_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  bytes = want;
  return 0;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

int Context::setup() {
  if (init) return 0;
  CUDA_TRY(cudaGetDevice(&device));
  CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
  CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  init = true;
  return 0;
}

void Context::release() {
  for (auto& p : pads) {
    p.scratch.release();
    p.counter.release();
    p.redo.release();
    if (p.done) cudaEventDestroy(p.done);
    p = Pad();
  }
  pad = nullptr;
  last_mixed = nullptr;
  for (auto& b : stage) b.release();
  if (stream) cudaStreamDestroy(stream);
  stream = nullptr;
  init = false;
}

Pad* Context::find(cudaStream_t s) {
  for (auto& p : pads)
    if (p.used && p.owner == s) return &p;
  return nullptr;
}

int Context::bind(cudaStream_t s) {
  Pad* p = find(s);
  if (!p) {
    for (auto& q : pads)
      if (!q.used) { p = &q; break; }
    if (!p) {  // all taken: the least recently used one that no captured graph holds
      for (auto& q : pads)
        if (!q.captured && (!p || q.last < p->last)) p = &q;
      if (!p)
        return set_error(AERORT_RC_ARG, "every library scratch pad is held by a stream whose work was captured "
                                        "in a CUDA graph (at most 16 such streams)");
    }
    if (!p->done) CUDA_TRY(cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming));
    if (p->used) CUDA_TRY(cudaStreamWaitEvent(s, p->done, 0));
    p->owner = s;
    p->used = true;
  }
  p->last = ++tick;
  pad = p;
  return 0;
}

// Work enqueued while `s` is being captured into a CUDA graph is replayed
// later, any number of times, on the pad's scratch: such a pad stays with its
// stream for good (never handed to another stream), and no event is recorded
// for it (an event recorded during capture cannot be waited on outside it).
int Context::unbind(cudaStream_t s) {
  if (pad) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CUDA_TRY(cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusNone) CUDA_TRY(cudaEventRecord(pad->done, s));
    else pad->captured = true;
  }
  pad = nullptr;
  return 0;
}

Context& ctx() {
  static Context c;
  return c;
}

static std::atomic<unsigned long long> g_launches{0};
void count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

int stream_index(int nstreams) {
  switch (nstreams) {
    case 4: return 0;
    case 6: return 1;
    case 8: return 2;
    case 12: return 3;
    case 16: return 4;
  }
  return -1;
}

void gauss_legendre01(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p0 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double pm = p0;
        p0 = p1;
        p1 = ((2.0 * j - 1.0) * z * p0 - (j - 1.0) * pm) / j;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double z1 = z;
      z = z1 - p1 / dp;
      if (std::fabs(z - z1) < 1e-15) break;
    }
    x[n - 1 - i] = 0.5 - 0.5 * z;
    w[n - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

}  // namespace aerort_internal


// =========================================================================================
// Mie tables and the aerosol-optics kernel (FP32, bit-identical to the reference)
// =========================================================================================
struct DevMieTable {
  int nrh, nch, nbin, nmom, npol;
  const float *rh, *bext, *bsca, *g, *pmom, *rha;
  const int* rhi;
};

struct aerort_mie {
  int ntables = 0, nch = 0;
  std::vector<float> channels_m;
  std::vector<DevMieTable> host_desc;  // device pointers
  std::vector<void*> allocs;
  DevMieTable* d_tables = nullptr;
};

namespace {
constexpr int kMaxTracers = 64;

__device__ __forceinline__ float lerp_ref(float y0, float y1, float w0, float arh) {
  // TABLE(irh)*(1.-arh) + TABLE(irhp1)*arh, rounded as two products and one sum
  return __fadd_rn(__fmul_rn(y0, w0), __fmul_rn(y1, arh));
}

constexpr int kMaxChannels = 16;

// Per-call lookup metadata passed by value (kernel parameter space), so the
// device entry point needs no host staging.
struct AopMeta {
  int idxch[kMaxChannels];
  int q_table[kMaxTracers];
  int q_bin[kMaxTracers];
};

// One tracer's contribution at one output element: its table, the two RH rows
// b0, b1, the interpolation weights, and tau, ssa of the tracer
// (Chem_MieQueryByInt, Chem_MieMod.F90:860-905, and VLIDORT_MieMod.F90:291-318).
struct TracerRow {
  const DevMieTable* T;
  int b0, b1;
  float arh, w0, tau, ssa;
};

// Fills r for tracer iq; false for a tracer without optics (q_table < 0).
// Recomputed in every pass of k_aop instead of kept in per-thread arrays:
// the same operations in the same order give the same bits each time.
__device__ __forceinline__ bool tracer_row(const DevMieTable* __restrict__ tabs, const AopMeta& meta, int iq,
                                           int ich, int isnap, float qmv, TracerRow& r) {
  const int tb = meta.q_table[iq];
  if (tb < 0) return false;
  const DevMieTable& T = tabs[tb];
  r.T = &T;
  r.arh = T.rha[isnap - 1];
  const int irh = T.rhi[isnap - 1];
  const int irhp1 = irh + 1 > T.nrh ? T.nrh : irh + 1;
  const int row = T.nrh * (ich + T.nch * meta.q_bin[iq]);
  r.b0 = (irh - 1) + row;
  r.b1 = (irhp1 - 1) + row;
  r.w0 = __fsub_rn(1.0f, r.arh);
  const float bext = lerp_ref(T.bext[r.b0], T.bext[r.b1], r.w0, r.arh);
  const float bsca = lerp_ref(T.bsca[r.b0], T.bsca[r.b1], r.w0, r.arh);
  r.tau = __fmul_rn(bext, qmv);
  r.ssa = __fdiv_rn(bsca, bext);
  return true;
}

// VLIDORT_getAOPvector (VLIDORT_MieMod.F90:124-336) with Chem_MieQuery per
// tracer, one thread per output element (layer fastest, so the qm, rh reads
// and every output store are coalesced).  Nothing is kept per tracer: a
// first pass sums tau, ssa, g over the tracers; then, per chunk of MC
// moments and per group of scattering-matrix elements, a pass over the
// tracers accumulates the moments in registers.  Elements that the
// reference couples travel together: for a four-element (spherical) table
// under nPol = 6 the reference sets P22 to the P11 sum and P44 to the P33
// sum after that tracer, so (P11, P22) and (P33, P44) share a pass.
template <int MC>
__global__ void __launch_bounds__(256) k_aop(const DevMieTable* __restrict__ tabs, int km, int nobs, int nch, int nq,
                                             const AopMeta meta, const float* __restrict__ qm,
                                             const float* __restrict__ rh, int nMom, int nPol,
                                             float* __restrict__ tau, float* __restrict__ ssa,
                                             float* __restrict__ g, float* __restrict__ pmom) {
  const long total = (long)km * nch * nobs;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int k = (int)(t % km);
  const long r = t / km;
  const int n = (int)(r % nch);
  const int i = (int)(r / nch);
  const int ich = meta.idxch[n];
  const float rhv = rh[k + (long)km * i];
  // RH snapping (Chem_MieMod.F90:860-867); the max(rh,0) result is discarded there too
  const float rhUse = fminf(rhv, 0.99f);
  int isnap = (int)__fmul_rn(__fadd_rn(rhUse, 0.001f), 1000.0f);
  if (isnap < 1) isnap = 1;
  const float* qcol = qm + k + (long)km * (long)nq * i;
  float ts = 0.0f, ss = 0.0f, gs = 0.0f;
  for (int iq = 0; iq < nq; ++iq) {
    TracerRow q;
    if (!tracer_row(tabs, meta, iq, ich, isnap, qcol[(long)km * iq], q)) continue;
    const float gg = lerp_ref(q.T->g[q.b0], q.T->g[q.b1], q.w0, q.arh);
    ts = __fadd_rn(ts, q.tau);
    ss = __fadd_rn(ss, __fmul_rn(q.ssa, q.tau));
    gs = __fadd_rn(gs, __fmul_rn(__fmul_rn(gg, q.ssa), q.tau));
  }
  // normalisation (VLIDORT_MieMod.F90:320-334)
  const float ssa_out = ts > 0.0f ? __fdiv_rn(ss, ts) : ss;
  const float st = __fmul_rn(ssa_out, ts);
  const float g_out = st > 0.0f ? __fdiv_rn(gs, st) : gs;
  const long o = k + (long)km * (n + (long)nch * i);
  tau[o] = ts;
  ssa[o] = ssa_out;
  g[o] = g_out;
  const long stride = total;
  // element groups: (first, partner or -1); the partner is the element a
  // spherical table copies from `first` under nPol = 6
  const int ngroups = nPol == 6 ? 4 : nPol;
  for (int grp = 0; grp < ngroups; ++grp) {
    const int ea = grp;
    const int eb = nPol == 6 ? (grp == 0 ? 4 : (grp == 2 ? 5 : -1)) : -1;
    for (int m0 = 0; m0 < nMom; m0 += MC) {
      const int mc = nMom - m0 < MC ? nMom - m0 : MC;
      float a[MC], b[MC];
#pragma unroll
      for (int j = 0; j < MC; ++j) { a[j] = 0.0f; b[j] = 0.0f; }
      for (int iq = 0; iq < nq; ++iq) {
        TracerRow q;
        if (!tracer_row(tabs, meta, iq, ich, isnap, qcol[(long)km * iq], q)) continue;
        const DevMieTable& T = *q.T;
        const bool sph = (nPol == 6 && T.npol == 4);
        const long s = (long)T.nrh * T.nch * T.nbin;
        const float* pa = T.pmom + (long)(m0 + T.nmom * ea) * s;
#pragma unroll
        for (int j = 0; j < MC; ++j) {
          if (j < mc) {
            const float p = lerp_ref(pa[(long)j * s + q.b0], pa[(long)j * s + q.b1], q.w0, q.arh);
            a[j] = __fadd_rn(a[j], __fmul_rn(__fmul_rn(p, q.ssa), q.tau));
          }
        }
        if (eb >= 0) {
          if (sph) {
#pragma unroll
            for (int j = 0; j < MC; ++j) b[j] = a[j];
          } else {
            const float* pb = T.pmom + (long)(m0 + T.nmom * eb) * s;
#pragma unroll
            for (int j = 0; j < MC; ++j) {
              if (j < mc) {
                const float p = lerp_ref(pb[(long)j * s + q.b0], pb[(long)j * s + q.b1], q.w0, q.arh);
                b[j] = __fadd_rn(b[j], __fmul_rn(__fmul_rn(p, q.ssa), q.tau));
              }
            }
          }
        }
      }
#pragma unroll
      for (int j = 0; j < MC; ++j) {
        if (j < mc) {
          float v = a[j];
          if (st > 0.0f) v = __fdiv_rn(v, st);
          pmom[o + stride * (m0 + j + (long)nMom * ea)] = v;
          if (eb >= 0) {
            float w = b[j];
            if (st > 0.0f) w = __fdiv_rn(w, st);
            pmom[o + stride * (m0 + j + (long)nMom * eb)] = w;
          }
        }
      }
    }
  }
}

// The same computation with the Mie-table rows staged in shared memory.
// Block (x, n) handles elements e0..e0 + 256*EPT of channel n (e = k + km i,
// layer fastest, so qm, rh reads and output stores stay coalesced).  The
// block first copies, for every tracer, the bext, bsca and g rows of its
// table and size bin at this channel (all RH nodes, row stride R), then for
// each chunk of MC moments of each element group the moment rows; the
// per-element lerps read them from shared memory instead of gathering them
// from L1/L2.  The first chunk's pass over the tracers also sums tau, ssa
// and g (so nMom <= MC needs one pass over the tracers, each tracer's rows
// and weights formed once per element); the later chunks recompute the rows
// and read the element's ssa tau from shared memory.  Operations and their
// order are those of k_aop for every accumulator, so the bits are too.
// Shared memory: nq (3 + P MC) R + 256 EPT floats, P = 2 for nPol = 6
// (paired elements), else 1.
template <int MC, int EPT>
__global__ void __launch_bounds__(256) k_aop_staged(const DevMieTable* __restrict__ tabs, int km, int nobs, int nch,
                                                    int nq, const AopMeta meta, const float* __restrict__ qm,
                                                    const float* __restrict__ rh, int nMom, int nPol, int R,
                                                    float* __restrict__ tau, float* __restrict__ ssa,
                                                    float* __restrict__ g, float* __restrict__ pmom) {
  extern __shared__ float aop_smem[];
  const int n = blockIdx.y;
  const int ich = meta.idxch[n];
  const long nel = (long)km * nobs;
  const long e0 = (long)blockIdx.x * (256L * EPT);
  if (e0 >= nel) return;
  const long e1 = nel < e0 + 256L * EPT ? nel : e0 + 256L * EPT;
  const int P = nPol == 6 ? 2 : 1;
  float* s_sc = aop_smem;                   // [q][3][R]: bext, bsca, g rows
  float* s_st = s_sc + (long)nq * 3 * R;    // [256 EPT]: ssa_out * tau_out of each element
  float* s_mo = s_st + 256L * EPT;          // [q][P][MC][R]: moment rows of the current chunk
  for (int x = threadIdx.x; x < nq * 3 * R; x += blockDim.x) {
    const int r = x % R, qty = (x / R) % 3, q = x / (3 * R);
    const int tb = meta.q_table[q];
    float v = 0.0f;
    if (tb >= 0) {
      const DevMieTable& T = tabs[tb];
      if (r < T.nrh) {
        const long row = r + (long)T.nrh * (ich + (long)T.nch * meta.q_bin[q]);
        v = (qty == 0 ? T.bext : (qty == 1 ? T.bsca : T.g))[row];
      }
    }
    s_sc[x] = v;
  }
  const long total = (long)km * nch * nobs;
  auto snap = [&](int k, int i) {
    const float rhUse = fminf(rh[k + (long)km * i], 0.99f);
    int isnap = (int)__fmul_rn(__fadd_rn(rhUse, 0.001f), 1000.0f);
    return isnap < 1 ? 1 : isnap;
  };
  // a tracer's RH rows (staged indices), weights, tau and ssa at one element
  struct Row { int r0, r1; float arh, w0, tau, ssa; };
  auto row_of = [&](int iq, int isnap, float qmv, Row& w) -> bool {
    const int tb = meta.q_table[iq];
    if (tb < 0) return false;
    const DevMieTable& T = tabs[tb];
    w.arh = T.rha[isnap - 1];
    const int irh = T.rhi[isnap - 1];
    const int irhp1 = irh + 1 > T.nrh ? T.nrh : irh + 1;
    w.r0 = irh - 1;
    w.r1 = irhp1 - 1;
    w.w0 = __fsub_rn(1.0f, w.arh);
    const float* sc = s_sc + (long)iq * 3 * R;
    const float bext = lerp_ref(sc[w.r0], sc[w.r1], w.w0, w.arh);
    const float bsca = lerp_ref(sc[R + w.r0], sc[R + w.r1], w.w0, w.arh);
    w.tau = __fmul_rn(bext, qmv);
    w.ssa = __fdiv_rn(bsca, bext);
    return true;
  };
  // tau, ssa, g of an element from its sums (VLIDORT_MieMod.F90:320-334); returns ssa_out * tau_out
  auto finish = [&](long e, int k, int i, float ts, float ss, float gs) -> float {
    const float ssa_out = ts > 0.0f ? __fdiv_rn(ss, ts) : ss;
    const float st = __fmul_rn(ssa_out, ts);
    const float g_out = st > 0.0f ? __fdiv_rn(gs, st) : gs;
    const long o = k + (long)km * (n + (long)nch * i);
    tau[o] = ts;
    ssa[o] = ssa_out;
    g[o] = g_out;
    s_st[e - e0] = st;
    return st;
  };
  if (nMom <= 0) {  // no moments: the scattering sums alone
    __syncthreads();
    for (long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      const int k = (int)(e % km), i = (int)(e / km);
      const int isnap = snap(k, i);
      const float* qcol = qm + k + (long)km * (long)nq * i;
      float ts = 0.0f, ss = 0.0f, gs = 0.0f;
      for (int iq = 0; iq < nq; ++iq) {
        Row w;
        if (!row_of(iq, isnap, qcol[(long)km * iq], w)) continue;
        const float* sc = s_sc + (long)iq * 3 * R;
        const float gg = lerp_ref(sc[2 * R + w.r0], sc[2 * R + w.r1], w.w0, w.arh);
        ts = __fadd_rn(ts, w.tau);
        ss = __fadd_rn(ss, __fmul_rn(w.ssa, w.tau));
        gs = __fadd_rn(gs, __fmul_rn(__fmul_rn(gg, w.ssa), w.tau));
      }
      finish(e, k, i, ts, ss, gs);
    }
    return;
  }
  const int ngroups = nPol == 6 ? 4 : nPol;
  for (int grp = 0; grp < ngroups; ++grp) {
    const int ea = grp;
    const int eb = nPol == 6 ? (grp == 0 ? 4 : (grp == 2 ? 5 : -1)) : -1;
    for (int m0 = 0; m0 < nMom; m0 += MC) {
      const int mc = nMom - m0 < MC ? nMom - m0 : MC;
      const bool first = grp == 0 && m0 == 0;
      __syncthreads();  // the previous chunk's readers are done (and s_sc is written)
      for (int x = threadIdx.x; x < nq * P * MC * R; x += blockDim.x) {
        const int r = x % R, j = (x / R) % MC, p = (x / (R * MC)) % P, q = x / (R * MC * P);
        const int tb = meta.q_table[q];
        float v = 0.0f;
        const int ip = p == 0 ? ea : eb;
        if (tb >= 0 && j < mc && ip >= 0) {
          const DevMieTable& T = tabs[tb];
          const bool sph = (nPol == 6 && T.npol == 4);
          if (r < T.nrh && !(p == 1 && sph)) {
            const long s = (long)T.nrh * T.nch * T.nbin;
            const long row = r + (long)T.nrh * (ich + (long)T.nch * meta.q_bin[q]);
            v = T.pmom[(long)(m0 + j + T.nmom * ip) * s + row];
          }
        }
        s_mo[x] = v;
      }
      __syncthreads();
      for (long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const int k = (int)(e % km), i = (int)(e / km);
        const int isnap = snap(k, i);
        const float* qcol = qm + k + (long)km * (long)nq * i;
        float a[MC], b[MC];
#pragma unroll
        for (int j = 0; j < MC; ++j) { a[j] = 0.0f; b[j] = 0.0f; }
        float ts = 0.0f, ss = 0.0f, gs = 0.0f;
        for (int iq = 0; iq < nq; ++iq) {
          Row w;
          if (!row_of(iq, isnap, qcol[(long)km * iq], w)) continue;
          if (first) {
            const float* sc = s_sc + (long)iq * 3 * R;
            const float gg = lerp_ref(sc[2 * R + w.r0], sc[2 * R + w.r1], w.w0, w.arh);
            ts = __fadd_rn(ts, w.tau);
            ss = __fadd_rn(ss, __fmul_rn(w.ssa, w.tau));
            gs = __fadd_rn(gs, __fmul_rn(__fmul_rn(gg, w.ssa), w.tau));
          }
          const bool sph = (nPol == 6 && tabs[meta.q_table[iq]].npol == 4);
          const float* pa = s_mo + (long)iq * P * MC * R;
#pragma unroll
          for (int j = 0; j < MC; ++j) {
            if (j < mc) {
              const float pv = lerp_ref(pa[j * R + w.r0], pa[j * R + w.r1], w.w0, w.arh);
              a[j] = __fadd_rn(a[j], __fmul_rn(__fmul_rn(pv, w.ssa), w.tau));
            }
          }
          if (eb >= 0) {
            if (sph) {
#pragma unroll
              for (int j = 0; j < MC; ++j) b[j] = a[j];
            } else {
              const float* pb = pa + MC * R;
#pragma unroll
              for (int j = 0; j < MC; ++j) {
                if (j < mc) {
                  const float pv = lerp_ref(pb[j * R + w.r0], pb[j * R + w.r1], w.w0, w.arh);
                  b[j] = __fadd_rn(b[j], __fmul_rn(__fmul_rn(pv, w.ssa), w.tau));
                }
              }
            }
          }
        }
        const float st = first ? finish(e, k, i, ts, ss, gs) : s_st[e - e0];
        const long o = k + (long)km * (n + (long)nch * i);
#pragma unroll
        for (int j = 0; j < MC; ++j) {
          if (j < mc) {
            float v = a[j];
            if (st > 0.0f) v = __fdiv_rn(v, st);
            pmom[o + total * (m0 + j + (long)nMom * ea)] = v;
            if (eb >= 0) {
              float u = b[j];
              if (st > 0.0f) u = __fdiv_rn(u, st);
              pmom[o + total * (m0 + j + (long)nMom * eb)] = u;
            }
          }
        }
      }
    }
  }
}

// Chem_MieTableMod.F90:612-627 in single precision.
void rh_map(int nrh, const float* rh, int* rhi, float* rha) {
  for (int j = 1; j <= 991; ++j) {
    for (int i = nrh; i >= 1; --i) {
      volatile float x = rh[i - 1] * 1000.0f;
      if ((j - 1) >= (int)x) {
        rhi[j - 1] = i;
        if (i + 1 > nrh) {
          rha[j - 1] = 0.0f;
        } else {
          volatile float num = (float)(j - 1) / 1000.0f;
          volatile float a = num - rh[i - 1];
          volatile float b = rh[i] - rh[i - 1];
          rha[j - 1] = a / b;
        }
        break;
      }
    }
  }
}
}  // namespace

extern "C" int aerort_mie_create(int ntables, const aerort_mie_table_desc* tables, int nch, const float* channels_m,
                                 aerort_mie** out) {
  if (!out || !tables || ntables <= 0 || nch <= 0 || !channels_m) return set_error(AERORT_RC_ARG, "mie_create: bad arguments");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  aerort_mie* m = new aerort_mie();
  m->ntables = ntables;
  m->nch = nch;
  m->channels_m.assign(channels_m, channels_m + nch);
  auto upload = [&](const void* src, size_t bytes, const void** dst) -> int {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 4);
    if (e != cudaSuccess) return set_error(AERORT_RC_CUDA, std::string("mie_create cudaMalloc: ") + cudaGetErrorString(e));
    m->allocs.push_back(p);
    if (bytes) {
      e = cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return set_error(AERORT_RC_CUDA, std::string("mie_create copy: ") + cudaGetErrorString(e));
    }
    *dst = p;
    return 0;
  };
  for (int t = 0; t < ntables; ++t) {
    const aerort_mie_table_desc& d = tables[t];
    if (d.nrh <= 0 || d.nbin <= 0 || d.nmom < 0 || d.npol <= 0 || !d.rh || !d.bext || !d.bsca || !d.g ||
        (d.nmom > 0 && !d.pmom)) {
      aerort_mie_destroy(m);
      return set_error(AERORT_RC_ARG, "mie_create: bad table descriptor");
    }
    DevMieTable T;
    T.nrh = d.nrh; T.nch = nch; T.nbin = d.nbin; T.nmom = d.nmom; T.npol = d.npol;
    size_t n3 = (size_t)d.nrh * nch * d.nbin;
    std::vector<int> rhi(991, 1);
    std::vector<float> rha(991, 0.0f);
    rh_map(d.nrh, d.rh, rhi.data(), rha.data());
    int rc = 0;
    rc |= upload(d.rh, sizeof(float) * d.nrh, (const void**)&T.rh);
    rc |= upload(d.bext, sizeof(float) * n3, (const void**)&T.bext);
    rc |= upload(d.bsca, sizeof(float) * n3, (const void**)&T.bsca);
    rc |= upload(d.g, sizeof(float) * n3, (const void**)&T.g);
    rc |= upload(d.pmom, sizeof(float) * n3 * d.nmom * d.npol, (const void**)&T.pmom);
    rc |= upload(rhi.data(), sizeof(int) * 991, (const void**)&T.rhi);
    rc |= upload(rha.data(), sizeof(float) * 991, (const void**)&T.rha);
    if (rc) { aerort_mie_destroy(m); return AERORT_RC_CUDA; }
    m->host_desc.push_back(T);
  }
  if (upload(m->host_desc.data(), sizeof(DevMieTable) * ntables, (const void**)&m->d_tables)) {
    aerort_mie_destroy(m);
    return AERORT_RC_CUDA;
  }
  *out = m;
  return AERORT_OK;
}

extern "C" int aerort_mie_destroy(aerort_mie* mie) {
  if (!mie) return AERORT_OK;
  for (void* p : mie->allocs) cudaFree(p);
  delete mie;
  return AERORT_OK;
}

namespace {
// Host-side checks of VLIDORT_getAOPvector: channel match (rc 99), moments (666), nPol (777).
int aop_check(const aerort_mie* mie, int nch, int nq, const float* channels_nm, const int* q_table, int nMom,
              int nPol, std::vector<int>& idxch) {
  if (nq > kMaxTracers) return set_error(AERORT_RC_ARG, "get_aop_vector: at most 64 tracers");
  if (nch > kMaxChannels) return set_error(AERORT_RC_ARG, "get_aop_vector: at most 16 channels per call");
  if (nPol < 1 || nPol > 6) return set_error(AERORT_RC_ARG, "get_aop_vector: nPol must be 1..6");
  idxch.assign(nch, -1);
  for (int n = 0; n < nch; ++n) {
    for (int mm = 0; mm < mie->nch; ++mm)
      if (std::fabs(channels_nm[n] - 1.0e9f * mie->channels_m[mm]) < 1.0f) { idxch[n] = mm; break; }
    if (idxch[n] < 0) return set_error(AERORT_RC_CHANNEL, "Mie resource files does not set the required channel");
  }
  for (int iq = 0; iq < nq; ++iq) {
    int t = q_table[iq];
    if (t < 0) continue;
    if (t >= mie->ntables) return set_error(AERORT_RC_ARG, "get_aop_vector: q_table out of range");
    const DevMieTable& T = mie->host_desc[t];
    if (nMom > T.nmom) return set_error(AERORT_RC_MOMENTS, "mieTables do not have enough moments");
    if (!(nPol <= T.npol || (nPol == 6 && T.npol == 4)))
      return set_error(AERORT_RC_NPOL, "inconsistent number of polarizations");
  }
  return 0;
}

int aop_launch(aerort_mie* mie, int km, int nobs, int nch, int nq, const std::vector<int>& idxch,
               const int* q_table, const int* q_bin, const float* qm, const float* rh, int nMom, int nPol,
               float* tau, float* ssa, float* g, float* pmom, cudaStream_t s) {
  AopMeta meta;
  std::memset(&meta, 0, sizeof(meta));
  for (int n = 0; n < nch; ++n) meta.idxch[n] = idxch[n];
  for (int q = 0; q < nq; ++q) { meta.q_table[q] = q_table[q]; meta.q_bin[q] = q_bin[q]; }
  long total = (long)km * nch * nobs;
  if (total == 0) return 0;
  // table rows staged in shared memory when they fit (k_aop_staged), else gathered (k_aop)
  // (16-moment chunks for one element per moment, 8 for the paired elements of nPol = 6)
  constexpr int kEPT = 16;
  constexpr size_t kSmemMax = 96 * 1024;
  int R = 1;
  for (int q = 0; q < nq; ++q)
    if (q_table[q] >= 0 && mie->host_desc[q_table[q]].nrh > R) R = mie->host_desc[q_table[q]].nrh;
  const int P = nPol == 6 ? 2 : 1;
  const int mc = P == 1 ? 16 : 8;
  const size_t smem = sizeof(float) * ((size_t)nq * (3 + P * mc) * R + 256 * kEPT);
  if (nq > 0 && smem <= kSmemMax) {
    static bool attr_set = false;
    if (!attr_set) {
      CUDA_TRY(cudaFuncSetAttribute(k_aop_staged<16, kEPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemMax));
      CUDA_TRY(cudaFuncSetAttribute(k_aop_staged<8, kEPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemMax));
      attr_set = true;
    }
    const long nel = (long)km * nobs;
    const dim3 grid((unsigned)((nel + 256L * kEPT - 1) / (256L * kEPT)), (unsigned)nch);
    if (mc == 16)
      k_aop_staged<16, kEPT><<<grid, 256, smem, s>>>(mie->d_tables, km, nobs, nch, nq, meta, qm, rh, nMom, nPol, R,
                                                     tau, ssa, g, pmom);
    else
      k_aop_staged<8, kEPT><<<grid, 256, smem, s>>>(mie->d_tables, km, nobs, nch, nq, meta, qm, rh, nMom, nPol, R,
                                                    tau, ssa, g, pmom);
  } else {
    const int bs = 256;
    const long nb = (total + bs - 1) / bs;
    k_aop<16><<<(unsigned)nb, bs, 0, s>>>(mie->d_tables, km, nobs, nch, nq, meta, qm, rh, nMom, nPol, tau, ssa, g,
                                          pmom);
  }
  CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return 0;
}
}  // namespace

extern "C" int aerort_get_aop_vector_dev(aerort_mie* mie, int km, int nobs, int nch, int nq,
                                         const float* channels_nm_host, const int* q_table_host,
                                         const int* q_bin_host, const float* qm_dev, const float* rh_dev, int nMom,
                                         int nPol, float* tau_dev, float* ssa_dev, float* g_dev, float* pmom_dev,
                                         void* stream) {
  if (!mie || km <= 0 || nobs < 0 || nch <= 0 || nq < 0) return set_error(AERORT_RC_ARG, "get_aop_vector_dev: bad arguments");
  std::vector<int> idxch;
  if (int rc = aop_check(mie, nch, nq, channels_nm_host, q_table_host, nMom, nPol, idxch)) return rc;
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  return aop_launch(mie, km, nobs, nch, nq, idxch, q_table_host, q_bin_host, qm_dev, rh_dev, nMom, nPol, tau_dev,
                    ssa_dev, g_dev, pmom_dev, (cudaStream_t)stream);
}

extern "C" int aerort_get_aop_vector(aerort_mie* mie, int km, int nobs, int nch, int nq, const float* channels_nm,
                                     const int* q_table, const int* q_bin, const float* qm, const float* rh,
                                     int nMom, int nPol, float* tau, float* ssa, float* g, float* pmom) {
  if (!mie || km <= 0 || nobs < 0 || nch <= 0 || nq < 0 || !channels_nm || !q_table || !q_bin || !qm || !rh || !tau ||
      !ssa || !g || (nMom > 0 && !pmom))
    return set_error(AERORT_RC_ARG, "get_aop_vector: bad arguments");
  std::vector<int> idxch;
  if (int rc = aop_check(mie, nch, nq, channels_nm, q_table, nMom, nPol, idxch)) return rc;
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  cudaStream_t s = c.stream;
  size_t nqm = (size_t)km * nq * nobs, nrh = (size_t)km * nobs, no = (size_t)km * nch * nobs;
  size_t npm = no * nMom * nPol;
  if (int rc = c.stage[0].ensure(4 * (nqm + 1))) return rc;
  if (int rc = c.stage[1].ensure(4 * (nrh + 1))) return rc;
  if (int rc = c.stage[2].ensure(4 * (3 * no + npm + 1))) return rc;
  float* dqm = (float*)c.stage[0].p;
  float* drh = (float*)c.stage[1].p;
  float* dout = (float*)c.stage[2].p;
  CUDA_TRY(cudaMemcpyAsync(dqm, qm, 4 * nqm, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(drh, rh, 4 * nrh, cudaMemcpyHostToDevice, s));
  if (int rc = aop_launch(mie, km, nobs, nch, nq, idxch, q_table, q_bin, dqm, drh, nMom, nPol, dout, dout + no,
                          dout + 2 * no, dout + 3 * no, s))
    return rc;
  CUDA_TRY(cudaMemcpyAsync(tau, dout, 4 * no, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(ssa, dout + no, 4 * no, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(g, dout + 2 * no, 4 * no, cudaMemcpyDeviceToHost, s));
  if (npm) CUDA_TRY(cudaMemcpyAsync(pmom, dout + 3 * no, 4 * npm, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return AERORT_OK;
}

// VLIDORT_getAOPscalar (VLIDORT_MieMod.F90:10-120): the vector routine without
// phase-function moments; with no moments requested neither the 666 nor the
// 777 check can fire, as in the reference, which has neither.
extern "C" int aerort_get_aop_scalar_dev(aerort_mie* mie, int km, int nobs, int nch, int nq,
                                         const float* channels_nm_host, const int* q_table_host,
                                         const int* q_bin_host, const float* qm_dev, const float* rh_dev,
                                         float* tau_dev, float* ssa_dev, float* g_dev, void* stream) {
  return aerort_get_aop_vector_dev(mie, km, nobs, nch, nq, channels_nm_host, q_table_host, q_bin_host, qm_dev, rh_dev,
                                   0, 1, tau_dev, ssa_dev, g_dev, nullptr, stream);
}

extern "C" int aerort_get_aop_scalar(aerort_mie* mie, int km, int nobs, int nch, int nq, const float* channels_nm,
                                     const int* q_table, const int* q_bin, const float* qm, const float* rh,
                                     float* tau, float* ssa, float* g) {
  return aerort_get_aop_vector(mie, km, nobs, nch, nq, channels_nm, q_table, q_bin, qm, rh, 0, 1, tau, ssa, g,
                               nullptr);
}

// =========================================================================================
// Scalar radiative transfer
// =========================================================================================
namespace aerort_internal {
// Sticky nadir-FO flag (VLIDORT_ScatMod.F90:1123-1126 as reached from
// VLIDORT_LAMBERT.F90:106-165): first pixel whose angles are valid, whose
// solar zenith is exactly 0 and that has at least one valid albedo.
__global__ void k_nadir_first(int nobs, int nch, const double* sza, const double* raa, const double* vza,
                              const double* albedo, double missing, int* first) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nobs) return;
  auto miss = [&](double x) { return fabs(x / missing - 1.0) < 0.001; };
  if (miss(sza[j]) || miss(vza[j]) || miss(raa[j]) || sza[j] != 0.0) return;
  for (int i = 0; i < nch; ++i)
    if (!miss(albedo[j + (long)nobs * i])) { atomicMin(first, j); return; }
}
__global__ void k_init_sched(int* counter, int* first, int nobs, int* zero) {
  *counter = 0;
  *first = nobs;
  if (zero) *zero = 0;
}
}  // namespace aerort_internal

namespace {

// AERORT_CONTRACT_* of the FP32 team solve (aerort_set_moment_contraction)
std::atomic<int> g_moment_contraction{AERORT_CONTRACT_FMA};

RtOptions lambert_options(int plane_parallel) {
  RtOptions o;
  o.moment_contraction = g_moment_contraction.load();
  o.do_focorr = 1;            // VLIDORT_Mod.F90: DO_FOCORR / DO_FOCORR_OUTGOING
  o.do_deltam = 1;            // DO_DELTAM_SCALING
  o.do_plane_parallel = plane_parallel ? 1 : 0;
  o.do_double_convtest = 1;   // DO_DOUBLE_CONVTEST
  o.nfine = 3;                // NFINELAYERS
  o.taylor_order = 3;         // TAYLOR_ORDER
  o.accuracy = kAccuracySingle;
  o.earth_radius = 6371.0;
  o.flux_factor = 1.0;
  o.max_fourier = -1;
  return o;
}

template <typename T>
int dispatch_lambert_t(Context& c, int nstreams, const RtOptions& opt, const LambertInputs& in, double* rad,
                       double* refl, int* nf, int* st, cudaStream_t s, const Worklist& wl) {
  const int si = stream_index(nstreams);
  const int prec = sizeof(T) == sizeof(float) ? AERORT_PREC_MIXED : AERORT_PREC_FP64;
  const int rk = si >= 0 ? resolve_kernel(c.sched[prec][si].kernel, prec, si, (long)in.nobs * in.nch, c.num_sms,
                                          wl.in_list != nullptr)
                         : 0;
  if (rk == 1 || rk == 3) {
    const bool terms = rk == 3;
    switch (nstreams) {
      case 4: return launch_scalar_lambert_team<4, T>(c, opt, in, rad, refl, nf, st, s, wl, terms);
      case 6: return launch_scalar_lambert_team<6, T>(c, opt, in, rad, refl, nf, st, s, wl, terms);
      case 8: return launch_scalar_lambert_team<8, T>(c, opt, in, rad, refl, nf, st, s, wl, terms);
      case 12: return launch_scalar_lambert_team<12, T>(c, opt, in, rad, refl, nf, st, s, wl, terms);
      case 16: return launch_scalar_lambert_team<16, T>(c, opt, in, rad, refl, nf, st, s, wl, terms);
    }
  }
  switch (nstreams) {
    case 4: return launch_scalar_lambert<4, T>(c, opt, in, rad, refl, nf, st, s, wl);
    case 6: return launch_scalar_lambert<6, T>(c, opt, in, rad, refl, nf, st, s, wl);
    case 8: return launch_scalar_lambert<8, T>(c, opt, in, rad, refl, nf, st, s, wl);
    case 12: return launch_scalar_lambert<12, T>(c, opt, in, rad, refl, nf, st, s, wl);
    case 16: return launch_scalar_lambert<16, T>(c, opt, in, rad, refl, nf, st, s, wl);
  }
  return set_error(AERORT_RC_UNSUPPORTED, "nstreams must be one of 4, 6, 8, 12, 16");
}

// The mixed method is two launches on one stream: the FP32 series for every
// solve, which lists the solves whose Fourier sum cancels by more than
// kRefineRatio, then the FP64 series for the listed solves only (their outputs
// overwrite the mixed ones).  The list and its count stay on the device.
int dispatch_lambert_on_pad(Context& c, int precision, int nstreams, const RtOptions& opt, const LambertInputs& in,
                            double* rad, double* refl, int* nf, int* st, cudaStream_t s) {
  if (precision == AERORT_PREC_FP64)
    return dispatch_lambert_t<double>(c, nstreams, opt, in, rad, refl, nf, st, s, Worklist());
  if (precision != AERORT_PREC_MIXED)
    return set_error(AERORT_RC_ARG, "precision must be AERORT_PREC_FP64 or AERORT_PREC_MIXED");
  const int nsolve = in.nobs * in.nch;
  Pad& p = *c.pad;
  c.last_mixed = c.pad;
  if (int rc = p.redo.ensure(sizeof(int) * ((size_t)nsolve + 1))) return rc;
  if (int rc = p.counter.ensure(4 * sizeof(int))) return rc;
  int* count = (int*)p.counter.p + 2;
  Worklist wm;
  wm.out_list = (int*)p.redo.p;
  wm.out_count = count;
  wm.ratio = kRefineRatio;
  if (int rc = dispatch_lambert_t<float>(c, nstreams, opt, in, rad, refl, nf, st, s, wm)) return rc;
  Worklist wd;
  wd.in_list = (const int*)p.redo.p;
  wd.in_count = count;
  return dispatch_lambert_t<double>(c, nstreams, opt, in, rad, refl, nf, st, s, wd);
}

int dispatch_lambert(Context& c, int precision, int nstreams, const RtOptions& opt, const LambertInputs& in,
                     double* rad, double* refl, int* nf, int* st, cudaStream_t s) {
  if (int rc = c.bind(s)) return rc;
  const int rc = dispatch_lambert_on_pad(c, precision, nstreams, opt, in, rad, refl, nf, st, s);
  const int rc2 = c.unbind(s);
  return rc ? rc : rc2;
}

}  // namespace

namespace aerort_internal {
// Largest nobs * nch of one RT call.  The persistent kernels hand out solves
// with an int work counter that every resident warp bumps (by up to 32) once
// more after the queue runs dry; the 16 Mi of headroom below INT_MAX covers
// 32 x (resident warps + 1) on any GPU with fewer than 512 Ki resident warps
// (GB300: 152 SMs x 64 warps), so the counter never wraps.
constexpr long long kMaxSolves = 0x7f000000LL;

int lambert_checks(int km, int nch, int nobs, int nstreams, int nMom) {
  if (km <= 0 || nch <= 0 || nobs < 0) return set_error(AERORT_RC_ARG, "scalar_lambert: bad sizes");
  if ((long long)nobs * nch > kMaxSolves)
    return set_error(AERORT_RC_ARG, "scalar_lambert: nobs * nch too large (at most 2130706432 solves per call)");
  if (nstreams > 25) return set_error(AERORT_RC_NSTREAMS, "NSTREAMS > MAXSTREAMS");
  if (km > kMaxLayers) return set_error(AERORT_RC_NLAYERS, "NLAYERS > MAXLAYERS");
  if (nMom > 1000) return set_error(AERORT_RC_NMOMENTS, "nmom > MAXMOMENTS_INPUT");
  if (nMom < 1) return set_error(AERORT_RC_ARG, "scalar_lambert: nMom must be >= 1");
  return 0;
}
}  // namespace aerort_internal

extern "C" int aerort_vlidort_scalar_lambert_dev(int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                                                 const double* ROT, const double* depol, const double* tau,
                                                 const double* ssa, const double* pmom, const double* he,
                                                 const double* albedo, const double* solar_zenith,
                                                 const double* relat_azymuth, const double* sensor_zenith,
                                                 double MISSING, double* radiance_VL, double* reflectance_VL,
                                                 int* nfourier, int* status, void* stream) {
  return aerort_vlidort_scalar_lambert_batch_dev(km, nch, nobs, nstreams, plane_parallel, nMom, nullptr, ROT, depol,
                                                 tau, ssa, pmom, nullptr, nullptr, nullptr, he, albedo, solar_zenith,
                                                 relat_azymuth, sensor_zenith, MISSING, radiance_VL, reflectance_VL,
                                                 nfourier, status, stream);
}

namespace {
int lambert_batch_dev(int precision, int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                      const int* nlay, const double* ROT, const double* depol, const double* tau, const double* ssa,
                      const double* pmom, const float* tau_f, const float* ssa_f, const float* pmom_f,
                      const double* he, const double* albedo, const double* solar_zenith, const double* relat_azymuth,
                      const double* sensor_zenith, double MISSING, double* radiance_VL, double* reflectance_VL,
                      int* nfourier, int* status, void* stream) {
  if (int rc = lambert_checks(km, nch, nobs, nstreams, nMom)) return rc;
  if ((!tau_f && (!tau || !ssa || !pmom)) || (tau_f && (!ssa_f || !pmom_f)))
    return set_error(AERORT_RC_ARG, "scalar_lambert_batch_dev: optics missing");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  LambertInputs in{km, nch, nobs, nMom, ROT, depol, tau, ssa, pmom, he, albedo, solar_zenith, relat_azymuth,
                   sensor_zenith, nlay, tau_f, ssa_f, pmom_f, nullptr, MISSING};
  return dispatch_lambert(c, precision, nstreams, lambert_options(plane_parallel), in, radiance_VL, reflectance_VL,
                          nfourier, status, (cudaStream_t)stream);
}
}  // namespace

extern "C" int aerort_vlidort_scalar_lambert_batch_dev(int km, int nch, int nobs, int nstreams, int plane_parallel,
                                                       int nMom, const int* nlay, const double* ROT,
                                                       const double* depol, const double* tau, const double* ssa,
                                                       const double* pmom, const float* tau_f, const float* ssa_f,
                                                       const float* pmom_f, const double* he, const double* albedo,
                                                       const double* solar_zenith, const double* relat_azymuth,
                                                       const double* sensor_zenith, double MISSING,
                                                       double* radiance_VL, double* reflectance_VL, int* nfourier,
                                                       int* status, void* stream) {
  return lambert_batch_dev(AERORT_PREC_FP64, km, nch, nobs, nstreams, plane_parallel, nMom, nlay, ROT, depol, tau,
                           ssa, pmom, tau_f, ssa_f, pmom_f, he, albedo, solar_zenith, relat_azymuth, sensor_zenith,
                           MISSING, radiance_VL, reflectance_VL, nfourier, status, stream);
}

extern "C" int aerort_vlidort_scalar_lambert_mixed_batch_dev(
    int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom, const int* nlay, const double* ROT,
    const double* depol, const double* tau, const double* ssa, const double* pmom, const float* tau_f,
    const float* ssa_f, const float* pmom_f, const double* he, const double* albedo, const double* solar_zenith,
    const double* relat_azymuth, const double* sensor_zenith, double MISSING, double* radiance_VL,
    double* reflectance_VL, int* nfourier, int* status, void* stream) {
  return lambert_batch_dev(AERORT_PREC_MIXED, km, nch, nobs, nstreams, plane_parallel, nMom, nlay, ROT, depol, tau,
                           ssa, pmom, tau_f, ssa_f, pmom_f, he, albedo, solar_zenith, relat_azymuth, sensor_zenith,
                           MISSING, radiance_VL, reflectance_VL, nfourier, status, stream);
}

extern "C" int aerort_set_schedule(int nstreams, int precision, int threads_per_block, int blocks_per_sm) {
  const int si = stream_index(nstreams);
  if (si < 0) return set_error(AERORT_RC_UNSUPPORTED, "set_schedule: nstreams must be one of 4, 6, 8, 12, 16");
  if (precision != AERORT_PREC_FP64 && precision != AERORT_PREC_MIXED)
    return set_error(AERORT_RC_ARG, "set_schedule: bad precision");
  if (threads_per_block < 32 || threads_per_block > 128 || threads_per_block % 32 != 0 || blocks_per_sm < 0)
    return set_error(AERORT_RC_ARG, "set_schedule: threads_per_block must be 32, 64, 96 or 128, blocks_per_sm >= 0");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  c.sched[precision][si].threads = threads_per_block;
  c.sched[precision][si].blocks_per_sm = blocks_per_sm;
  return AERORT_OK;
}

extern "C" int aerort_refined_count(void* stream, int* count) {
  if (!count) return set_error(AERORT_RC_ARG, "refined_count: null pointer");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  *count = 0;
  Pad* p = stream ? c.find((cudaStream_t)stream) : c.last_mixed;
  if (!p || !p->counter.p || p->counter.bytes < 4 * sizeof(int)) return AERORT_OK;
  CUDA_TRY(cudaMemcpyAsync(count, (int*)p->counter.p + 2, sizeof(int), cudaMemcpyDeviceToHost, p->owner));
  CUDA_TRY(cudaStreamSynchronize(p->owner));
  return AERORT_OK;
}

extern "C" int aerort_set_kernel(int nstreams, int precision, int kernel) {
  const int si = stream_index(nstreams);
  if (si < 0) return set_error(AERORT_RC_UNSUPPORTED, "set_kernel: nstreams must be one of 4, 6, 8, 12, 16");
  if ((precision != AERORT_PREC_FP64 && precision != AERORT_PREC_MIXED) ||
      (kernel != AERORT_KERNEL_THREAD && kernel != AERORT_KERNEL_TEAM && kernel != AERORT_KERNEL_AUTO &&
       kernel != AERORT_KERNEL_TERMS))
    return set_error(AERORT_RC_ARG, "set_kernel: bad precision or kernel");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  c.sched[precision][si].kernel = kernel;
  return AERORT_OK;
}

extern "C" int aerort_set_moment_contraction(int mode) {
  if (mode != AERORT_CONTRACT_FMA && mode != AERORT_CONTRACT_TF32X3)
    return set_error(AERORT_RC_ARG, "set_moment_contraction: mode must be AERORT_CONTRACT_FMA or _TF32X3");
  g_moment_contraction.store(mode);
  return AERORT_OK;
}

extern "C" int aerort_get_moment_contraction(void) { return g_moment_contraction.load(); }

extern "C" int aerort_get_kernel(int nstreams, int precision) {
  const int si = stream_index(nstreams);
  if (si < 0 || (precision != AERORT_PREC_FP64 && precision != AERORT_PREC_MIXED))
    return set_error(AERORT_RC_ARG, "get_kernel: bad argument") * -1;
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  return c.sched[precision][si].kernel;
}

extern "C" int aerort_get_schedule(int nstreams, int precision, int* threads_per_block, int* blocks_per_sm) {
  const int si = stream_index(nstreams);
  if (si < 0 || (precision != AERORT_PREC_FP64 && precision != AERORT_PREC_MIXED) || !threads_per_block ||
      !blocks_per_sm)
    return set_error(AERORT_RC_ARG, "get_schedule: bad argument");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  *threads_per_block = c.sched[precision][si].threads;
  *blocks_per_sm = c.sched[precision][si].blocks_per_sm;
  return AERORT_OK;
}

namespace {
template <typename T>
int dispatch_fixed_t(int nstreams, const RtOptions& opt, const LambertInputs& in, void* arena, size_t bytes, int* sched,
                     int num_sms, const Schedule& sc, double* r, double* f, int* nf, int* st, cudaStream_t s,
                     const Worklist& wl) {
  switch (nstreams) {
    case 4: return launch_scalar_lambert_fixed<4, T>(opt, in, arena, bytes, sched, num_sms, sc, r, f, nf, st, s, wl);
    case 6: return launch_scalar_lambert_fixed<6, T>(opt, in, arena, bytes, sched, num_sms, sc, r, f, nf, st, s, wl);
    case 8: return launch_scalar_lambert_fixed<8, T>(opt, in, arena, bytes, sched, num_sms, sc, r, f, nf, st, s, wl);
    case 12: return launch_scalar_lambert_fixed<12, T>(opt, in, arena, bytes, sched, num_sms, sc, r, f, nf, st, s, wl);
    case 16: return launch_scalar_lambert_fixed<16, T>(opt, in, arena, bytes, sched, num_sms, sc, r, f, nf, st, s, wl);
  }
  return set_error(AERORT_RC_UNSUPPORTED, "nstreams must be one of 4, 6, 8, 12, 16");
}
// On fixed storage the refinement list of the mixed method takes the first
// bytes of the arena (4 per solve) and its count the third scheduling int.
int dispatch_fixed(int precision, int nstreams, const RtOptions& opt, const LambertInputs& in, void* arena,
                   size_t bytes, int* sched, int num_sms, const Schedule& sc, const Schedule& sc64, double* r,
                   double* f, int* nf, int* st, cudaStream_t s) {
  const int si = stream_index(nstreams);
  const long nsolve = (long)in.nobs * in.nch;
  Schedule s32 = sc, s64 = sc64, s64_list = sc64;
  s32.kernel = resolve_kernel(sc.kernel, AERORT_PREC_MIXED, si, nsolve, num_sms, false);
  s64.kernel = resolve_kernel(sc64.kernel, AERORT_PREC_FP64, si, nsolve, num_sms, false);
  s64_list.kernel = resolve_kernel(sc64.kernel, AERORT_PREC_FP64, si, nsolve, num_sms, true);
  if (s64.kernel == 3) s64.kernel = 1;  // fixed storage: the team kernel for the term-parallel choice
  if (precision == AERORT_PREC_FP64)
    return dispatch_fixed_t<double>(nstreams, opt, in, arena, bytes, sched, num_sms, s64, r, f, nf, st, s,
                                    Worklist());
  if (precision != AERORT_PREC_MIXED)
    return set_error(AERORT_RC_ARG, "precision must be AERORT_PREC_FP64 or AERORT_PREC_MIXED");
  const size_t list_bytes = (sizeof(int) * ((size_t)in.nobs * in.nch + 1) + 255) / 256 * 256;
  if (bytes <= list_bytes) return set_error(AERORT_RC_ARG, "workspace too small for the refinement list");
  Worklist wm;
  wm.out_list = (int*)arena;
  wm.out_count = sched + 2;
  wm.ratio = kRefineRatio;
  void* rest = (char*)arena + list_bytes;
  if (int rc = dispatch_fixed_t<float>(nstreams, opt, in, rest, bytes - list_bytes, sched, num_sms, s32, r, f, nf,
                                       st, s, wm))
    return rc;
  Worklist wd;
  wd.in_list = (const int*)arena;
  wd.in_count = sched + 2;
  return dispatch_fixed_t<double>(nstreams, opt, in, rest, bytes - list_bytes, sched, num_sms, s64_list, r, f, nf, st,
                                  s, wd);
}
}  // namespace

// Caller-owned RT workspace: device scratch plus the two scheduling ints of
// one launch at a time.  Launches on different workspaces may run
// concurrently on different streams.
struct aerort_workspace {
  int device = -1, num_sms = 0;
  void* arena = nullptr;
  size_t bytes = 0;
  int* sched = nullptr;
};

extern "C" int aerort_workspace_create(size_t bytes, aerort_workspace** out) {
  if (!out || bytes < 4096) return set_error(AERORT_RC_ARG, "workspace_create: bytes must be >= 4096");
  *out = nullptr;
  auto* ws = new aerort_workspace;
  cudaError_t e = cudaGetDevice(&ws->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ws->num_sms, cudaDevAttrMultiProcessorCount, ws->device);
  if (e == cudaSuccess) e = cudaMalloc(&ws->arena, bytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&ws->sched, 256);
  if (e != cudaSuccess) {
    if (ws->arena) cudaFree(ws->arena);
    delete ws;
    return set_error(AERORT_RC_CUDA, std::string("workspace_create: ") + cudaGetErrorString(e));
  }
  ws->bytes = bytes;
  *out = ws;
  return AERORT_OK;
}

extern "C" int aerort_workspace_destroy(aerort_workspace* ws) {
  if (!ws) return AERORT_OK;
  cudaFree(ws->arena);
  cudaFree(ws->sched);
  delete ws;
  return AERORT_OK;
}

extern "C" long aerort_workspace_bytes_per_thread(int km, int nstreams, int precision) {
  const bool f = (precision == AERORT_PREC_MIXED);
  switch (nstreams) {
    case 4: return f ? ScratchLayout<4>(km).bytes<float>() : ScratchLayout<4>(km).bytes<double>();
    case 6: return f ? ScratchLayout<6>(km).bytes<float>() : ScratchLayout<6>(km).bytes<double>();
    case 8: return f ? ScratchLayout<8>(km).bytes<float>() : ScratchLayout<8>(km).bytes<double>();
    case 12: return f ? ScratchLayout<12>(km).bytes<float>() : ScratchLayout<12>(km).bytes<double>();
    case 16: return f ? ScratchLayout<16>(km).bytes<float>() : ScratchLayout<16>(km).bytes<double>();
  }
  return -1;
}

extern "C" int aerort_vlidort_scalar_lambert_ws_dev(
    aerort_workspace* ws, int precision, int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
    const int* nlay, const double* ROT, const double* depol, const double* tau, const double* ssa,
    const double* pmom, const float* tau_f, const float* ssa_f, const float* pmom_f, const double* he,
    const double* albedo, const double* solar_zenith, const double* relat_azymuth, const double* sensor_zenith,
    double MISSING, double* radiance_VL, double* reflectance_VL, int* nfourier, int* status, void* stream) {
  if (!ws) return set_error(AERORT_RC_ARG, "scalar_lambert_ws_dev: null workspace");
  if (int rc = lambert_checks(km, nch, nobs, nstreams, nMom)) return rc;
  if ((!tau_f && (!tau || !ssa || !pmom)) || (tau_f && (!ssa_f || !pmom_f)))
    return set_error(AERORT_RC_ARG, "scalar_lambert_ws_dev: optics missing");
  Schedule sc, sc64;
  {
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    const int si = stream_index(nstreams);
    if (si >= 0 && (precision == AERORT_PREC_FP64 || precision == AERORT_PREC_MIXED)) {
      sc = c.sched[precision][si];
      sc64 = c.sched[AERORT_PREC_FP64][si];
    }
  }
  LambertInputs in{km, nch, nobs, nMom, ROT, depol, tau, ssa, pmom, he, albedo, solar_zenith, relat_azymuth,
                   sensor_zenith, nlay, tau_f, ssa_f, pmom_f, nullptr, MISSING};
  return dispatch_fixed(precision, nstreams, lambert_options(plane_parallel), in, ws->arena, ws->bytes, ws->sched,
                        ws->num_sms, sc, sc64, radiance_VL, reflectance_VL, nfourier, status, (cudaStream_t)stream);
}

extern "C" int aerort_vlidort_scalar_lambert_batch_dev_noalloc(
    int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom, const int* nlay, const double* ROT,
    const double* depol, const double* tau, const double* ssa, const double* pmom, const float* tau_f,
    const float* ssa_f, const float* pmom_f, const double* he, const double* albedo, const double* solar_zenith,
    const double* relat_azymuth, const double* sensor_zenith, double MISSING, double* radiance_VL,
    double* reflectance_VL, int* nfourier, int* status, void* stream) {
  if (int rc = lambert_checks(km, nch, nobs, nstreams, nMom)) return rc;
  if ((!tau_f && (!tau || !ssa || !pmom)) || (tau_f && (!ssa_f || !pmom_f)))
    return set_error(AERORT_RC_ARG, "scalar_lambert_noalloc: optics missing");
  double* arena = nullptr;
  size_t arena_doubles = 0;
  int* sched = nullptr;
  int num_sms = 0;
  if (int rc = static_arena(&arena, &arena_doubles, &sched, &num_sms)) return rc;
  LambertInputs in{km, nch, nobs, nMom, ROT, depol, tau, ssa, pmom, he, albedo, solar_zenith, relat_azymuth,
                   sensor_zenith, nlay, tau_f, ssa_f, pmom_f, nullptr, MISSING};
  Schedule sc;  // the library's kernel choice for this stream count; 32-thread blocks (thread kernel) or
                // two-warp blocks (team kernel), occupancy-limited
  {
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    const int si = stream_index(nstreams);
    if (si >= 0) sc.kernel = c.sched[AERORT_PREC_FP64][si].kernel;
  }
  return dispatch_fixed(AERORT_PREC_FP64, nstreams, lambert_options(plane_parallel), in, arena,
                        arena_doubles * sizeof(double), sched, num_sms, sc, sc, radiance_VL, reflectance_VL, nfourier,
                        status, (cudaStream_t)stream);
}

extern "C" int aerort_vlidort_scalar_lambert_ex(int km, int nch, int nobs, const double* channels, int nstreams,
                                                int plane_parallel, int nMom, int nPol, const double* ROT,
                                                const double* depol, const double* tau, const double* ssa,
                                                const double* g, const double* pmom, const double* pe,
                                                const double* he, const double* te, const double* albedo,
                                                const double* solar_zenith, const double* relat_azymuth,
                                                const double* sensor_zenith, double MISSING, int verbose,
                                                double* radiance_VL, double* reflectance_VL, int* nfourier,
                                                int* status) {
  (void)channels; (void)nPol; (void)g; (void)pe; (void)te; (void)verbose;
  if (int rc = lambert_checks(km, nch, nobs, nstreams, nMom)) return rc;
  if (!ROT || !depol || !tau || !ssa || !pmom || !he || !albedo || !solar_zenith || !relat_azymuth ||
      !sensor_zenith || !radiance_VL || !reflectance_VL)
    return set_error(AERORT_RC_ARG, "scalar_lambert: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  cudaStream_t s = c.stream;
  const size_t nl = (size_t)km * nobs * nch, np = nl * nMom, nh = (size_t)(km + 1) * nobs, nx = (size_t)nobs * nch;
  // staging (the P11 moments are the first nMom*km*nch*nobs doubles of pmom)
  struct { const void* src; size_t bytes; } ins[] = {
      {ROT, 8 * nl}, {depol, 8 * (size_t)nch}, {tau, 8 * nl}, {ssa, 8 * nl}, {pmom, 8 * np}, {he, 8 * nh},
      {albedo, 8 * nx}, {solar_zenith, 8 * (size_t)nobs}, {relat_azymuth, 8 * (size_t)nobs},
      {sensor_zenith, 8 * (size_t)nobs}};
  const double* d[10];
  for (int k = 0; k < 10; ++k) {
    if (int rc = c.stage[k].ensure(ins[k].bytes + 8)) return rc;
    CUDA_TRY(cudaMemcpyAsync(c.stage[k].p, ins[k].src, ins[k].bytes, cudaMemcpyHostToDevice, s));
    d[k] = (const double*)c.stage[k].p;
  }
  if (int rc = c.stage[10].ensure(16 * nx + 8 * nx + 8)) return rc;
  double* drad = (double*)c.stage[10].p;
  double* drefl = drad + nx;
  int* dnf = (int*)(drefl + nx);
  int* dst = dnf + nx;
  LambertInputs in{km, nch, nobs, nMom, d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8], d[9],
                   nullptr, nullptr, nullptr, nullptr, nullptr, MISSING};
  if (int rc = dispatch_lambert(c, AERORT_PREC_FP64, nstreams, lambert_options(plane_parallel), in, drad, drefl, dnf, dst, s))
    return rc;
  CUDA_TRY(cudaMemcpyAsync(radiance_VL, drad, 8 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(reflectance_VL, drefl, 8 * nx, cudaMemcpyDeviceToHost, s));
  if (nfourier) CUDA_TRY(cudaMemcpyAsync(nfourier, dnf, 4 * nx, cudaMemcpyDeviceToHost, s));
  if (status) CUDA_TRY(cudaMemcpyAsync(status, dst, 4 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return AERORT_OK;
}

namespace {
int lambert_batch_host(int precision, int km, int nch, int nobs, int nstreams, int plane_parallel, int nMom,
                       const int* nlay, const double* ROT, const double* depol, const double* tau, const double* ssa,
                       const double* pmom, const double* he, const double* albedo, const double* solar_zenith,
                       const double* relat_azymuth, const double* sensor_zenith, double MISSING, double* radiance_VL,
                       double* reflectance_VL, int* nfourier, int* status) {
  if (int rc = lambert_checks(km, nch, nobs, nstreams, nMom)) return rc;
  if (!ROT || !depol || !tau || !ssa || !pmom || !he || !albedo || !solar_zenith || !relat_azymuth ||
      !sensor_zenith || !radiance_VL || !reflectance_VL)
    return set_error(AERORT_RC_ARG, "scalar_lambert_batch: null array");
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  if (int rc = c.setup()) return rc;
  cudaStream_t s = c.stream;
  const size_t nl = (size_t)km * nobs * nch, np = nl * nMom, nh = (size_t)(km + 1) * nobs, nx = (size_t)nobs * nch;
  struct { const void* src; size_t bytes; } ins[] = {
      {ROT, 8 * nl}, {depol, 8 * (size_t)nch}, {tau, 8 * nl}, {ssa, 8 * nl}, {pmom, 8 * np}, {he, 8 * nh},
      {albedo, 8 * nx}, {solar_zenith, 8 * (size_t)nobs}, {relat_azymuth, 8 * (size_t)nobs},
      {sensor_zenith, 8 * (size_t)nobs}, {nlay, nlay ? 4 * (size_t)nobs : 0}};
  const void* d[11];
  for (int k = 0; k < 11; ++k) {
    d[k] = nullptr;
    if (!ins[k].src) continue;
    if (int rc = c.stage[k].ensure(ins[k].bytes + 8)) return rc;
    CUDA_TRY(cudaMemcpyAsync(c.stage[k].p, ins[k].src, ins[k].bytes, cudaMemcpyHostToDevice, s));
    d[k] = c.stage[k].p;
  }
  if (int rc = c.stage[11].ensure(16 * nx + 8 * nx + 8)) return rc;
  double* drad = (double*)c.stage[11].p;
  double* drefl = drad + nx;
  int* dnf = (int*)(drefl + nx);
  int* dst = dnf + nx;
  LambertInputs in{km, nch, nobs, nMom, (const double*)d[0], (const double*)d[1], (const double*)d[2],
                   (const double*)d[3], (const double*)d[4], (const double*)d[5], (const double*)d[6],
                   (const double*)d[7], (const double*)d[8], (const double*)d[9], (const int*)d[10], nullptr, nullptr,
                   nullptr, nullptr, MISSING};
  if (int rc = dispatch_lambert(c, precision, nstreams, lambert_options(plane_parallel), in, drad, drefl, dnf, dst, s))
    return rc;
  CUDA_TRY(cudaMemcpyAsync(radiance_VL, drad, 8 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(reflectance_VL, drefl, 8 * nx, cudaMemcpyDeviceToHost, s));
  if (nfourier) CUDA_TRY(cudaMemcpyAsync(nfourier, dnf, 4 * nx, cudaMemcpyDeviceToHost, s));
  if (status) CUDA_TRY(cudaMemcpyAsync(status, dst, 4 * nx, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return AERORT_OK;
}
}  // namespace

extern "C" int aerort_vlidort_scalar_lambert_batch(int km, int nch, int nobs, int nstreams, int plane_parallel,
                                                   int nMom, const int* nlay, const double* ROT, const double* depol,
                                                   const double* tau, const double* ssa, const double* pmom,
                                                   const double* he, const double* albedo, const double* solar_zenith,
                                                   const double* relat_azymuth, const double* sensor_zenith,
                                                   double MISSING, double* radiance_VL, double* reflectance_VL,
                                                   int* nfourier, int* status) {
  return lambert_batch_host(AERORT_PREC_FP64, km, nch, nobs, nstreams, plane_parallel, nMom, nlay, ROT, depol, tau,
                            ssa, pmom, he, albedo, solar_zenith, relat_azymuth, sensor_zenith, MISSING, radiance_VL,
                            reflectance_VL, nfourier, status);
}

extern "C" int aerort_vlidort_scalar_lambert_mixed_batch(int km, int nch, int nobs, int nstreams, int plane_parallel,
                                                         int nMom, const int* nlay, const double* ROT,
                                                         const double* depol, const double* tau, const double* ssa,
                                                         const double* pmom, const double* he, const double* albedo,
                                                         const double* solar_zenith, const double* relat_azymuth,
                                                         const double* sensor_zenith, double MISSING,
                                                         double* radiance_VL, double* reflectance_VL, int* nfourier,
                                                         int* status) {
  return lambert_batch_host(AERORT_PREC_MIXED, km, nch, nobs, nstreams, plane_parallel, nMom, nlay, ROT, depol, tau,
                            ssa, pmom, he, albedo, solar_zenith, relat_azymuth, sensor_zenith, MISSING, radiance_VL,
                            reflectance_VL, nfourier, status);
}


extern "C" int aerort_vlidort_scalar_lambert(int km, int nch, int nobs, const double* channels, int nstreams,
                                             int plane_parallel, int nMom, int nPol, const double* ROT,
                                             const double* depol, const double* tau, const double* ssa,
                                             const double* g, const double* pmom, const double* pe, const double* he,
                                             const double* te, const double* albedo, const double* solar_zenith,
                                             const double* relat_azymuth, const double* sensor_zenith,
                                             double MISSING, int verbose, double* radiance_VL,
                                             double* reflectance_VL) {
  return aerort_vlidort_scalar_lambert_ex(km, nch, nobs, channels, nstreams, plane_parallel, nMom, nPol, ROT, depol,
                                          tau, ssa, g, pmom, pe, he, te, albedo, solar_zenith, relat_azymuth,
                                          sensor_zenith, MISSING, verbose, radiance_VL, reflectance_VL, nullptr,
                                          nullptr);
}

extern "C" const char* aerort_last_error(void) { return g_last_error.c_str(); }
extern "C" int aerort_version(void) { return 10; }
extern "C" int aerort_release(void) {
  Context& c = ctx();
  std::lock_guard<std::mutex> lk(c.mu);
  c.release();
  static_arena_forget();
  return AERORT_OK;
}

// ----------------------------------------------------------------------------------------------
// FP64 issue-rate probe: 8 independent FMA chains per thread, `iters` rounds.
// Used by bench.py to measure the FP64 pipe peak that bounds the RT kernel.
namespace {
__global__ void k_dfma_probe(int iters, double* out) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double b = 0.999999999, c = 1e-12;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  double r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == 1234.5) out[0] = r;  // keeps the chains live
}
__global__ void k_ffma_probe(int iters, float* out) {
  float a0 = threadIdx.x * 1e-9f, a1 = a0 + 1e-9f, a2 = a0 + 2e-9f, a3 = a0 + 3e-9f;
  float a4 = a0 + 4e-9f, a5 = a0 + 5e-9f, a6 = a0 + 6e-9f, a7 = a0 + 7e-9f;
  const float b = 0.9999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
    a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
    a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
  }
  float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == 1234.5f) out[0] = r;
}
}  // namespace

extern "C" int aerort_probe_ffma(int blocks, int threads, int iters, float* out_dev, void* stream) {
  if (blocks <= 0 || threads <= 0 || iters <= 0 || !out_dev) return set_error(AERORT_RC_ARG, "probe_ffma: bad arguments");
  k_ffma_probe<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, out_dev);
  CUDA_TRY(cudaGetLastError());
  return AERORT_OK;
}

extern "C" int aerort_probe_dfma(int blocks, int threads, int iters, double* out_dev, void* stream) {
  if (blocks <= 0 || threads <= 0 || iters <= 0 || !out_dev) return set_error(AERORT_RC_ARG, "probe_dfma: bad arguments");
  k_dfma_probe<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, out_dev);
  CUDA_TRY(cudaGetLastError());
  return AERORT_OK;
}


extern "C" unsigned long long aerort_launch_count(void) {
  return aerort_internal::g_launches.load(std::memory_order_relaxed);
}

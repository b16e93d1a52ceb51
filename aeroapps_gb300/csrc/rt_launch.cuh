// Scalar RT kernel and launcher, instantiated once per stream count in
// rt_ns{4,6,8,12,16}.cu so the instantiations compile in parallel.
#pragma once
#include "aerort_internal.cuh"
#include "rt_team.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace aerort_internal {
using namespace aerort;

// Sticky nadir-FO flag (VLIDORT_ScatMod.F90:1123-1126 as reached from
// VLIDORT_LAMBERT.F90:106-165): first pixel whose angles are valid, whose
// solar zenith is exactly 0 and that has at least one valid albedo.
__global__ void k_nadir_first(int nobs, int nch, const double* sza, const double* raa, const double* vza,
                              const double* albedo, double missing, int* first);
// counter <- 0, first <- nobs, *zero <- 0 when given (device-side, so launches
// need no host staging)
__global__ void k_init_sched(int* counter, int* first, int nobs, int* zero);

template <int NS, typename T>
__global__ void __launch_bounds__(128) k_scalar_lambert(RtOptions opt, LambertInputs in, Quad q, void* scratch,
                                                        long nthreads, int nsolve, int* counter, double* rad,
                                                        double* refl, int* nf, int* st, Worklist wl) {
  const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const SolveScratch<T> S = make_scratch<NS, T>(scratch, tid, nthreads, in.km);
  const int lane = threadIdx.x & 31;
  const int n = wl.count(nsolve);
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(counter, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const int s = base + lane;
    if (s < n) solve_lambert<NS, T>(opt, in, wl.solve(s), q.qx, q.qw, q.tu, q.wu, S, rad, refl, nf, st, wl);
    __syncwarp();
  }
}

// Largest solves per warp grab for the team kernel and the grid: enough warps
// for the batch, at most the resident ones (resident_blocks x wpb warps), and
// at most 32 solves per grab (one set-up lane per solve).  The kernel's grabs
// shrink from there as the queue drains (guided self-scheduling, kGrabShare).
inline int team_chunk(int nsolve, long resident_blocks, int wpb, long* nblocks) {
  const long resident_warps = resident_blocks * wpb;
  long chunk = (nsolve + resident_warps - 1) / resident_warps;
  if (chunk < 1) chunk = 1;
  if (chunk > 32) chunk = 32;
  const long warps = (nsolve + chunk - 1) / chunk;
  long need = (warps + wpb - 1) / wpb;
  if (need > resident_blocks) need = resident_blocks;
  if (need < 1) need = 1;
  *nblocks = need;
  return (int)chunk;
}

// Team kernel: each warp takes c (1..chunk) solves, runs their set-up thread
// per solve (lanes 0..c-1), then runs their Fourier series one after another as
// a team (rt_team.cuh).  c is 1/kGrabShare of the remaining solves' fair share
// per warp: large grabs early keep the set-up lanes busy, single solves at the
// end keep every warp busy to the last solve (solves differ 20x in cost: 20-72
// layers, 2-32 Fourier terms).  Measured on GB300 at ~13,000 solves per
// launch: 1.5-1.9x faster than one fixed grab per warp.  WPB warps per block,
// one TeamMem per warp in dynamic shared memory.
constexpr int kGrabShare = 4;
template <int NS, typename T, int WPB>
// FP32: a register cap so that the resident warps are limited by the
// shared-memory working set rather than by registers: 8 two-warp blocks (16
// warps, <= 128 registers) up to 8 streams, 6 blocks (12 warps, <= 170
// registers) above, where 128 registers would spill (measured on GB300).
__global__ void __launch_bounds__(32 * WPB, sizeof(T) == sizeof(float) ? (NS <= 8 ? 8 : 6) : 1) k_scalar_lambert_team(RtOptions opt, LambertInputs in, Quad q,
                                                                   void* scratch, long nthreads, int nsolve, int chunk,
                                                                   int* counter, double* rad, double* refl, int* nf,
                                                                   int* st, Worklist wl) {
  extern __shared__ __align__(16) unsigned char team_smem[];
  const int lane = threadIdx.x & 31;
  TeamMem<NS, T>& M = reinterpret_cast<TeamMem<NS, T>*>(team_smem)[threadIdx.x >> 5];
  const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long tid0 = tid - lane;
  const ScratchLayout<NS> lay(in.km, false);
  const SolveScratch<T> S = make_scratch<NS, T>(scratch, tid, nthreads, in.km, false);
  const Team tm{lane, nullptr, nullptr};
  const int n = wl.count(nsolve);
  const int share = (int)(gridDim.x * (blockDim.x >> 5)) * kGrabShare;
  for (;;) {
    int base = 0, c = 1;
    if (lane == 0) {
      if (chunk > 1) {
        const int rem = n - *(volatile int*)counter;
        c = (rem + share - 1) / share;
        c = c < 1 ? 1 : (c > chunk ? chunk : c);
      }
      base = atomicAdd(counter, c);
    }
    base = __shfl_sync(0xffffffffu, base, 0);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (base >= n) break;
    const int s = base + lane;
    bool live = false;
    int sidx = 0;
    if (lane < c && s < n) {
      sidx = wl.solve(s);
      SetupRecord r;
      live = solve_setup<NS, T>(opt, in, sidx, q.tu, q.wu, S, rad, refl, nf, st, r);
      if (live) r.store(S.D, lay.rec);
    }
    unsigned mask = __ballot_sync(0xffffffffu, live);
    __syncwarp();
    while (mask) {
      const int b = __ffs(mask) - 1;
      mask &= mask - 1;
      const SolveScratch<T> Sb = make_scratch<NS, T>(scratch, tid0 + b, nthreads, in.km, false);
      SetupRecord rb;
      rb.load(Sb.D, lay.rec);
      const int sb = __shfl_sync(0xffffffffu, sidx, b);
      team_fourier_series<NS, T>(tm, M, opt, in, rb, q.qx, q.qw, Sb.W, lay, rad, refl, nf, st, wl, sb);
    }
  }
}

// Two-pass team solve (library scratch, whole batches): k_team_setup runs the
// set-up of every solve of a slice, one thread per solve and all lanes busy;
// k_team_series then runs the Fourier series, each warp taking one solve at a
// time in index order.  Against the fused kernel this removes the set-up from
// the team kernel (one or two busy lanes per grab there) and its code from
// the team kernel's instruction footprint.  Per-solve scratch (set-up record
// and layer arrays, element-major / solve-minor) for at most kSetupSlice
// solves at once.
constexpr int kSetupSlice = 1 << 17;

template <int NS, typename T>
__global__ void __launch_bounds__(32) k_team_setup(RtOptions opt, LambertInputs in, Quad q, void* scratch, int base,
                                                   int count, double* rad, double* refl, int* nf, int* st,
                                                   unsigned char* live) {
  const ScratchLayout<NS> lay(in.km, false);
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x) {
    const SolveScratch<T> S = make_scratch<NS, T>(scratch, s, count, in.km, false);
    SetupRecord r;
    const bool ok = solve_setup<NS, T>(opt, in, base + s, q.tu, q.wu, S, rad, refl, nf, st, r);
    if (ok) r.store(S.D, lay.rec);
    live[s] = ok ? 1 : 0;
  }
}

// FP32 register caps as for the fused kernel; without the set-up code the
// 12-stream series kernel also fits 128 registers (16 warps per SM, no spills).
template <int NS, typename T, int WPB>
__global__ void __launch_bounds__(32 * WPB, sizeof(T) == sizeof(float) ? (NS <= 12 ? 8 : 6) : 1)
    k_team_series(RtOptions opt, LambertInputs in, Quad q, void* scratch, int base, int count, int* counter,
                  const unsigned char* live, double* rad, double* refl, int* nf, int* st, Worklist wl) {
  extern __shared__ __align__(16) unsigned char team_smem[];
  const int lane = threadIdx.x & 31;
  TeamMem<NS, T>& M = reinterpret_cast<TeamMem<NS, T>*>(team_smem)[threadIdx.x >> 5];
  const ScratchLayout<NS> lay(in.km, false);
  const Team tm{lane, nullptr, nullptr};
  for (;;) {
    int s = 0;
    if (lane == 0) s = atomicAdd(counter, 1);
    s = __shfl_sync(0xffffffffu, s, 0);
    if (s >= count) break;
    if (!live[s]) continue;
    const SolveScratch<T> S = make_scratch<NS, T>(scratch, s, count, in.km, false);
    SetupRecord r;
    r.load(S.D, lay.rec);
    team_fourier_series<NS, T>(tm, M, opt, in, r, q.qx, q.qw, S.W, lay, rad, refl, nf, st, wl, base + s);
  }
}

// Term-parallel FP64 team solve: each solve's Fourier terms spread over the W
// warps of a block.  Warp w runs terms m0 + w of each round, one thread adds
// the round's terms to the Fourier sum in order with the convergence test,
// and the round that ends the series ends the solve (its later terms are
// discarded).  Every term is the one team_fourier_series would compute
// (team_skip_terms carries P~_m^m over the terms a warp skips), so the
// results are the sequential series'.  A solve's latency drops from the whole
// series on one warp to about a W-th of it, at the cost of up to W - 1
// discarded terms: the form for few solves -- a mixed launch's refinement
// list (wl.in_list), or a batch too small to fill the GPU one warp per solve
// (AERORT_KERNEL_TERMS).  One solve per block at a time; the block's set-up
// thread fills its scratch.
template <int NS, int W>
__global__ void __launch_bounds__(32 * W, 1)
    k_refine_terms(RtOptions opt, LambertInputs in, Quad q, void* scratch, int nsolve, int* counter, double* rad,
                   double* refl, int* nf, int* st, Worklist wl) {
  extern __shared__ __align__(16) unsigned char team_smem[];
  __shared__ double s_sf[W];
  __shared__ int s_tst[W];
  __shared__ int s_idx, s_live, s_stop, s_m, s_st;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  TeamMem<NS, double>& M = reinterpret_cast<TeamMem<NS, double>*>(team_smem)[w];
  const ScratchLayout<NS> lay(in.km, false);
  const SolveScratch<double> S = make_scratch<NS, double>(scratch, blockIdx.x, gridDim.x, in.km, false);
  const Team tm{lane, nullptr, nullptr};
  const int n = wl.count(nsolve);
  for (;;) {
    if (threadIdx.x == 0) s_idx = atomicAdd(counter, 1);
    __syncthreads();
    const int idx = s_idx;
    if (idx >= n) break;
    const int sidx = wl.solve(idx);
    if (threadIdx.x == 0) {
      SetupRecord r;
      const bool ok = solve_setup<NS, double>(opt, in, sidx, q.tu, q.wu, S, rad, refl, nf, st, r);
      if (ok) r.store(S.D, lay.rec);
      s_live = ok ? 1 : 0;
    }
    __syncthreads();
    if (s_live) {
      SetupRecord r;
      r.load(S.D, lay.rec);
      SolveCtx<NS, double> c;
      team_series_init<NS, double>(tm, M, r, q.qx, q.qw, c);
      FourierSum sum;  // thread 0's
      int last = -1;
      for (int m0 = 0;; m0 += W) {
        const int m = m0 + w;
        int tst = RT_OK;
        double sf = 0.0;
        if (m <= r.n_fouriers) {
          team_skip_terms<NS, double>(tm, M, c, last, m);
          tst = team_fourier_term<NS, double>(tm, M, c, opt, m, S.W, lay, &sf);
          last = m;
        }
        if (lane == 0) {
          s_sf[w] = sf;
          s_tst[w] = tst;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          int stop = 0;
          for (int k = 0; k < W && !stop; ++k) {
            const int mk = m0 + k;
            if (mk > r.n_fouriers) { stop = 1; s_m = mk; s_st = RT_OK; }
            else if (s_tst[k] != RT_OK) { stop = 1; s_m = mk; s_st = s_tst[k]; }
            else if (sum.add(opt, r, mk, s_sf[k])) { stop = 1; s_m = mk; s_st = RT_OK; }
          }
          s_stop = stop;
        }
        __syncthreads();
        if (s_stop) break;
      }
      if (threadIdx.x == 0) solve_finish(opt, in, r, s_st, s_m, sum.stokes, rad, refl, nf, st);
    }
    __syncthreads();
  }
}

// Warps per block of k_refine_terms.  A block's footprint is kept to that of
// a two-warp series block (about 72 KB of shared memory at 16 streams, half
// an SM's registers at most), so the re-solves of one launch group share the
// SMs with the other groups' launches in flight rather than taking whole SMs
// (measured on GB300 at 16 streams: six-warp blocks of 215 KB cut the
// largest group's own time by 0.6 s but left the concurrent step at 17.3 s;
// two-warp blocks gave 17.0 s).
template <int NS>
constexpr int kRefineWarps = (NS >= 16) ? 2 : (NS >= 12 ? 3 : 4);

// Enqueue the two-pass team solve on storage at `base`: per-solve scratch for
// `slice` solves and their live flags at live_off; counter and first are two
// scheduling ints.
template <int NS, typename T>
int enqueue_team_two_pass(const RtOptions& opt, const LambertInputs& in, const Quad& q, char* base, size_t live_off,
                          long nblocks, int slice, int* counter, int* first, double* rad, double* refl, int* nf,
                          int* st, cudaStream_t s, const Worklist& wl) {
  constexpr int WPB = 2;
  const int nsolve = in.nobs * in.nch;
  const size_t smem = sizeof(TeamMem<NS, T>) * WPB;
  k_init_sched<<<1, 1, 0, s>>>(counter, first, in.nobs, wl.out_count);
  k_nadir_first<<<(in.nobs + 127) / 128, 128, 0, s>>>(in.nobs, in.nch, in.sza, in.raa, in.vza, in.albedo, in.missing,
                                                       first);
  CUDA_TRY(cudaGetLastError());
  count_launches(2);
  LambertInputs in2 = in;
  in2.nadir_first = first;
  for (int b0 = 0; b0 < nsolve; b0 += slice) {
    const int cnt = nsolve - b0 < slice ? nsolve - b0 : slice;
    if (b0 > 0) CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), s));
    k_team_setup<NS, T><<<(unsigned)((cnt + 31) / 32), 32, 0, s>>>(opt, in2, q, base, b0, cnt, rad, refl, nf, st,
                                                                   (unsigned char*)(base + live_off));
    k_team_series<NS, T, WPB><<<(unsigned)nblocks, 32 * WPB, smem, s>>>(
        opt, in2, q, base, b0, cnt, counter, (const unsigned char*)(base + live_off), rad, refl, nf, st, wl);
    CUDA_TRY(cudaGetLastError());
    count_launches(2);
  }
  return 0;
}

// Resident two-warp blocks of the series kernel per SM (sets its shared-memory attribute).
template <int NS, typename T>
int team_series_blocks_per_sm(int* per_sm) {
  constexpr int WPB = 2;
  const size_t smem = sizeof(TeamMem<NS, T>) * WPB;
  CUDA_TRY(cudaFuncSetAttribute(k_team_series<NS, T, WPB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_team_series<NS, T, WPB>, 32 * WPB, smem));
  if (*per_sm < 1) return set_error(AERORT_RC_CUDA, "team kernel does not fit on an SM");
  return 0;
}

template <int NS, typename T>
int launch_scalar_lambert_team(Context& c, const RtOptions& opt, const LambertInputs& in, double* rad, double* refl,
                               int* nf, int* st, cudaStream_t s, const Worklist& wl, bool terms) {
  constexpr int WPB = 2;
  const int nsolve = in.nobs * in.nch;
  if (nsolve == 0) return 0;
  Quad q;
  std::memset(&q, 0, sizeof(q));
  gauss_legendre01(NS, q.qx, q.qw);
  if (opt.nfine > 0) gauss_legendre01(opt.nfine, q.tu, q.wu);
  const int bs = 32 * WPB;
  const size_t smem = sizeof(TeamMem<NS, T>) * WPB;
  if (sizeof(T) == sizeof(double) && (wl.in_list || terms)) {
    // refinement list or a small batch: the term-parallel FP64 solve, as many
    // blocks as the occupancy calculator places (a list: at most two per SM)
    constexpr int W = kRefineWarps<NS>;
    const size_t rsmem = sizeof(TeamMem<NS, double>) * W;
    CUDA_TRY(cudaFuncSetAttribute(k_refine_terms<NS, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem));
    int rper_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rper_sm, k_refine_terms<NS, W>, 32 * W, rsmem));
    if (rper_sm < 1) return set_error(AERORT_RC_CUDA, "term-parallel kernel does not fit on an SM");
    if (wl.in_list && rper_sm > 2) rper_sm = 2;
    long nblocks = (long)rper_sm * c.num_sms;
    if (nblocks > nsolve) nblocks = nsolve;
    const ScratchLayout<NS> lay(in.km, false);
    if (int rc = c.pad->scratch.ensure((size_t)lay.template bytes<double>() * nblocks)) return rc;
    if (int rc = c.pad->counter.ensure(4 * sizeof(int))) return rc;
    int* counter = (int*)c.pad->counter.p;
    int* first = counter + 1;
    k_init_sched<<<1, 1, 0, s>>>(counter, first, in.nobs, wl.out_count);
    k_nadir_first<<<(in.nobs + 127) / 128, 128, 0, s>>>(in.nobs, in.nch, in.sza, in.raa, in.vza, in.albedo,
                                                         in.missing, first);
    CUDA_TRY(cudaGetLastError());
    LambertInputs in2 = in;
    in2.nadir_first = first;
    k_refine_terms<NS, W><<<(unsigned)nblocks, 32 * W, rsmem, s>>>(opt, in2, q, c.pad->scratch.p, nsolve, counter,
                                                                   rad, refl, nf, st, wl);
    CUDA_TRY(cudaGetLastError());
    count_launches(3);
    return 0;
  }
  if (!wl.in_list) {
    int per_sm = 0;
    if (int rc = team_series_blocks_per_sm<NS, T>(&per_sm)) return rc;
    const Schedule& sc = c.sched[sizeof(T) == sizeof(float) ? 1 : 0][stream_index(NS)];
    if (sc.blocks_per_sm > 0 && sc.blocks_per_sm < per_sm) per_sm = sc.blocks_per_sm;
    const int slice = nsolve < kSetupSlice ? nsolve : kSetupSlice;
    long nblocks = (long)per_sm * c.num_sms;
    if (nblocks > (slice + WPB - 1) / WPB) nblocks = (slice + WPB - 1) / WPB;
    const ScratchLayout<NS> lay(in.km, false);
    auto up256 = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t live_off = up256((size_t)lay.template bytes<T>() * slice);
    if (int rc = c.pad->scratch.ensure(live_off + up256((size_t)slice))) return rc;
    if (int rc = c.pad->counter.ensure(4 * sizeof(int))) return rc;
    int* counter = (int*)c.pad->counter.p;
    return enqueue_team_two_pass<NS, T>(opt, in, q, (char*)c.pad->scratch.p, live_off, nblocks, slice, counter,
                                        counter + 1, rad, refl, nf, st, s, wl);
  }
  CUDA_TRY(cudaFuncSetAttribute(k_scalar_lambert_team<NS, T, WPB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
  int per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scalar_lambert_team<NS, T, WPB>, bs, smem));
  if (per_sm < 1) return set_error(AERORT_RC_CUDA, "team kernel does not fit on an SM");
  const Schedule& sc = c.sched[sizeof(T) == sizeof(float) ? 1 : 0][stream_index(NS)];
  if (sc.blocks_per_sm > 0 && sc.blocks_per_sm < per_sm) per_sm = sc.blocks_per_sm;
  long nblocks = 0;
  // a refinement pass (solve list) holds few solves: one per warp grab
  const int chunk = wl.in_list ? team_chunk(1, (long)per_sm * c.num_sms, WPB, &nblocks)
                               : team_chunk(nsolve, (long)per_sm * c.num_sms, WPB, &nblocks);
  if (wl.in_list) nblocks = (long)per_sm * c.num_sms < (nsolve + WPB - 1) / WPB ? (long)per_sm * c.num_sms
                                                                                : (nsolve + WPB - 1) / WPB;
  const long nthreads = nblocks * bs;
  const ScratchLayout<NS> lay(in.km, false);
  if (int rc = c.pad->scratch.ensure((size_t)lay.template bytes<T>() * nthreads)) return rc;
  if (int rc = c.pad->counter.ensure(4 * sizeof(int))) return rc;
  int* counter = (int*)c.pad->counter.p;
  int* first = counter + 1;
  k_init_sched<<<1, 1, 0, s>>>(counter, first, in.nobs, wl.out_count);
  k_nadir_first<<<(in.nobs + 127) / 128, 128, 0, s>>>(in.nobs, in.nch, in.sza, in.raa, in.vza, in.albedo, in.missing,
                                                       first);
  CUDA_TRY(cudaGetLastError());
  LambertInputs in2 = in;
  in2.nadir_first = first;
  k_scalar_lambert_team<NS, T, WPB><<<(unsigned)nblocks, bs, smem, s>>>(opt, in2, q, c.pad->scratch.p, nthreads,
                                                                        nsolve, chunk, counter, rad, refl, nf, st,
                                                                        wl);
  CUDA_TRY(cudaGetLastError());
  count_launches(3);
  return 0;
}

template <int NS, typename T>
int launch_scalar_lambert(Context& c, const RtOptions& opt, const LambertInputs& in, double* rad, double* refl,
                          int* nf, int* st, cudaStream_t s, const Worklist& wl) {
  const int nsolve = in.nobs * in.nch;
  if (nsolve == 0) return 0;
  Quad q;
  std::memset(&q, 0, sizeof(q));
  gauss_legendre01(NS, q.qx, q.qw);
  if (opt.nfine > 0) gauss_legendre01(opt.nfine, q.tu, q.wu);
  const Schedule& sc = c.sched[sizeof(T) == sizeof(float) ? 1 : 0][stream_index(NS)];
  int bs = sc.threads, per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scalar_lambert<NS, T>, bs, 0));
  if (per_sm < 1) per_sm = 1;
  if (sc.blocks_per_sm > 0 && sc.blocks_per_sm < per_sm) per_sm = sc.blocks_per_sm;
  long maxblocks = (long)per_sm * c.num_sms;
  if (wl.in_list && maxblocks > (64L * c.num_sms + bs - 1) / bs) maxblocks = (64L * c.num_sms + bs - 1) / bs;
  long nblocks = (nsolve + bs - 1) / bs;
  if (nblocks > maxblocks) nblocks = maxblocks;
  const long nthreads = nblocks * bs;
  const ScratchLayout<NS> lay(in.km);
  if (int rc = c.pad->scratch.ensure((size_t)lay.template bytes<T>() * nthreads)) return rc;
  if (int rc = c.pad->counter.ensure(4 * sizeof(int))) return rc;
  int* counter = (int*)c.pad->counter.p;
  int* first = counter + 1;
  k_init_sched<<<1, 1, 0, s>>>(counter, first, in.nobs, wl.out_count);
  k_nadir_first<<<(in.nobs + 127) / 128, 128, 0, s>>>(in.nobs, in.nch, in.sza, in.raa, in.vza, in.albedo, in.missing,
                                                       first);
  CUDA_TRY(cudaGetLastError());
  LambertInputs in2 = in;
  in2.nadir_first = first;
  k_scalar_lambert<NS, T><<<(unsigned)nblocks, bs, 0, s>>>(opt, in2, q, c.pad->scratch.p, nthreads, nsolve, counter,
                                                           rad, refl, nf, st, wl);
  CUDA_TRY(cudaGetLastError());
  count_launches(3);
  return 0;
}

// Same launch on fixed storage owned by the caller: the per-thread scratch
// comes from an arena of arena_bytes and the two scheduling ints from sched
// (both reset or fully rewritten here, so neither needs to start at zero).
// The persistent grid is capped so that its threads' scratch fits the arena;
// any nobs is then covered by the work queue.
template <int NS, typename T>
int launch_scalar_lambert_fixed(const RtOptions& opt, const LambertInputs& in, void* arena, size_t arena_bytes,
                                int* sched, int num_sms, const Schedule& sc, double* rad, double* refl, int* nf,
                                int* st, cudaStream_t s, const Worklist& wl) {
  const int nsolve = in.nobs * in.nch;
  if (nsolve == 0) return 0;
  if (sc.kernel == 1 && !wl.in_list) {
    // two-pass team solve when the arena holds per-solve scratch for a slice of
    // at least two solves per resident warp (or the whole batch)
    constexpr int WPB = 2;
    int per_sm = 0;
    if (int rc = team_series_blocks_per_sm<NS, T>(&per_sm)) return rc;
    if (sc.blocks_per_sm > 0 && sc.blocks_per_sm < per_sm) per_sm = sc.blocks_per_sm;
    long nblocks = (long)per_sm * num_sms;
    if (nblocks > ((long)nsolve + WPB - 1) / WPB) nblocks = ((long)nsolve + WPB - 1) / WPB;
    const ScratchLayout<NS> lay(in.km, false);
    auto up256 = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t per_solve = (size_t)lay.template bytes<T>() + 1;
    long fit = arena_bytes > 1024 ? (long)((arena_bytes - 1024) / per_solve) : 0;
    long slice = nsolve < kSetupSlice ? nsolve : kSetupSlice;
    if (slice > fit) slice = fit;
    if (slice >= nsolve || slice >= 2 * nblocks * WPB) {
      Quad q;
      std::memset(&q, 0, sizeof(q));
      gauss_legendre01(NS, q.qx, q.qw);
      if (opt.nfine > 0) gauss_legendre01(opt.nfine, q.tu, q.wu);
      const size_t live_off = up256((size_t)lay.template bytes<T>() * slice);
      return enqueue_team_two_pass<NS, T>(opt, in, q, (char*)arena, live_off, nblocks, (int)slice, sched, sched + 1,
                                          rad, refl, nf, st, s, wl);
    }
  }
  if (sc.kernel == 1) {
    // fused team kernel: per warp 32 set-up scratches inside the arena
    constexpr int WPB = 2;
    const ScratchLayout<NS> tlay(in.km, false);
    const size_t per_warp = 32 * (size_t)tlay.template bytes<T>();
    const long fit_blocks_t = (long)(arena_bytes / (per_warp * WPB));
    if (fit_blocks_t < 1)
      return set_error(AERORT_RC_ARG, "scalar_lambert: one team block needs more scratch than the workspace holds");
    Quad q;
    std::memset(&q, 0, sizeof(q));
    gauss_legendre01(NS, q.qx, q.qw);
    if (opt.nfine > 0) gauss_legendre01(opt.nfine, q.tu, q.wu);
    const size_t smem = sizeof(TeamMem<NS, T>) * WPB;
    CUDA_TRY(cudaFuncSetAttribute(k_scalar_lambert_team<NS, T, WPB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    int per_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scalar_lambert_team<NS, T, WPB>, 32 * WPB, smem));
    if (per_sm < 1) return set_error(AERORT_RC_CUDA, "team kernel does not fit on an SM");
    if (sc.blocks_per_sm > 0 && sc.blocks_per_sm < per_sm) per_sm = sc.blocks_per_sm;
    long resident = (long)per_sm * num_sms;
    if (resident > fit_blocks_t) resident = fit_blocks_t;
    long nblocks = 0;
    const int chunk = team_chunk(wl.in_list ? 1 : nsolve, resident, WPB, &nblocks);
    if (wl.in_list) nblocks = resident < (nsolve + WPB - 1) / WPB ? resident : (nsolve + WPB - 1) / WPB;
    const long nthreads = nblocks * 32 * WPB;
    int* counter = sched;
    int* first = sched + 1;
    k_init_sched<<<1, 1, 0, s>>>(counter, first, in.nobs, wl.out_count);
    k_nadir_first<<<(in.nobs + 127) / 128, 128, 0, s>>>(in.nobs, in.nch, in.sza, in.raa, in.vza, in.albedo,
                                                         in.missing, first);
    CUDA_TRY(cudaGetLastError());
    LambertInputs in2 = in;
    in2.nadir_first = first;
    k_scalar_lambert_team<NS, T, WPB><<<(unsigned)nblocks, 32 * WPB, smem, s>>>(
        opt, in2, q, arena, nthreads, nsolve, chunk, counter, rad, refl, nf, st, wl);
    CUDA_TRY(cudaGetLastError());
    count_launches(3);
    return 0;
  }
  const int bs = sc.threads;
  const ScratchLayout<NS> lay(in.km);
  const long fit_blocks = (long)(arena_bytes / ((size_t)lay.template bytes<T>() * bs));
  if (fit_blocks < 1)
    return set_error(AERORT_RC_ARG, "scalar_lambert: one block needs more scratch than the workspace holds");
  Quad q;
  std::memset(&q, 0, sizeof(q));
  gauss_legendre01(NS, q.qx, q.qw);
  if (opt.nfine > 0) gauss_legendre01(opt.nfine, q.tu, q.wu);
  int per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scalar_lambert<NS, T>, bs, 0));
  if (per_sm < 1) per_sm = 1;
  if (sc.blocks_per_sm > 0 && sc.blocks_per_sm < per_sm) per_sm = sc.blocks_per_sm;
  long nblocks = (nsolve + bs - 1) / bs;
  if (nblocks > (long)per_sm * num_sms) nblocks = (long)per_sm * num_sms;
  if (nblocks > fit_blocks) nblocks = fit_blocks;
  const long nthreads = nblocks * bs;
  int* counter = sched;
  int* first = sched + 1;
  k_init_sched<<<1, 1, 0, s>>>(counter, first, in.nobs, wl.out_count);
  k_nadir_first<<<(in.nobs + 127) / 128, 128, 0, s>>>(in.nobs, in.nch, in.sza, in.raa, in.vza, in.albedo, in.missing,
                                                       first);
  CUDA_TRY(cudaGetLastError());
  LambertInputs in2 = in;
  in2.nadir_first = first;
  k_scalar_lambert<NS, T><<<(unsigned)nblocks, bs, 0, s>>>(opt, in2, q, arena, nthreads, nsolve, counter, rad, refl,
                                                           nf, st, wl);
  CUDA_TRY(cudaGetLastError());
  count_launches(3);
  return 0;
}

// ---------------------------------------------------------------------------------- RTLS BRDF surface
// VLIDORT_Scalar_LandMODIS and VLIDORT_Scalar_CX on the two-pass team solve
// (FP64): k_brdf_setup runs each solve's set-up with its BRDF block
// (rt_brdf.cuh), k_brdf_series the Fourier series with the BRDF surface.  The
// BRDF inputs are a __grid_constant__ parameter: the kernels read them from
// parameter space through a pointer, without a per-thread copy.

// Sticky nadir-FO flag of the BRDF wrappers (VLIDORT_BRDF_MODIS.F90:113-185,
// VLIDORT_BRDF_CX.F90:497-560): the first pixel with valid angles, solar
// zenith exactly 0 and a channel that reaches Run_Scalar (RTLS: its exact
// BRDF is not negative; Cox-Munk: its winds and refractive index are set).
template <int NS>
__global__ void k_brdf_nadir_first(LambertInputs in, const __grid_constant__ BrdfInputs b, int* first) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= in.nobs) return;
  auto miss = [&](double x) { return fabs(x / in.missing - 1.0) < 0.001; };
  if (miss(in.sza[j]) || miss(in.vza[j]) || miss(in.raa[j]) || in.sza[j] != 0.0) return;
  for (int i = 0; i < in.nch; ++i) {
    const long w = (long)i + (long)in.nch * j;
    bool solved;
    if (b.kind != kBrdfRTLS) {
      solved = !(miss(b.u10[j]) || miss(b.v10[j]) || miss(b.mr[i]));
    } else {
      const int t = b.tab ? b.tab[w] : 0;
      solved = !(brdf_exact(b.kw + 3 * w, b.tpar[2 * t], b.tpar[2 * t + 1], in.sza[j], in.vza[j], in.raa[j]) < 0.0);
    }
    if (solved) {
      atomicMin(first, j);
      return;
    }
  }
}

template <int NS>
__global__ void __launch_bounds__(32) k_brdf_setup(RtOptions opt, LambertInputs in, Quad q,
                                                   const __grid_constant__ BrdfInputs b, void* scratch, int base,
                                                   int count, double* rad, double* refl, int* nf, int* st,
                                                   unsigned char* live) {
  const ScratchLayout<NS> lay(in.km, false);
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x) {
    const SolveScratch<double> S = make_scratch<NS, double>(scratch, s, count, in.km, false);
    SetupRecord r;
    const bool ok = solve_setup<NS, double>(opt, in, base + s, q.tu, q.wu, S, rad, refl, nf, st, r, &b, s);
    if (ok) r.store(S.D, lay.rec);
    live[s] = ok ? 1 : 0;
  }
}

template <int NS, int WPB>
__global__ void __launch_bounds__(32 * WPB, 1)
    k_brdf_series(RtOptions opt, LambertInputs in, Quad q, const __grid_constant__ BrdfInputs b, void* scratch,
                  int base, int count, int* counter, const unsigned char* live, double* rad, double* refl, int* nf,
                  int* st) {
  extern __shared__ __align__(16) unsigned char team_smem[];
  const int lane = threadIdx.x & 31;
  TeamMem<NS, double>& M = reinterpret_cast<TeamMem<NS, double>*>(team_smem)[threadIdx.x >> 5];
  const ScratchLayout<NS> lay(in.km, false);
  const Team tm{lane, nullptr, nullptr};
  for (;;) {
    int s = 0;
    if (lane == 0) s = atomicAdd(counter, 1);
    s = __shfl_sync(0xffffffffu, s, 0);
    if (s >= count) break;
    if (!live[s]) continue;
    const SolveScratch<double> S = make_scratch<NS, double>(scratch, s, count, in.km, false);
    SetupRecord r;
    r.load(S.D, lay.rec);
    team_fourier_series<NS, double, true>(tm, M, opt, in, r, q.qx, q.qw, S.W, lay, rad, refl, nf, st, Worklist(),
                                          base + s, &b, s);
  }
}

// The BRDF surface of a call (BrdfSurface, aerort_internal.cuh): RTLS kernel
// amplitudes kw (3, nch, nobs) on the device, ntab Li-sparse (h/b, b/r) pairs
// tpar_host and the table of every solve tab_host (nch x nobs, null when
// ntab == 1) on the host; or Cox-Munk winds u10, v10 (nobs) and refractive
// index mr (nch) on the device.  br (nobs, nch) output on the device.
template <int NS>
int launch_scalar_brdf(Context& c, const RtOptions& opt, const LambertInputs& in, const BrdfSurface& sf, double* rad,
                       double* refl, double* br, int* nf, int* st, cudaStream_t s) {
  constexpr int WPB = 2;
  const int nsolve = in.nobs * in.nch;
  if (nsolve == 0) return 0;
  const bool cx = sf.kind != kBrdfRTLS;  // a glint kernel
  Quad q;
  std::memset(&q, 0, sizeof(q));
  gauss_legendre01(NS, q.qx, q.qw);
  if (opt.nfine > 0) gauss_legendre01(opt.nfine, q.tu, q.wu);
  BrdfInputs b;
  std::memset(&b, 0, sizeof(b));
  b.kind = sf.kind;
  b.q.nb = cx ? kBrdfAzimuthCX : kBrdfAzimuth;
  {
    double x[kBrdfAzimuthCX], w[kBrdfAzimuthCX];
    gauss_legendre01(b.q.nb, x, w);
    for (int k = 0; k < b.q.nb; ++k) {
      b.q.phi[k] = kPIE * x[k];
      b.q.a[k] = w[k];
      b.q.c[k] = std::cos(b.q.phi[k]);
      b.q.s[k] = std::sin(b.q.phi[k]);
    }
  }
  for (int k = 0; k < NS; ++k) b.qx[k] = q.qx[k];
  // RTLS: quadrature-to-quadrature tables, Ross-thick then Li-sparse per
  // parameter pair; Cox-Munk: the azimuth weights a_k cos(m phi_k)
  std::vector<double> qq;
  const int ntab = cx ? 0 : sf.ntab;
  if (cx) {
    qq.resize((size_t)2 * NS * b.q.nb);
    for (int m = 0; m < 2 * NS; ++m)
      for (int k = 0; k < b.q.nb; ++k)
        qq[(size_t)m * b.q.nb + k] = (m == 0) ? b.q.a[k] : b.q.a[k] * std::cos((double)m * b.q.phi[k]);
  } else {
    const size_t tab_elems = (size_t)2 * NS * NS * NS;
    qq.resize((size_t)(1 + ntab) * tab_elems);
    brdf_qq_table(NS, q.qx, b.q, false, 0.0, 0.0, qq.data());
    for (int t = 0; t < ntab; ++t)
      brdf_qq_table(NS, q.qx, b.q, true, sf.tpar_host[2 * t], sf.tpar_host[2 * t + 1],
                    qq.data() + (1 + t) * tab_elems);
  }
  int per_sm = 0;
  {
    const size_t smem = sizeof(TeamMem<NS, double>) * WPB;
    CUDA_TRY(cudaFuncSetAttribute(k_brdf_series<NS, WPB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_brdf_series<NS, WPB>, 32 * WPB, smem));
    if (per_sm < 1) return set_error(AERORT_RC_CUDA, "BRDF team kernel does not fit on an SM");
  }
  // Cox-Munk blocks hold each solve's 2N x N x N components: slices of at
  // most ~2 GB of them
  const long block = cx ? BrdfBlock<NS>::total_cx : BrdfBlock<NS>::total;
  long max_slice = cx ? (2L << 30) / (8 * block) : kSetupSlice;
  if (max_slice > kSetupSlice) max_slice = kSetupSlice;
  const int slice = nsolve < max_slice ? nsolve : (int)max_slice;
  long nblocks = (long)per_sm * c.num_sms;
  if (nblocks > (slice + WPB - 1) / WPB) nblocks = (slice + WPB - 1) / WPB;
  const ScratchLayout<NS> lay(in.km, false);
  auto up256 = [](size_t v) { return (v + 255) / 256 * 256; };
  const size_t live_off = up256((size_t)lay.template bytes<double>() * slice);
  const size_t terms_off = live_off + up256((size_t)slice);
  const size_t qq_off = terms_off + up256(sizeof(double) * (size_t)block * slice);
  const size_t tpar_off = qq_off + up256(sizeof(double) * qq.size());
  const size_t tab_off = tpar_off + up256(sizeof(double) * 2 * (size_t)ntab);
  const size_t total = tab_off + (sf.tab_host && !cx ? up256(sizeof(int) * (size_t)nsolve) : 0);
  if (int rc = c.pad->scratch.ensure(total)) return rc;
  if (int rc = c.pad->counter.ensure(4 * sizeof(int))) return rc;
  char* base = (char*)c.pad->scratch.p;
  // pageable-memory copies: the host buffers may go once the calls return
  CUDA_TRY(cudaMemcpyAsync(base + qq_off, qq.data(), sizeof(double) * qq.size(), cudaMemcpyHostToDevice, s));
  if (cx) {
    b.u10 = sf.u10;
    b.v10 = sf.v10;
    b.mr = sf.mr;
    b.cf = (const double*)(base + qq_off);
  } else {
    CUDA_TRY(cudaMemcpyAsync(base + tpar_off, sf.tpar_host, sizeof(double) * 2 * (size_t)ntab,
                             cudaMemcpyHostToDevice, s));
    if (sf.tab_host)
      CUDA_TRY(cudaMemcpyAsync(base + tab_off, sf.tab_host, sizeof(int) * (size_t)nsolve, cudaMemcpyHostToDevice, s));
    b.kw = sf.kw;
    b.tab = sf.tab_host ? (const int*)(base + tab_off) : nullptr;
    b.tpar = (const double*)(base + tpar_off);
    b.qq = (const double*)(base + qq_off);
  }
  b.br = br;
  b.terms = (double*)(base + terms_off);
  b.stride = slice;
  int* counter = (int*)c.pad->counter.p;
  int* first = counter + 1;
  k_init_sched<<<1, 1, 0, s>>>(counter, first, in.nobs, nullptr);
  k_brdf_nadir_first<NS><<<(in.nobs + 127) / 128, 128, 0, s>>>(in, b, first);
  CUDA_TRY(cudaGetLastError());
  count_launches(2);
  LambertInputs in2 = in;
  in2.nadir_first = first;
  const size_t smem = sizeof(TeamMem<NS, double>) * WPB;
  for (int b0 = 0; b0 < nsolve; b0 += slice) {
    const int cnt = nsolve - b0 < slice ? nsolve - b0 : slice;
    if (b0 > 0) CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), s));
    k_brdf_setup<NS><<<(unsigned)((cnt + 31) / 32), 32, 0, s>>>(opt, in2, q, b, base, b0, cnt, rad, refl, nf, st,
                                                                 (unsigned char*)(base + live_off));
    k_brdf_series<NS, WPB><<<(unsigned)nblocks, 32 * WPB, smem, s>>>(
        opt, in2, q, b, base, b0, cnt, counter, (const unsigned char*)(base + live_off), rad, refl, nf, st);
    CUDA_TRY(cudaGetLastError());
    count_launches(2);
  }
  return 0;
}

}  // namespace aerort_internal

#define AERORT_INSTANTIATE_RT(NS)                                                                             \
  template int aerort_internal::launch_scalar_lambert<NS, double>(                                             \
      aerort_internal::Context&, const aerort::RtOptions&, const aerort::LambertInputs&, double*, double*, int*, \
      int*, cudaStream_t, const aerort::Worklist&);                                                                                      \
  template int aerort_internal::launch_scalar_lambert<NS, float>(                                              \
      aerort_internal::Context&, const aerort::RtOptions&, const aerort::LambertInputs&, double*, double*, int*, \
      int*, cudaStream_t, const aerort::Worklist&);                                                                                      \
  template int aerort_internal::launch_scalar_lambert_team<NS, double>(                                        \
      aerort_internal::Context&, const aerort::RtOptions&, const aerort::LambertInputs&, double*, double*, int*, \
      int*, cudaStream_t, const aerort::Worklist&, bool);                                                                                \
  template int aerort_internal::launch_scalar_lambert_team<NS, float>(                                         \
      aerort_internal::Context&, const aerort::RtOptions&, const aerort::LambertInputs&, double*, double*, int*, \
      int*, cudaStream_t, const aerort::Worklist&, bool);                                                                                      \
  template int aerort_internal::launch_scalar_lambert_fixed<NS, double>(                                       \
      const aerort::RtOptions&, const aerort::LambertInputs&, void*, size_t, int*, int,                         \
      const aerort_internal::Schedule&, double*, double*, int*, int*, cudaStream_t, const aerort::Worklist&);                            \
  template int aerort_internal::launch_scalar_lambert_fixed<NS, float>(                                        \
      const aerort::RtOptions&, const aerort::LambertInputs&, void*, size_t, int*, int,                         \
      const aerort_internal::Schedule&, double*, double*, int*, int*, cudaStream_t, const aerort::Worklist&); \
  template int aerort_internal::launch_scalar_brdf<NS>(                                                        \
      aerort_internal::Context&, const aerort::RtOptions&, const aerort::LambertInputs&,                         \
      const aerort_internal::BrdfSurface&, double*, double*, double*, int*, int*, cudaStream_t);

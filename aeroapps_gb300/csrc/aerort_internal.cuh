// Internal declarations shared by the aerort translation units.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/aerort.h"
#include "rt_solve.cuh"

namespace aerort_internal {

int set_error(int rc, const std::string& msg);

// Kernel launches made by the library since it was loaded (aerort_launch_count).
void count_launches(int n);

#define CUDA_TRY(expr)                                                                                   \
  do {                                                                                                   \
    cudaError_t e_ = (expr);                                                                             \
    if (e_ != cudaSuccess)                                                                               \
      return ::aerort_internal::set_error(AERORT_RC_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Grow-only device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t n);
  void release();
};

// Launch schedule of the RT kernel for one (precision, stream count):
// threads per block (a multiple of 32, <= 128) and resident blocks per SM
// (0 = as many as the occupancy calculator allows).
// kernel: 0 = thread per solve, 1 = team (one warp per solve for the Fourier
// series, rt_team.cuh), 2 = automatic (resolve_kernel), 3 = term-parallel team
// solve (FP64: each solve's Fourier terms over the warps of a block).
struct Schedule {
  int threads = 32;  // one warp per block spreads small batches over more SMs
  int blocks_per_sm = 0;
  int kernel = 2;
};
int stream_index(int nstreams);  // 0..4 for 4, 6, 8, 12, 16; -1 otherwise

// Automatic kernel choice.  The thread kernel runs 32 solves per warp, so it
// needs a large batch to keep the SMs busy; the team kernel has the lower
// per-solve latency.  Measured on GB300 (ragged columns, 20-72 layers), the
// thread kernel wins only at these (precision, stream count) pairs and only
// from this many warps of 32 solves per SM on ([precision][stream index
// 0..4 = 4, 6, 8, 12, 16]; 0 = never).  The FP64 re-solve of a mixed launch's
// short refinement list always takes the team kernel.
constexpr int kThreadMinWarpsPerSm[2][5] = {{2, 3, 3, 0, 0}, {2, 0, 4, 0, 0}};
inline int resolve_kernel(int kernel, int precision, int si, long nsolve, int num_sms, bool list) {
  if (list) return 1;
  if (kernel == 3) return precision == 0 ? 3 : 1;  // the term-parallel form exists in FP64
  if (kernel == 0 || kernel == 1) return kernel;
  if (si < 0 || precision < 0 || precision > 1) return 0;
  const int w = kThreadMinWarpsPerSm[precision][si];
  return (w > 0 && nsolve >= 32L * w * num_sms) ? 0 : 1;
}

// Device scratch of the library's own RT launches for one caller stream:
// per-thread solve scratch, the scheduling ints and the mixed method's
// refinement list.
struct Pad {
  DevBuf scratch, counter, redo;
  cudaStream_t owner = nullptr;
  cudaEvent_t done = nullptr;  // recorded on `owner` after the last launch that used the pad
  bool captured = false;       // used by work captured into a CUDA graph: stays with `owner`
  unsigned long last = 0;
  bool used = false;
};

// Library context: stream, scratch pads, staging buffers.  One per process;
// host calls are serialised by the mutex (the reference library is serial per
// process).  Device work enqueued on different caller streams gets different
// pads (up to kPads streams at once), so it may overlap on the GPU; a pad
// handed from one stream to another makes the new stream wait, on the device,
// for the work last enqueued on it.
struct Context {
  static constexpr int kPads = 16;
  std::mutex mu;
  bool init = false;
  int device = -1, num_sms = 0;
  cudaStream_t stream = nullptr;
  Pad pads[kPads];
  Pad* pad = nullptr;         // the pad of the call in progress (set by bind)
  Pad* last_mixed = nullptr;  // the pad of the last mixed-method call
  unsigned long tick = 0;
  DevBuf stage[24];
  Schedule sched[2][5];  // [precision][stream index]
  int setup();
  void release();
  int bind(cudaStream_t s);    // select the pad of stream s
  int unbind(cudaStream_t s);  // mark the pad busy until the work enqueued on s so far is done
  Pad* find(cudaStream_t s);
};

Context& ctx();

// Gauss-Legendre nodes/weights on (0,1), ascending (as VLIDORT's GETQUAD2).
void gauss_legendre01(int n, double* x, double* w);

struct Quad {
  double qx[16], qw[16], tu[aerort::kMaxFine], wu[aerort::kMaxFine];
};

template <int NS, typename T>
int launch_scalar_lambert(Context& c, const aerort::RtOptions& opt, const aerort::LambertInputs& in, double* rad,
                          double* refl, int* nf, int* st, cudaStream_t s, const aerort::Worklist& wl);

// terms: the term-parallel team solve (k_refine_terms) for every solve (FP64;
// a refinement list always takes it)
template <int NS, typename T>
int launch_scalar_lambert_team(Context& c, const aerort::RtOptions& opt, const aerort::LambertInputs& in, double* rad,
                               double* refl, int* nf, int* st, cudaStream_t s, const aerort::Worklist& wl,
                               bool terms = false);
template <int NS, typename T>
int launch_scalar_lambert_fixed(const aerort::RtOptions& opt, const aerort::LambertInputs& in, void* arena,
                                size_t arena_bytes, int* sched, int num_sms, const Schedule& sc, double* rad,
                                double* refl, int* nf, int* st, cudaStream_t s, const aerort::Worklist& wl);

// VLIDORT_Init limits and the solve-count guard shared by every RT entry point
// (rc 2, 3, 5 as the reference; AERORT_RC_ARG for bad sizes).
int lambert_checks(int km, int nch, int nobs, int nstreams, int nMom);

// VLIDORT_Scalar_LandMODIS (RTLS BRDF surface), FP64 two-pass team solve.
// The BRDF surface of a VLIDORT_Scalar_LandMODIS or VLIDORT_Scalar_CX call.
struct BrdfSurface {
  int kind = aerort::kBrdfRTLS;
  // RTLS: kernel amplitudes (3, nch, nobs) on the device; Li-sparse
  // parameter pairs and each solve's pair (null: one pair) on the host
  const double* kw = nullptr;
  const int* tab_host = nullptr;
  const double* tpar_host = nullptr;
  int ntab = 0;
  // Cox-Munk: winds (nobs) and refractive index (nch) on the device
  const double* u10 = nullptr;
  const double* v10 = nullptr;
  const double* mr = nullptr;
};

template <int NS>
int launch_scalar_brdf(Context& c, const aerort::RtOptions& opt, const aerort::LambertInputs& in,
                       const BrdfSurface& sf, double* rad, double* refl, double* br, int* nf, int* st,
                       cudaStream_t s);

// Static device arena of the allocation-free entry point (rt_static.cu):
// address of the calling thread's current device's copy, set up on first use.
int static_arena(double** arena, size_t* arena_doubles, int** sched, int* num_sms);
void static_arena_forget();

}  // namespace aerort_internal

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
// series, rt_team.cuh).
struct Schedule {
  int threads = 32;  // one warp per block spreads small batches over more SMs
  int blocks_per_sm = 0;
  int kernel = 0;
};
int stream_index(int nstreams);  // 0..4 for 4, 6, 8, 12, 16; -1 otherwise

// Library context: stream, scratch, staging buffers.  One per process; calls
// are serialised by the mutex (the reference library is serial per process).
struct Context {
  std::mutex mu;
  bool init = false;
  int device = -1, num_sms = 0;
  cudaStream_t stream = nullptr;
  DevBuf scratch, counter, redo, stage[24];
  Schedule sched[2][5];  // [precision][stream index]
  Context() {
    // measured on GB300: the team kernel wins at 6, 12 and 16 streams in the
    // mixed method and at 12 and 16 in FP64 (stream index 0..4 = 4, 6, 8, 12, 16)
    sched[1][1].kernel = 1;
    sched[1][3].kernel = 1;
    sched[1][4].kernel = 1;
    sched[0][3].kernel = 1;
    sched[0][4].kernel = 1;
  }
  int setup();
  void release();
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

template <int NS, typename T>
int launch_scalar_lambert_team(Context& c, const aerort::RtOptions& opt, const aerort::LambertInputs& in, double* rad,
                               double* refl, int* nf, int* st, cudaStream_t s, const aerort::Worklist& wl);
template <int NS, typename T>
int launch_scalar_lambert_fixed(const aerort::RtOptions& opt, const aerort::LambertInputs& in, void* arena,
                                size_t arena_bytes, int* sched, int num_sms, const Schedule& sc, double* rad,
                                double* refl, int* nf, int* st, cudaStream_t s, const aerort::Worklist& wl);

// Static device arena of the allocation-free entry point (rt_static.cu):
// address of the calling thread's current device's copy, set up on first use.
int static_arena(double** arena, size_t* arena_doubles, int** sched, int* num_sms);

}  // namespace aerort_internal

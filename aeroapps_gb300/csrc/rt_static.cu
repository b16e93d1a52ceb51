// Fixed device storage of aerort_vlidort_scalar_lambert_batch_dev_noalloc.
//
// Some callers cannot let a library allocate device memory in the middle of a
// run: a model that hands all device memory to its own pool allocator at start
// up, or a serving loop with other streams in flight, where cudaFree (which
// synchronises the whole device) or a failing cudaMalloc would stall or break
// unrelated work.  For them the RT scratch lives in a file-scope array that
// the CUDA module reserves when it is loaded, so a call only launches kernels.
//
// The arena is in its own translation unit, hence its own CUDA module.  Under
// lazy module loading (the CUDA default) a process that never calls this entry
// point does not reserve it; with CUDA_MODULE_LOADING=EAGER every process that
// loads the library reserves the 256 MiB on each device it initialises.
#include "aerort_internal.cuh"

namespace aerort_internal {

// 256 MiB of FP64 scratch.  One 32-thread block of the thread-per-solve RT
// kernel needs 32 x ScratchLayout(km).total doubles (about 11 MiB at 16
// streams and 72 layers), one two-warp block of the team kernel 64 set-up
// scratches, so every supported (nstreams, km) fits;
// the grid is capped to what the arena holds, which bounds throughput at
// large stream counts.
constexpr size_t kArenaDoubles = (size_t)32 << 20;
static __device__ __align__(256) double g_rt_arena[kArenaDoubles];
// Work counter and sticky-nadir index; reset on the stream by every call.
static __device__ __align__(256) int g_rt_sched[2];

namespace {
constexpr int kMaxDevices = 64;
struct ArenaSlot {
  bool ready = false;
  double* arena = nullptr;
  int* sched = nullptr;
  int num_sms = 0;
};
std::mutex g_arena_mu;
ArenaSlot g_arena[kMaxDevices];
}  // namespace

// Per-device set-up on first use, with that device current: the symbol
// lookups may load this module (and reserve the arena), so the first call on
// a device should come before any stream capture.
int static_arena(double** arena, size_t* arena_doubles, int** sched, int* num_sms) {
  int dev = -1;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(AERORT_RC_ARG, "scalar_lambert_noalloc: device index >= 64");
  std::lock_guard<std::mutex> lk(g_arena_mu);
  ArenaSlot& slot = g_arena[dev];
  if (!slot.ready) {
    void* a = nullptr;
    void* s = nullptr;
    int sms = 0;
    CUDA_TRY(cudaGetSymbolAddress(&a, g_rt_arena));
    CUDA_TRY(cudaGetSymbolAddress(&s, g_rt_sched));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    slot.arena = (double*)a;
    slot.sched = (int*)s;
    slot.num_sms = sms;
    slot.ready = true;
  }
  *arena = slot.arena;
  *arena_doubles = kArenaDoubles;
  *sched = slot.sched;
  *num_sms = slot.num_sms;
  return 0;
}

// Forget the cached symbol addresses (aerort_release): after a device reset
// the module is loaded again, possibly at another address.
void static_arena_forget() {
  std::lock_guard<std::mutex> lk(g_arena_mu);
  for (auto& slot : g_arena) slot = ArenaSlot();
}

}  // namespace aerort_internal

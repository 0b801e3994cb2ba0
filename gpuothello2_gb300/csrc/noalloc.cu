// solve_batch_device_noalloc: the batched solver for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc: a host program that has handed all
// device memory to its own pool allocator, a plugin whose host application
// forbids allocation after start-up, or code that must not hit the implicit
// device synchronisation an allocation can cause.  This entry point runs the
// same bucketing and batched search kernels as solve_batch_device, but every
// scratch buffer they need (queue order, bucket counters, status word,
// overflow frame slots) lives in one fixed array, g_noalloc_scratch, compiled
// into the library.  Every GPU that loads the library holds that array
// (about 12 MiB) until the process exits.  The caller passes device arrays
// for the inputs and the scores.
//
// Limits: at most GPO_NOALLOC_MAX_POSITIONS positions and depth at most
// GPO_NOALLOC_MAX_DEPTH per call; larger calls are rejected with GPO_ERR_ARG
// / GPO_ERR_DEPTH before any GPU work.  The transposition table is off (it
// needs its own buffer); helping between the lanes of a warp needs no
// buffer and stays on; scores are the same exact scores.  When the frame
// slots do not fit in shared memory and would not fit the array for the
// full grid, the launch uses fewer blocks (the largest grid that fits).
//
// The array is shared by every call and keeps the last call's contents: the
// status word and bucket counters are cleared at the start of each call, and
// calls that overlap on the GPU (different streams or threads) race on it.
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (once per device, with that device current); make
// that first call before any stream capture.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/gpuothello2.h"
#include "kernels.h"

namespace gpo {
namespace {

constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

constexpr size_t kStatsOff = 0;
constexpr size_t kHistOff = align_up(kStatsOff + sizeof(DeviceStats));
constexpr size_t kCursorOff = align_up(kHistOff + 65 * sizeof(unsigned));
constexpr size_t kPermOff = align_up(kCursorOff + 65 * sizeof(unsigned));
constexpr size_t kFramesOff =
    align_up(kPermOff + static_cast<size_t>(GPO_NOALLOC_MAX_POSITIONS) * sizeof(unsigned));
constexpr size_t kFramesBytes = 8u << 20;  // frame slots above the shared-memory tier
constexpr size_t kScratchBytes = kFramesOff + kFramesBytes;

std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};

}  // namespace

// The scratch array.  Host code must not use its name as an address: the
// device address comes from cudaGetSymbolAddress (scratch_address below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

int scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return GPO_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return GPO_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      std::fprintf(stderr, "gpuothello2: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
      return GPO_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return GPO_OK;
}

}  // namespace
}  // namespace gpo

using namespace gpo;

extern "C" int solve_batch_device_noalloc(const uint64_t* d_player, const uint64_t* d_opp, int n,
                                          int depth, int8_t* d_score, void* stream) {
  if (n < 0 || n > GPO_NOALLOC_MAX_POSITIONS) return GPO_ERR_ARG;
  if (n > 0 && (!d_player || !d_opp || !d_score)) return GPO_ERR_ARG;
  if (depth < 1 || depth > GPO_NOALLOC_MAX_DEPTH) return GPO_ERR_DEPTH;
  if (n == 0) return GPO_OK;
  unsigned char* base = nullptr;
  int rc = scratch_address(&base);
  if (rc != GPO_OK) return rc;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return GPO_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DeviceStats* stats = reinterpret_cast<DeviceStats*>(base + kStatsOff);
  unsigned* hist = reinterpret_cast<unsigned*>(base + kHistOff);
  unsigned* cursor = reinterpret_cast<unsigned*>(base + kCursorOff);
  unsigned* perm = reinterpret_cast<unsigned*>(base + kPermOff);
  const u64* P = reinterpret_cast<const u64*>(d_player);
  const u64* O = reinterpret_cast<const u64*>(d_opp);

  // Everything that must start at zero is cleared here (no allocation).
  if (cudaMemsetAsync(stats, 0, sizeof(DeviceStats), s) != cudaSuccess) return GPO_ERR_CUDA;
  if (cudaMemsetAsync(hist, 0, 65 * sizeof(unsigned), s) != cudaSuccess) return GPO_ERR_CUDA;
  if (launch_bucket(P, O, n, depth, hist, cursor, perm, stats, sms, s) != cudaSuccess)
    return GPO_ERR_CUDA;

  BatchedArgs a = {};
  a.player = P;
  a.opp = O;
  a.perm = perm;
  a.n = n;
  a.depth = depth;
  a.score = reinterpret_cast<signed char*>(d_score);
  a.stats = stats;
  a.ff = 6;
  a.stab_min = 4;
  a.stab_gate = 10;
  a.help_min = 7;
  a.wait_limit_ns = 600000ULL * 1000000ULL;
  BatchedLaunch cfg;
  cfg.threads = 128;
  cfg.grid = 0;
  if (batched_plan(cfg.threads, depth, &a.smem_top) != cudaSuccess) return GPO_ERR_CUDA;
  size_t smem = 0;
  if (batched_grid(cfg.threads, a.smem_top, sms, &cfg.grid, &smem) != cudaSuccess)
    return GPO_ERR_CUDA;
  // Frame slots that do not fit in shared memory come from the fixed array:
  // when they would not fit it for the full grid, the grid shrinks to the
  // largest that fits.
  const size_t per_block = batched_gframe_bytes(depth, a.smem_top, cfg.threads);
  if (per_block > 0) {
    const int grid_cap = static_cast<int>(kFramesBytes / per_block);
    if (grid_cap < 1) return GPO_ERR_DEPTH;
    if (cfg.grid > grid_cap) cfg.grid = grid_cap;
  }
  const long warps = static_cast<long>(cfg.grid) * (cfg.threads / 32);
  const long per = (n + warps - 1) / warps;
  a.roots_per_warp = static_cast<int>(per < 1 ? 1 : (per > 32 ? 32 : per));
  a.gframes = base + kFramesOff;
  if (launch_batched(a, cfg, sms, s) != cudaSuccess) return GPO_ERR_CUDA;

  DeviceStats hs;
  if (cudaMemcpyAsync(&hs, stats, sizeof(hs), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return GPO_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return GPO_ERR_CUDA;
  if (hs.status & kErrOverlap) return GPO_ERR_BOARD;
  if (hs.status & kErrDepth) return GPO_ERR_DEPTH;
  if (hs.status & (kErrBudget | kErrWait)) return GPO_ERR_TIMEOUT;
  if (hs.status & (kErrInternal | kErrTable)) return GPO_ERR_INTERNAL;
  return GPO_OK;
}

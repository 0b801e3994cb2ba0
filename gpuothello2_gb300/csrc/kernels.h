// Host launchers of the solver kernels (one per kernel file), used by the
// C-ABI layer.  Each returns the launch's cudaError_t.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace gpo {

struct BatchedArgs {
  const u64* player;
  const u64* opp;
  const unsigned* perm;  // queue order: position index for each slot
  int n;
  int depth;             // largest empty count allowed (positions above it are rejected)
  int levels;            // push levels provided by the frame storage
  int ff;                // fastest-first threshold (empties)
  signed char* score;
  signed char* best;               // may be null
  unsigned long long* nodes_out;   // may be null
  DeviceStats* stats;
  unsigned long long node_budget;  // 0 = none
};

struct BatchedLaunch {
  int threads;      // threads per block
  bool smem_stack;  // frames in shared (true) or local memory
  int grid;         // out: blocks launched
  size_t smem;      // out: dynamic shared memory per block
};

cudaError_t launch_plain(const u64* player, const u64* opp, int n, int depth, signed char* score,
                         unsigned long long* nodes_out, DeviceStats* stats, cudaStream_t s);
cudaError_t launch_bucket(const u64* player, const u64* opp, int n, int depth, unsigned* hist,
                          unsigned* cursor, unsigned* perm, DeviceStats* stats, int sms,
                          cudaStream_t s);
cudaError_t launch_batched(const BatchedArgs& args, BatchedLaunch& cfg, int sms, cudaStream_t s);
cudaError_t launch_generate(u64 seed, u64 first, int n, int min_e, int max_e, u64* out_p,
                            u64* out_o, cudaStream_t s);

// Frame levels the batched kernel needs for positions of up to `depth`
// empties: nodes with more than kSmallMax + 1 empties push a frame.
int batched_levels(int depth);

}  // namespace gpo

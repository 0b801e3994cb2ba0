// Host launchers of the solver kernels (one per kernel file), used by the
// C-ABI layer.  Each returns the launch's cudaError_t.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace gpo {

struct DonatedTask {
  u64 player, opp;   // position to search, side to move first
  int alpha, beta;   // window
  unsigned slot;     // accumulator slot of this task
  unsigned pad;
};

struct BatchedArgs {
  const u64* player;
  const u64* opp;
  const unsigned* perm;  // queue order: position index for each slot
  int n;
  int depth;             // largest empty count allowed (positions above it are rejected)
  int ff;                // fastest-first threshold (empties)
  signed char* score;
  signed char* best;               // may be null
  unsigned long long* nodes_out;   // may be null
  DeviceStats* stats;
  unsigned long long node_budget;  // 0 = none
  // Frame slots: a node with E empties saves its frame in slot E when it
  // pushes a child.  Slots 2..smem_top live in shared memory, slots
  // smem_top+1..depth in the global array gframes (per-lane, SoA).
  int smem_top;
  unsigned char* gframes;  // (depth - smem_top) * 20 bytes per grid thread, or null
  // Work donation (splitting hard positions across lanes).  Task slots
  // 0..n-1 are the input positions; donated subtrees get slots n.. .
  int donate_min;            // a task root needs this many empties to donate (0 = off)
  unsigned task_cap;         // donated tasks that fit in the arrays below
  unsigned* acc;             // per slot: packed (value + 128) << 8 | move, atomicMax
  unsigned* pending;         // per slot: local search + donated children still running
  unsigned* parent;          // per donated slot: slot to report to
  unsigned char* psq;        // per donated slot: move from the parent
  unsigned* top;             // per donated slot: input position it belongs to
  DonatedTask* queue;        // donation queue records (task_cap)
  unsigned* ready;           // per queue record: 1 once written
  unsigned long long wait_limit_ns;  // bound on an idle lane's wait for work
};

struct BatchedLaunch {
  int threads;      // threads per block
  int grid;         // blocks (0 = fill the GPU at the kernel's occupancy)
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

// Grid size (blocks) the batched kernel runs at for a launch shape; the
// global frame area must cover grid * threads lanes.
cudaError_t batched_grid(int threads, int smem_top, int sms, int* grid, size_t* smem);
// Largest shared-memory frame tier (slots 2..smem_top) that keeps the
// register-limited occupancy of a `threads`-wide block.
cudaError_t batched_plan(int threads, int depth, int* smem_top);

}  // namespace gpo

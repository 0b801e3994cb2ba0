// Host launchers of the solver kernels (one per kernel file), used by the
// C-ABI layer.  Each returns the launch's cudaError_t.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace gpo {

// Devices a process may use the library on (per-device contexts).
constexpr int kMaxDevices = 64;

// Bytes per search frame slot (move word, flips, packed window) and per
// lane of split-node state, both in shared memory (batched.cu).
constexpr int kFrameBytes = 20;
constexpr int kSplitBytes = 40;

struct BatchedArgs {
  const u64* player;
  const u64* opp;
  const unsigned* perm;  // queue order: position index for each slot
  int n;
  int depth;             // largest empty count allowed (positions above it are rejected)
  signed char* score;
  signed char* best;               // may be null
  unsigned long long* nodes_out;   // may be null
  DeviceStats* stats;
  int ff;                // fastest-first ordering at nodes with >= ff empties
  int stab_min;          // stability cutoff at nodes with >= stab_min empties (0 = off) ...
  int stab_gate;         // ... whose alpha is at least stab_gate + 3 * empties
  int help_min;          // split nodes need >= help_min empties (0 = no helping)
  int roots_per_warp;    // input positions a warp searches at once (1..32)
  unsigned long long hard_nodes;  // a warp with a search past this many nodes takes no new
                                  // positions, its free lanes help (0 = off)
  // Frame slots: a node with E empties saves its frame in slot E (3..depth)
  // when it pushes a child.  depth <= smem_top: every slot in shared memory;
  // else every slot in the global array gframes (per lane, SoA).
  int smem_top;
  unsigned char* gframes;  // batched_gframe_bytes(depth, smem_top, lanes), or null
  // Transposition table (table.cuh): 2^tt_bits entries of 16 bytes; nodes
  // with at least tt_min empties probe it when created and store a bound
  // when closed.  tt_min = 0 disables it.
  unsigned long long* tt;
  int tt_bits;
  int tt_min;
  // Learned order table (mlp.cu): 2^order_bits entries of {x, y, list, 0};
  // a node with at least learned_min empties and two or more moves found
  // there searches its moves in the listed order instead of fastest-first
  // (null = off).
  const u64* order_table;
  int order_bits;
  int learned_min;
  unsigned long long node_budget;    // per input position, 0 = none (watchdog)
  unsigned long long wait_limit_ns;  // deadline of the launch, from its start
  // Tail handoff: once the queue is used up and at most tail_count input
  // positions are unfinished, every search stops and its position's score
  // is kUnsolvedDev, for the host to solve spread over the whole GPU
  // (0 = off).
  unsigned tail_count;
  // Per input position, the root's lower bound when it was handed back: the
  // best value of its completed moves (-65 = none yet); null = not wanted.
  signed char* tail_bound;
  // Per input position, the root's window (alpha, beta); null = (-64, 64).
  // A root searched with a window gets a fail-soft score: exact inside the
  // window, a bound outside it.
  const signed char* root_window;
};

struct BatchedLaunch {
  int threads;      // threads per block
  int grid;         // blocks (0 = fill the GPU at the kernel's occupancy)
  size_t smem;      // out: dynamic shared memory per block
};

// limit_ns: deadline of the launch from its first block's start; positions
// still running then stop and the call reports GPO_ERR_TIMEOUT.
cudaError_t launch_plain(const u64* player, const u64* opp, int n, int depth, signed char* score,
                         unsigned long long* nodes_out, DeviceStats* stats,
                         unsigned long long limit_ns, cudaStream_t s);
cudaError_t launch_bucket(const u64* player, const u64* opp, int n, int depth, unsigned* hist,
                          unsigned* cursor, unsigned* perm, DeviceStats* stats, int sms,
                          cudaStream_t s);
cudaError_t launch_batched(const BatchedArgs& args, BatchedLaunch& cfg, int sms, cudaStream_t s);
// The launch alone, with a shape from batched_grid (no attribute calls: usable
// inside a stream capture).
cudaError_t launch_batched_shape(const BatchedArgs& args, int grid, int threads, size_t smem,
                                 cudaStream_t s);
cudaError_t launch_generate(u64 seed, u64 first, int n, int min_e, int max_e, u64* out_p,
                            u64* out_o, cudaStream_t s);

// Grid size (blocks) the batched kernel runs at for a launch shape; the
// global frame area must cover grid * threads lanes.
cudaError_t batched_grid(int threads, int smem_top, int sms, int* grid, size_t* smem);
// Frame placement for a `threads`-wide block: smem_top = depth when every
// frame slot fits in shared memory at the register-limited occupancy, else 2
// (all slots in global memory).
cudaError_t batched_plan(int threads, int depth, int* smem_top);
// Dynamic shared memory of one block, and the global frame bytes for
// `lanes` grid threads.
size_t batched_smem_bytes(int threads, int smem_top);
size_t batched_gframe_bytes(int depth, int smem_top, size_t lanes);

// Learned orderer (mlp.cu).
bool mlp_loaded();
// Learned order table for the roots d_idx[0..count) (mlp.cu): frontier of
// nodes with >= L empties two plies deep, scored by the network, inserted
// into `table` (2^table_bits entries of 32 bytes, cleared by the call).
// *launched receives the number of kernels it launched, *frontier the
// frontier nodes scored.
int mlp_order_frontier(const u64* d_player, const u64* d_opp, const unsigned* d_idx, long count,
                       int L, u64* frontP, u64* frontO, long cap, unsigned long long* counter,
                       u64* table, int table_bits, cudaStream_t s, unsigned* launched,
                       long* frontier);

}  // namespace gpo

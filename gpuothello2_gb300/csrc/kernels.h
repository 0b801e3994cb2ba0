// Host launchers of the solver kernels (one per kernel file), used by the
// C-ABI layer.  Each returns the launch's cudaError_t.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace gpo {

struct DonatedTask {
  u64 player, opp;   // position to search, side to move first
  unsigned window;   // alpha & 0xff | (beta & 0xff) << 8 | move from the donor << 16
  unsigned mbox;     // mailbox index of the donating node
  unsigned top;      // input position the subtree belongs to
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
  int budget_mark;       // 1: an input position over budget gets score -128, no error
  // Frame slots: a node with E empties saves its frame in slot E when it
  // pushes a child.  Slots 2..smem_top live in shared memory, slots
  // smem_top+1..depth in the global array gframes (per-lane, SoA).
  int smem_top;
  unsigned char* gframes;  // (depth - smem_top) * 20 bytes per grid thread, or null
  // Work donation (young brothers wait, any depth).  A node whose first
  // move has returned may hand further moves to idle lanes; results come
  // back through its mailbox (one per lane and empty count).
  int donate_min;            // a donating node needs this many empties (0 = off)
  unsigned long long long_nodes;  // a root past this many nodes hands out moves unasked
  unsigned* pos_tasks;       // per input position: handed-out subtrees not yet done
  // Transposition table (table.cuh): 2^tt_bits entries of 16 bytes; nodes
  // with at least tt_min empties probe it when created and store a bound
  // when closed.  tt_min = 0 disables it.
  unsigned long long* tt;
  int tt_bits;
  int tt_min;
  // Learned root orders (mlp.cu): for an input position with at least
  // learned_min empties, root_lists[pos] replaces the root's ordering
  // probes (null = off).
  const u64* root_lists;
  int learned_min;
  unsigned max_tasks;        // cap on pos_tasks (bounds the search overhead of splitting)
  unsigned task_cap;         // queue records (a ring: ticket t uses record t % task_cap)
  unsigned* mbox_acc;        // [(kMaxEmpties + 1) * grid threads] packed (value+128)<<8 | move
  unsigned* mbox_pend;       // same shape: handed-out moves not yet reported
  unsigned* mbox_cancel;     // same shape: 1 = the node was cut off, helpers may stop
  DonatedTask* queue;        // records, filled in ticket order
  unsigned* ready;           // per record: ticket + 1 of the last fill
  unsigned* consumed;        // per record: ticket + 1 of the last read
  unsigned long long wait_limit_ns;  // deadline of the launch, from its start
  // Search window of each input position (null = -64, 64).  A narrower
  // window gives the fail-soft value: exact inside it, a bound outside.
  const signed char* root_alpha;
  const signed char* root_beta;
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

// Learned orderer (mlp.cu).
bool mlp_loaded();
// *launched receives the number of kernels it launched.
int mlp_order_roots(const u64* d_player, const u64* d_opp, const unsigned* d_idx, long count,
                    u64* d_lists, cudaStream_t s, unsigned* launched);

// Positions whose score is -128 (over budget in a first pass), compacted:
// idx[0..*count) = their indices, in order.
cudaError_t launch_collect_marked(const signed char* score, int n, unsigned* idx, unsigned* count,
                                  cudaStream_t s);
cudaError_t launch_gather(const u64* P, const u64* O, const unsigned* idx, int count, u64* outP,
                          u64* outO, cudaStream_t s);
cudaError_t launch_scatter_scores(const signed char* sc, const signed char* best,
                                  const unsigned long long* nodes, const unsigned* idx, int count,
                                  signed char* score_out, signed char* best_out,
                                  unsigned long long* nodes_out, cudaStream_t s);

// Expansion of hard positions into their children and the bottom-up
// combination of the children's exact scores (prep.cu).
// pa/pb: search windows of the level's positions (null = full window);
// ca/cb receive the children's windows (written only when pa is given).
cudaError_t launch_expand(const u64* P, const u64* O, const unsigned* idx, int m, u64* cP, u64* cO,
                          unsigned* cparent, unsigned char* cmove, unsigned* counter, unsigned cap,
                          const signed char* pa, const signed char* pb, signed char* ca,
                          signed char* cb, cudaStream_t s);
// Principal-variation-first expansion: first children (set A, one per
// marked position, at its slot) and the rest (set B); the parents' values
// through A; B's null windows; the B children that beat the bound (set C,
// with the window (-64, -bound)).
cudaError_t launch_expand_first(const u64* P, const u64* O, const unsigned* idx, int m, u64* aP,
                                u64* aO, unsigned* aparent, unsigned char* amove, u64* bP, u64* bO,
                                unsigned* bparent, unsigned char* bmove, unsigned* counter,
                                unsigned cap, cudaStream_t s);
cudaError_t launch_pvs_bound(const signed char* ascore, const unsigned* aparent, int m,
                             signed char* bound, cudaStream_t s);
cudaError_t launch_pvs_window(const unsigned* bparent, int nb, const signed char* bound,
                              signed char* ba, signed char* bb, cudaStream_t s);
cudaError_t launch_pvs_research(const u64* bP, const u64* bO, const unsigned* bparent,
                                const unsigned char* bmove, const signed char* bscore, int nb,
                                const signed char* bound, u64* cP, u64* cO, unsigned* cparent,
                                unsigned char* cmove, signed char* ca, signed char* cb,
                                unsigned* counter, cudaStream_t s);
// Recursive principal-variation-first expansion: children's windows from
// their parents' (null = full); siblings of first children with null windows
// (cut parents skipped; flag = parent needs a re-search); the flagged
// siblings that beat the bound, with the window above it; and the
// siblings' combination (node counts always, values unless skip[i]; see
// pvs_siblings_kernel in prep.cu for when a sibling's value is left out).
cudaError_t launch_child_window(const unsigned* cparent, int count, const signed char* pa,
                                const signed char* pb, signed char* ca, signed char* cb,
                                cudaStream_t s);
cudaError_t launch_pvs_siblings(const u64* bP, const u64* bO, const unsigned* bparent,
                                const unsigned char* bmove, int nb, const signed char* pa,
                                const signed char* pb, const signed char* bound, u64* oP, u64* oO,
                                unsigned* opar, unsigned char* omove, signed char* oa,
                                signed char* ob, unsigned char* oflag, unsigned char* oskip,
                                unsigned* counter, cudaStream_t s);
cudaError_t launch_pvs_research2(const u64* sP, const u64* sO, const unsigned* spar,
                                 const unsigned char* smove, const signed char* sscore,
                                 const unsigned char* sflag, int ns, const signed char* pa,
                                 const signed char* pb, const signed char* bound, u64* cP, u64* cO,
                                 unsigned* cpar, unsigned char* cmove, signed char* ca,
                                 signed char* cb, unsigned* counter, cudaStream_t s);
cudaError_t launch_combine_masked(const signed char* cscore, const unsigned* cparent,
                                  const unsigned char* cmove, const unsigned long long* cnodes,
                                  const unsigned char* skip, int count, unsigned* acc,
                                  unsigned long long* nodes, cudaStream_t s);
cudaError_t launch_combine(const signed char* cscore, const unsigned* cparent,
                           const unsigned char* cmove, const unsigned long long* cnodes, int count,
                           unsigned* acc, unsigned long long* nodes, cudaStream_t s);
cudaError_t launch_finalize(const unsigned* idx, int m, const unsigned* acc, signed char* score,
                            signed char* best, cudaStream_t s);

}  // namespace gpo

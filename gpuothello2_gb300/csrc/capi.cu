// C-ABI layer: library context, device buffers, the solve pipeline and
// error mapping.  Replaces the reference's BatchedTask resource owner
// (solver.cuh:8-25, solver.cu:313-348): instead of managed memory migrated
// inside the timed region and a host busy-poll (main.cu:149-155), inputs are
// copied explicitly into grow-only device buffers, the pipeline runs on one
// stream, and the call waits on that stream.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gpuothello2.h"
#include "kernels.h"

namespace gpo {
namespace {

// One context per CUDA device, created on first use with that device
// current; every call uses the context of the device current at the call.
struct Context {
  int device = -1;
  int sms = 0;
  size_t mem = 0;  // device memory in bytes
  char name[256] = {0};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  size_t cap = 0;  // host-buffer entry points: staged inputs and outputs
  u64* dP = nullptr;
  u64* dO = nullptr;
  signed char* dScore = nullptr;
  signed char* dBest = nullptr;
  unsigned long long* dNodes = nullptr;
  size_t pass_cap = 0;  // per-position scratch of a search: queue order
  unsigned* dPerm = nullptr;
  long front_cap = 0;   // learned ordering: frontier positions and the order table
  u64* dFrontP = nullptr;
  u64* dFrontO = nullptr;
  u64* dOrder = nullptr;
  int order_bits = 0;
  unsigned long long* dCounter = nullptr;
  unsigned* dHist = nullptr;    // 65 buckets
  unsigned* dCursor = nullptr;  // 65 bucket cursors
  DeviceStats* dStats = nullptr;
  unsigned char* dFrames = nullptr;  // batched kernel's global frame slots
  size_t frames_cap = 0;
  unsigned long long* dTable = nullptr;  // transposition table
  int table_bits = 0;
  size_t split_cap = 0;  // root split: frontier positions and their results
  u64* dSplitP = nullptr;
  u64* dSplitO = nullptr;
  signed char* dSplitScore = nullptr;
  signed char* dSplitBest = nullptr;
  unsigned long long* dSplitNodes = nullptr;
  signed char* dSplitWin = nullptr;  // frontier windows (alpha, beta)
  size_t bound_cap = 0;  // tail handoff: the roots' lower bounds
  signed char* dBound = nullptr;
  unsigned long long launches = 0;  // kernels launched since the context was made
};

std::mutex g_mutex;
Context* g_ctx[kMaxDevices] = {nullptr};

int cuda_fail(cudaError_t e, const char* what) {
  std::fprintf(stderr, "gpuothello2: %s: %s (%s)\n", what, cudaGetErrorName(e), cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? GPO_ERR_NOMEM : GPO_ERR_CUDA;
}

#define GPO_CK(call)                                 \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

int ensure_table(Context* c, int bits) {
  if (c->dTable && c->table_bits == bits) return GPO_OK;
  cudaFree(c->dTable);
  c->dTable = nullptr;
  c->table_bits = 0;
  GPO_CK(cudaMalloc(&c->dTable, (static_cast<size_t>(16)) << bits));
  c->table_bits = bits;
  return GPO_OK;
}

void free_buffers(Context* c) {
  cudaFree(c->dP);
  cudaFree(c->dO);
  cudaFree(c->dScore);
  cudaFree(c->dBest);
  cudaFree(c->dNodes);
  c->dP = c->dO = nullptr;
  c->dScore = c->dBest = nullptr;
  c->dNodes = nullptr;
  c->cap = 0;
}

void free_split(Context* c) {
  cudaFree(c->dSplitP);
  cudaFree(c->dSplitO);
  cudaFree(c->dSplitScore);
  cudaFree(c->dSplitBest);
  cudaFree(c->dSplitNodes);
  cudaFree(c->dSplitWin);
  c->dSplitP = c->dSplitO = nullptr;
  c->dSplitScore = c->dSplitBest = c->dSplitWin = nullptr;
  c->dSplitNodes = nullptr;
  c->split_cap = 0;
}

void free_context(Context* c) {
  cudaStreamSynchronize(c->stream);
  free_buffers(c);
  free_split(c);
  cudaFree(c->dBound);
  cudaFree(c->dPerm);
  cudaFree(c->dFrontP);
  cudaFree(c->dFrontO);
  cudaFree(c->dOrder);
  cudaFree(c->dCounter);
  cudaFree(c->dFrames);
  cudaFree(c->dTable);
  cudaFree(c->dHist);
  cudaFree(c->dCursor);
  cudaFree(c->dStats);
  cudaEventDestroy(c->ev0);
  cudaEventDestroy(c->ev1);
  cudaStreamDestroy(c->stream);
  delete c;
}

int ensure_context(Context** out) {
  int dev = 0;
  GPO_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return GPO_ERR_CUDA;
  if (!g_ctx[dev]) {
    cudaDeviceProp prop;
    GPO_CK(cudaGetDeviceProperties(&prop, dev));
    Context* c = new Context();
    c->device = dev;
    c->sms = prop.multiProcessorCount;
    c->mem = prop.totalGlobalMem;
    std::snprintf(c->name, sizeof(c->name), "%s", prop.name);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&c->dHist, 65 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&c->dCursor, 65 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&c->dStats, sizeof(DeviceStats));
    if (e == cudaSuccess) e = cudaMalloc(&c->dCounter, sizeof(unsigned long long));
    if (e != cudaSuccess) {
      free_context(c);
      return cuda_fail(e, "context setup");
    }
    g_ctx[dev] = c;
  }
  *out = g_ctx[dev];
  return GPO_OK;
}

int ensure_capacity(Context* c, size_t n) {
  if (n <= c->cap) return GPO_OK;
  free_buffers(c);
  size_t cap = 1024;
  while (cap < n) cap *= 2;
  GPO_CK(cudaMalloc(&c->dP, cap * sizeof(u64)));
  GPO_CK(cudaMalloc(&c->dO, cap * sizeof(u64)));
  GPO_CK(cudaMalloc(&c->dScore, cap));
  GPO_CK(cudaMalloc(&c->dBest, cap));
  GPO_CK(cudaMalloc(&c->dNodes, cap * sizeof(unsigned long long)));
  c->cap = cap;
  return GPO_OK;
}

// Frontier positions of a root split and their results, grown on demand;
// apart from the caller's arrays, so that a split can finish part of a
// batch whose outputs are still in use.
int ensure_split(Context* c, size_t n) {
  if (n <= c->split_cap) return GPO_OK;
  free_split(c);
  size_t cap = 1024;
  while (cap < n) cap *= 2;
  GPO_CK(cudaMalloc(&c->dSplitP, cap * sizeof(u64)));
  GPO_CK(cudaMalloc(&c->dSplitO, cap * sizeof(u64)));
  GPO_CK(cudaMalloc(&c->dSplitScore, cap));
  GPO_CK(cudaMalloc(&c->dSplitBest, cap));
  GPO_CK(cudaMalloc(&c->dSplitNodes, cap * sizeof(unsigned long long)));
  GPO_CK(cudaMalloc(&c->dSplitWin, 2 * cap));
  c->split_cap = cap;
  return GPO_OK;
}

int ensure_bound(Context* c, size_t n) {
  if (n <= c->bound_cap) return GPO_OK;
  cudaFree(c->dBound);
  c->dBound = nullptr;
  c->bound_cap = 0;
  size_t cap = 1024;
  while (cap < n) cap *= 2;
  GPO_CK(cudaMalloc(&c->dBound, cap));
  c->bound_cap = cap;
  return GPO_OK;
}

// Per-position scratch of a search (queue order), grown on demand and kept
// by the context: repeated calls of the same size allocate nothing.
int ensure_pass_scratch(Context* c, size_t n) {
  if (n <= c->pass_cap) return GPO_OK;
  cudaFree(c->dPerm);
  c->dPerm = nullptr;
  c->pass_cap = 0;
  size_t cap = 1024;
  while (cap < n) cap *= 2;
  GPO_CK(cudaMalloc(&c->dPerm, cap * sizeof(unsigned)));
  c->pass_cap = cap;
  return GPO_OK;
}

// Learned ordering: frontier positions (capacity cap) and an order table of
// at least twice as many entries, grown on demand.
int ensure_frontier(Context* c, long cap) {
  if (cap <= c->front_cap) return GPO_OK;
  cudaFree(c->dFrontP);
  cudaFree(c->dFrontO);
  cudaFree(c->dOrder);
  c->dFrontP = c->dFrontO = c->dOrder = nullptr;
  c->front_cap = 0;
  int bits = 10;
  while ((1L << bits) < 2 * cap) ++bits;
  GPO_CK(cudaMalloc(&c->dFrontP, cap * sizeof(u64)));
  GPO_CK(cudaMalloc(&c->dFrontO, cap * sizeof(u64)));
  GPO_CK(cudaMalloc(&c->dOrder, (static_cast<size_t>(32)) << bits));
  c->order_bits = bits;
  c->front_cap = cap;
  return GPO_OK;
}

// Frontier nodes reserved per deep root: a position with two plies of
// >= L empties below it has about 70 (1 + ~8 children + ~60 grandchildren);
// the rare larger ones past the capacity keep the fastest-first order.
constexpr long kFrontierPerRoot = 96;

int status_to_error(unsigned st) {
  if (st & kErrOverlap) return GPO_ERR_BOARD;
  if (st & kErrDepth) return GPO_ERR_DEPTH;
  if (st & (kErrBudget | kErrWait)) return GPO_ERR_TIMEOUT;
  if (st & (kErrInternal | kErrTable)) return GPO_ERR_INTERNAL;
  return GPO_OK;
}

int check_options(const gpo_options* opt) {
  if (!opt) return GPO_OK;
  if (opt->table_bits != 0 && (opt->table_bits < 17 || opt->table_bits > 32)) return GPO_ERR_ARG;
  if (opt->method != GPO_METHOD_BATCHED && opt->method != GPO_METHOD_PLAIN) return GPO_ERR_ARG;
  // the batched kernel is compiled for at most 256 threads per block
  if (opt->threads_per_block != 0 &&
      (opt->threads_per_block < 32 || opt->threads_per_block > 256 || opt->threads_per_block % 32))
    return GPO_ERR_ARG;
  if (opt->roots_per_warp < 0 || opt->roots_per_warp > 32) return GPO_ERR_ARG;
  if (opt->fastest_first_empties < 0 || opt->learned_min_empties < 0 || opt->wait_limit_ms < 0)
    return GPO_ERR_ARG;
  return GPO_OK;
}

// Defaults of the batched search (the autotuner can choose others per GPU):
// fastest-first from 6 empties, table from 9, the stability cutoff from 4
// empties when alpha >= 10 + 3 * empties, helping from 7.
constexpr int kDefaultFF = 6;
constexpr int kDefaultTableMin = 9;
// Table size: tens of thousands of searches run at once and share it, so
// it pays to give it real capacity: 2^28 entries (4 GiB) on a device with
// at least 64 GiB, else 2^24 (256 MiB).
constexpr int kDefaultTableBitsLarge = 28;
constexpr int kDefaultTableBitsSmall = 24;
int default_table_bits(const Context* c) {
  return c->mem >= (static_cast<size_t>(64) << 30) ? kDefaultTableBitsLarge : kDefaultTableBitsSmall;
}
constexpr int kDefaultStabMin = 4;
constexpr int kDefaultStabGate = 10;
constexpr int kDefaultHelpMin = 7;
constexpr unsigned long long kDefaultHardNodes = 1ULL << 23;
// Learned ordering at the top two plies' nodes with >= 12 empties (the
// network was trained on positions with 12-14 empties).
constexpr int kDefaultLearnedMin = 12;

int finish_tail(Context* c, const u64* dP, const u64* dO, int n, int depth, signed char* dScore,
                signed char* dBest, unsigned long long* dNodes, const gpo_options& o,
                cudaStream_t s, gpo_stats* stats, long warps, unsigned handed,
                const signed char* dBound);

// Tail handoff (batches of DEPTH >= 14): once the queue is used up and at
// most warps / kTailWarpsDiv positions are unfinished, the kernel hands them
// back and a root split finishes them over the whole GPU.
constexpr int kTailWarpsDiv = 16;

// Bucketing, learned orders and the persistent search, enqueued on s; waits
// for them and returns the status.  tail: the tail handoff is allowed (not
// for the searches of a root split's frontier); clear_table: the
// transposition table starts empty (a root split finishing a tail keeps the
// entries of the search it finishes: they are exact bounds of the same
// positions' subtrees); dWin: per-position root windows, or null.
int run_batched(Context* c, const u64* dP, const u64* dO, int n, int depth, signed char* dScore,
                signed char* dBest, unsigned long long* dNodes, const gpo_options& o,
                cudaStream_t s, gpo_stats* stats, bool tail, bool clear_table,
                const signed char* dWin) {
  const int rcs = ensure_pass_scratch(c, static_cast<size_t>(n));
  if (rcs != GPO_OK) return rcs;
  GPO_CK(cudaMemsetAsync(c->dStats, 0, sizeof(DeviceStats), s));
  GPO_CK(cudaMemsetAsync(c->dHist, 0, 65 * sizeof(unsigned), s));
  GPO_CK(launch_bucket(dP, dO, n, depth, c->dHist, c->dCursor, c->dPerm, c->dStats, c->sms, s));
  c->launches += 3;
  // Learned ordering for the positions with >= learned_min empties (the
  // front of the bucketed queue): the network scores the top two plies of
  // their trees ahead of the search (mlp_order_frontier).
  const int lmin = o.learned_min_empties > 0 ? o.learned_min_empties : kDefaultLearnedMin;
  const bool learned = (o.use_learned > 0 || (o.use_learned < 0 && mlp_loaded())) && depth >= lmin;
  long learned_count = 0, frontier = 0;
  if (learned) {
    if (!mlp_loaded()) return GPO_ERR_ARG;
    unsigned hist[65];
    GPO_CK(cudaMemcpyAsync(hist, c->dHist, sizeof(hist), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaStreamSynchronize(s));
    for (int e = lmin; e <= 64; ++e) learned_count += hist[e];
    if (learned_count > 0) {
      const int rcf = ensure_frontier(c, learned_count * kFrontierPerRoot);
      if (rcf != GPO_OK) return rcf;
      unsigned launched = 0;
      const int rcl = mlp_order_frontier(dP, dO, c->dPerm, learned_count, lmin, c->dFrontP,
                                         c->dFrontO, c->front_cap, c->dCounter, c->dOrder,
                                         c->order_bits, s, &launched, &frontier);
      c->launches += launched;
      if (rcl != GPO_OK) return rcl;
    }
  }
  BatchedArgs a = {};
  a.player = dP;
  a.opp = dO;
  a.perm = c->dPerm;
  a.n = n;
  a.depth = depth;
  a.score = dScore;
  a.best = dBest;
  a.nodes_out = dNodes;
  a.stats = c->dStats;
  a.ff = o.fastest_first_empties > 0 ? o.fastest_first_empties : kDefaultFF;
  a.stab_min = o.stability_min_empties > 0 ? o.stability_min_empties
                                           : (o.stability_min_empties < 0 ? 0 : kDefaultStabMin);
  a.stab_gate = kDefaultStabGate;
  a.help_min = o.help_min_empties > 0 ? o.help_min_empties
                                      : (o.help_min_empties < 0 ? 0 : kDefaultHelpMin);
  a.node_budget = o.node_budget;
  a.hard_nodes = o.hard_nodes > 0 ? static_cast<unsigned long long>(o.hard_nodes)
                                  : (o.hard_nodes < 0 ? 0ULL : kDefaultHardNodes);
  a.order_table = frontier > 0 ? c->dOrder : nullptr;
  a.order_bits = c->order_bits;
  a.learned_min = lmin;
  a.wait_limit_ns =
      static_cast<unsigned long long>(o.wait_limit_ms > 0 ? o.wait_limit_ms : 600000) * 1000000ULL;
  BatchedLaunch cfg;
  cfg.threads = o.threads_per_block > 0 ? o.threads_per_block : 128;
  GPO_CK(batched_plan(cfg.threads, depth, &a.smem_top));
  // all frame slots in shared memory or none: a cap below depth - 2 slots
  // (or a negative value) puts them in global memory
  if (o.smem_frames < 0 || (o.smem_frames > 0 && o.smem_frames < depth - 2)) a.smem_top = 2;
  cfg.grid = 0;
  size_t smem = 0;
  GPO_CK(batched_grid(cfg.threads, a.smem_top, c->sms, &cfg.grid, &smem));
  // Few positions: spread them over the warps so that each keeps helpers.
  const long warps = static_cast<long>(cfg.grid) * (cfg.threads / 32);
  if (o.roots_per_warp > 0) {
    a.roots_per_warp = o.roots_per_warp;
  } else {
    const long per = (n + warps - 1) / warps;
    a.roots_per_warp = static_cast<int>(per < 1 ? 1 : (per > 32 ? 32 : per));
  }
  if (tail && depth >= 14 && o.tail_split_positions >= 0) {
    const long cnt = o.tail_split_positions > 0 ? o.tail_split_positions : warps / kTailWarpsDiv;
    a.tail_count = static_cast<unsigned>(cnt < n ? cnt : n);
    if (a.tail_count > 0) {
      const int rcb = ensure_bound(c, static_cast<size_t>(n));
      if (rcb != GPO_OK) return rcb;
      a.tail_bound = c->dBound;
    }
  }
  a.root_window = dWin;
  const size_t need = batched_gframe_bytes(depth, a.smem_top,
                                           static_cast<size_t>(cfg.grid) * cfg.threads);
  if (need > c->frames_cap) {
    cudaFree(c->dFrames);
    c->dFrames = nullptr;
    c->frames_cap = 0;
    GPO_CK(cudaMalloc(&c->dFrames, need));
    c->frames_cap = need;
  }
  a.gframes = c->dFrames;
  if (o.use_table != 0) {
    const int bits = o.table_bits > 0 ? o.table_bits : default_table_bits(c);
    const int rct = ensure_table(c, bits);
    if (rct != GPO_OK) return rct;
    // cleared at every call: no result carries over from an earlier call
    if (clear_table) GPO_CK(cudaMemsetAsync(c->dTable, 0, static_cast<size_t>(16) << bits, s));
    a.tt = c->dTable;
    a.tt_bits = bits;
    a.tt_min = o.table_min_empties > 0 ? o.table_min_empties : kDefaultTableMin;
  }
  if (dNodes) GPO_CK(cudaMemsetAsync(dNodes, 0, static_cast<size_t>(n) * sizeof(u64), s));
  GPO_CK(cudaEventRecord(c->ev0, s));
  GPO_CK(launch_batched(a, cfg, c->sms, s));
  c->launches += 1;
  GPO_CK(cudaEventRecord(c->ev1, s));
  DeviceStats hs;
  GPO_CK(cudaMemcpyAsync(&hs, c->dStats, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->nodes = hs.nodes;
    stats->table_probes = hs.tt_probes;
    stats->table_hits = hs.tt_hits;
    stats->table_updates = hs.tt_updates;
    stats->learned_calls = static_cast<uint64_t>(frontier);
    stats->splits = hs.handouts;
    stats->stability_cuts = hs.stab_cuts;
    stats->table_bits = a.tt ? a.tt_bits : 0;
    stats->kernel_ms = ms;
  }
  const int rc = status_to_error(hs.status);
  if (rc != GPO_OK || hs.handed == 0) return rc;
  return finish_tail(c, dP, dO, n, depth, dScore, dBest, dNodes, o, s, stats, warps, hs.handed,
                     c->dBound);
}

// ---- small batches: split at the root ----
// A batch with fewer positions than a fraction of the GPU's warps leaves most
// of the GPU idle however well each warp searches.  Such a batch is expanded
// on the host a few plies deep (at most a few hundred positions, so this is
// bookkeeping, not search); every frontier position is solved exactly by the
// batched kernel in one launch, and the values are taken back up by negamax.
// Solving every frontier position with a full window does more work than
// principal-variation search would, but it spreads a deep position over
// thousands of lanes.

u64 host_mobility(u64 P, u64 O) {
  u64 moves = 0;
  const u64 empty = ~(P | O);
  const int dr[8] = {0, 0, 1, -1, 1, 1, -1, -1}, dc[8] = {1, -1, 0, 0, 1, -1, 1, -1};
  for (int sq = 0; sq < 64; ++sq) {
    if (!((empty >> sq) & 1)) continue;
    for (int d = 0; d < 8; ++d) {
      int r = sq / 8 + dr[d], c = sq % 8 + dc[d], run = 0;
      while (r >= 0 && r < 8 && c >= 0 && c < 8 && ((O >> (r * 8 + c)) & 1)) {
        r += dr[d];
        c += dc[d];
        ++run;
      }
      if (run && r >= 0 && r < 8 && c >= 0 && c < 8 && ((P >> (r * 8 + c)) & 1)) {
        moves |= 1ULL << sq;
        break;
      }
    }
  }
  return moves;
}

u64 host_flip(u64 P, u64 O, int sq) {
  u64 flips = 0;
  const int dr[8] = {0, 0, 1, -1, 1, 1, -1, -1}, dc[8] = {1, -1, 0, 0, 1, -1, 1, -1};
  for (int d = 0; d < 8; ++d) {
    u64 run = 0;
    int r = sq / 8 + dr[d], c = sq % 8 + dc[d];
    while (r >= 0 && r < 8 && c >= 0 && c < 8 && ((O >> (r * 8 + c)) & 1)) {
      run |= 1ULL << (r * 8 + c);
      r += dr[d];
      c += dc[d];
    }
    if (r >= 0 && r < 8 && c >= 0 && c < 8 && ((P >> (r * 8 + c)) & 1)) flips |= run;
  }
  return flips;
}

int host_final(u64 P, u64 O) {
  const int pc = __builtin_popcountll(P), oc = __builtin_popcountll(O);
  return pc == oc ? 0 : (pc > oc ? 64 - 2 * oc : 2 * pc - 64);
}

struct SplitNode {
  u64 P, O;
  int parent;  // -1 for an input position
  int move;    // move from the parent (GPO_MOVE_PASS for a pass)
  int first;   // children [first, first + count), or count = 0 with a value
  int count;
  int leaf;    // index in the GPU batch, or -1
  int value;   // exact value once known
  unsigned long long nodes;
};

// Positions per warp below which a batch is split at the root, and the
// frontier size (in warps) that is enough.
constexpr int kSplitBelowWarpsDiv = 8;

// Root split core: the positions hp / ho (valid, at most `depth` empties)
// are expanded on the host by at least min_plies and up to 3 plies
// (plies_opt > 0: exactly that many) until the frontier has enough positions
// for the GPU; the frontier is solved in one batched launch and the values go
// back up by negamax.  Results (score, best move, nodes) for each input in
// sc / bm / nds.
//
// lb (optional): a known lower bound L of each input's score (-65 = none).
// Only the frontier values that can decide a score >= L are then needed
// exactly: a frontier position an even number of plies below its root is
// searched with the window (L - 1, 64), one an odd number below with
// (-64, 1 - L).  A move whose subtree holds a value outside its window is
// worth at most L - 1 to the root, below the score; the move that makes the
// score has every value of its subtree inside the windows, so negamax over
// the fail-soft results still gives the exact score and a best move.
int split_solve(Context* c, const std::vector<u64>& hp, const std::vector<u64>& ho, int depth,
                const gpo_options& o, cudaStream_t s, long warps, int plies_opt, int min_plies,
                bool clear_table, const std::vector<int>* lb, std::vector<signed char>& sc,
                std::vector<signed char>& bm, std::vector<unsigned long long>& nds,
                gpo_stats* stats) {
  const int n = static_cast<int>(hp.size());
  std::vector<SplitNode> t;
  t.reserve(static_cast<size_t>(n) * 64);
  for (int i = 0; i < n; ++i) t.push_back(SplitNode{hp[i], ho[i], -1, kMoveNoneDev, 0, 0, -1, 0, 0});
  // expand ply by ply until the frontier has enough positions
  size_t lo = 0, hi = t.size();
  const int max_plies = plies_opt > 0 ? plies_opt : 3;
  for (int ply = 0; ply < max_plies; ++ply) {
    if (plies_opt <= 0 && ply >= min_plies &&
        static_cast<long>(hi - lo) * kSplitBelowWarpsDiv >= warps * 4)
      break;
    for (size_t k = lo; k < hi; ++k) {
      const u64 P = t[k].P, O = t[k].O;  // copies: push_back below may move t
      if (64 - __builtin_popcountll(P | O) <= 12) continue;  // small enough to solve whole
      u64 moves = host_mobility(P, O);
      const int first = static_cast<int>(t.size());
      if (moves) {
        int cnt = 0;
        while (moves) {
          const int sq = __builtin_ctzll(moves);
          moves &= moves - 1;
          const u64 f = host_flip(P, O, sq);
          t.push_back(SplitNode{O ^ f, P ^ f ^ (1ULL << sq), static_cast<int>(k), sq, 0, 0, -1, 0, 0});
          ++cnt;
        }
        t[k].first = first;
        t[k].count = cnt;
      } else if (host_mobility(O, P)) {
        t.push_back(SplitNode{O, P, static_cast<int>(k), kMovePassDev, 0, 0, -1, 0, 0});
        t[k].first = first;
        t[k].count = 1;
      } else {
        t[k].value = host_final(P, O);  // game over: count stays 0, no leaf
        t[k].leaf = -2;
      }
    }
    lo = hi;
    hi = t.size();
  }
  // frontier positions (no children, value unknown) go to the GPU
  std::vector<u64> lp, lo_;
  for (size_t k = 0; k < t.size(); ++k) {
    if (t[k].count == 0 && t[k].leaf != -2) {
      t[k].leaf = static_cast<int>(lp.size());
      lp.push_back(t[k].P);
      lo_.push_back(t[k].O);
    }
  }
  const int m = static_cast<int>(lp.size());
  std::vector<signed char> lsc(m), lbest(m, kMoveNoneDev);
  std::vector<unsigned long long> lnodes(m, 0);
  std::vector<signed char> win;
  if (lb) {
    win.resize(2 * static_cast<size_t>(m));
    for (size_t k = 0; k < t.size(); ++k) {
      if (t[k].leaf < 0) continue;
      int root = static_cast<int>(k), plies = 0;
      while (t[root].parent >= 0) {
        root = t[root].parent;
        ++plies;
      }
      const int L = (*lb)[root];
      int a = -64, b = 64;
      if (L > -63 && L <= 64) {
        if (plies & 1) {
          b = 1 - L;
        } else {
          a = L - 1;
        }
      }
      win[2 * t[k].leaf] = static_cast<signed char>(a);
      win[2 * t[k].leaf + 1] = static_cast<signed char>(b);
    }
  }
  gpo_stats inner;
  std::memset(&inner, 0, sizeof(inner));
  if (m > 0) {
    int rc = ensure_split(c, static_cast<size_t>(m));
    if (rc != GPO_OK) return rc;
    GPO_CK(cudaMemcpyAsync(c->dSplitP, lp.data(), m * sizeof(u64), cudaMemcpyHostToDevice, s));
    GPO_CK(cudaMemcpyAsync(c->dSplitO, lo_.data(), m * sizeof(u64), cudaMemcpyHostToDevice, s));
    if (lb) GPO_CK(cudaMemcpyAsync(c->dSplitWin, win.data(), 2 * m, cudaMemcpyHostToDevice, s));
    rc = run_batched(c, c->dSplitP, c->dSplitO, m, depth, c->dSplitScore, c->dSplitBest,
                     c->dSplitNodes, o, s, &inner, false, clear_table,
                     lb ? c->dSplitWin : nullptr);
    if (rc != GPO_OK) return rc;
    GPO_CK(cudaMemcpyAsync(lsc.data(), c->dSplitScore, m, cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaMemcpyAsync(lbest.data(), c->dSplitBest, m, cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaMemcpyAsync(lnodes.data(), c->dSplitNodes, m * sizeof(u64), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaStreamSynchronize(s));
  }
  // negamax from the deepest nodes up (children come after their parents)
  std::vector<int> bestmove(t.size(), kMoveNoneDev);
  for (size_t k = t.size(); k-- > 0;) {
    SplitNode& nd = t[k];
    nd.nodes += 1;
    if (nd.leaf >= 0) {
      nd.value = lsc[nd.leaf];
      nd.nodes = lnodes[nd.leaf];
      bestmove[k] = lbest[nd.leaf];  // used where an input position was not expanded
    } else if (nd.count > 0) {
      int best = -65;
      for (int j = nd.first; j < nd.first + nd.count; ++j) {
        nd.nodes += t[j].nodes;
        if (-t[j].value > best) {
          best = -t[j].value;
          bestmove[k] = t[j].move;
        }
      }
      nd.value = best;
    }
  }
  sc.resize(n);
  bm.resize(n);
  nds.resize(n);
  for (int i = 0; i < n; ++i) {
    sc[i] = static_cast<signed char>(t[i].value);
    bm[i] = static_cast<signed char>(bestmove[i]);
    nds[i] = t[i].nodes;
  }
  if (stats) {
    *stats = inner;
    stats->nodes = inner.nodes + (t.size() - static_cast<size_t>(m));
    stats->root_split_positions = static_cast<uint64_t>(m);
  }
  return GPO_OK;
}

// Small batches: the whole batch goes through the root split.  Returns 1
// without doing anything when an input must be rejected (the batched
// kernel then reports it).
int run_root_split(Context* c, const u64* dP, const u64* dO, int n, int depth, signed char* dScore,
                   signed char* dBest, unsigned long long* dNodes, const gpo_options& o,
                   cudaStream_t s, gpo_stats* stats, long warps, int plies_opt) {
  std::vector<u64> hp(n), ho(n);
  GPO_CK(cudaMemcpyAsync(hp.data(), dP, n * sizeof(u64), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaMemcpyAsync(ho.data(), dO, n * sizeof(u64), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  for (int i = 0; i < n; ++i)
    if ((hp[i] & ho[i]) || 64 - __builtin_popcountll(hp[i] | ho[i]) > depth) return 1;
  std::vector<signed char> sc, bm;
  std::vector<unsigned long long> nds;
  const int rc =
      split_solve(c, hp, ho, depth, o, s, warps, plies_opt, 0, true, nullptr, sc, bm, nds, stats);
  if (rc != GPO_OK) return rc;
  GPO_CK(cudaMemcpyAsync(dScore, sc.data(), n, cudaMemcpyHostToDevice, s));
  if (dBest) GPO_CK(cudaMemcpyAsync(dBest, bm.data(), n, cudaMemcpyHostToDevice, s));
  if (dNodes) GPO_CK(cudaMemcpyAsync(dNodes, nds.data(), n * sizeof(u64), cudaMemcpyHostToDevice, s));
  GPO_CK(cudaStreamSynchronize(s));
  return GPO_OK;
}

// Tail handoff: the `handed` positions the kernel gave back unsolved (score
// kUnsolvedDev) are finished by a root split with the table kept, and their
// results written into place.  Node counts add both searches.
int finish_tail(Context* c, const u64* dP, const u64* dO, int n, int depth, signed char* dScore,
                signed char* dBest, unsigned long long* dNodes, const gpo_options& o,
                cudaStream_t s, gpo_stats* stats, long warps, unsigned handed,
                const signed char* dBound) {
  std::vector<signed char> all(static_cast<size_t>(n));
  GPO_CK(cudaMemcpyAsync(all.data(), dScore, n, cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  std::vector<int> idx;
  for (int i = 0; i < n; ++i)
    if (all[i] == kUnsolvedDev) idx.push_back(i);
  if (idx.size() != handed) return GPO_ERR_INTERNAL;
  const size_t k = idx.size();
  std::vector<u64> hp(k), ho(k);
  std::vector<unsigned long long> first(k, 0);
  std::vector<signed char> bound(k, -65);
  for (size_t j = 0; j < k; ++j) {
    GPO_CK(cudaMemcpyAsync(&hp[j], dP + idx[j], sizeof(u64), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaMemcpyAsync(&ho[j], dO + idx[j], sizeof(u64), cudaMemcpyDeviceToHost, s));
    if (dNodes)
      GPO_CK(cudaMemcpyAsync(&first[j], dNodes + idx[j], sizeof(u64), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaMemcpyAsync(&bound[j], dBound + idx[j], 1, cudaMemcpyDeviceToHost, s));
  }
  GPO_CK(cudaStreamSynchronize(s));
  // the stopped searches' lower bounds narrow the frontier's windows
  const std::vector<int> lb(bound.begin(), bound.end());
  std::vector<signed char> sc, bm;
  std::vector<unsigned long long> nds;
  gpo_stats inner;
  std::memset(&inner, 0, sizeof(inner));
  // the handed-back positions are the slowest of the batch: at least two
  // plies, so that each spreads over thousands of lanes
  const int rc = split_solve(c, hp, ho, depth, o, s, warps, 0, 2, false, &lb, sc, bm, nds, &inner);
  if (rc != GPO_OK) return rc;
  for (size_t j = 0; j < k; ++j) {
    nds[j] += first[j];
    GPO_CK(cudaMemcpyAsync(dScore + idx[j], &sc[j], 1, cudaMemcpyHostToDevice, s));
    if (dBest) GPO_CK(cudaMemcpyAsync(dBest + idx[j], &bm[j], 1, cudaMemcpyHostToDevice, s));
    if (dNodes)
      GPO_CK(cudaMemcpyAsync(dNodes + idx[j], &nds[j], sizeof(u64), cudaMemcpyHostToDevice, s));
  }
  GPO_CK(cudaStreamSynchronize(s));
  if (stats) {
    stats->nodes += inner.nodes;
    stats->table_probes += inner.table_probes;
    stats->table_hits += inner.table_hits;
    stats->table_updates += inner.table_updates;
    stats->learned_calls += inner.learned_calls;
    stats->splits += inner.splits;
    stats->stability_cuts += inner.stability_cuts;
    stats->kernel_ms += inner.kernel_ms;
    stats->root_split_positions = inner.root_split_positions;
    stats->tail_positions = k;
  }
  return GPO_OK;
}

// Runs the solve pipeline on device arrays already in place.
int run_solve(Context* c, const u64* dP, const u64* dO, int n, int depth, signed char* dScore,
              signed char* dBest, unsigned long long* dNodes, const gpo_options* opt,
              gpo_stats* stats, cudaStream_t s) {
  gpo_options o;
  gpo_default_options(&o);
  if (opt) o = *opt;
  if (o.method == GPO_METHOD_PLAIN) {
    GPO_CK(cudaMemsetAsync(c->dStats, 0, sizeof(DeviceStats), s));
    GPO_CK(cudaEventRecord(c->ev0, s));
    const unsigned long long limit =
        static_cast<unsigned long long>(o.wait_limit_ms > 0 ? o.wait_limit_ms : 600000) * 1000000ULL;
    GPO_CK(launch_plain(dP, dO, n, depth, dScore, dNodes, c->dStats, limit, s));
    c->launches += 1;
    GPO_CK(cudaEventRecord(c->ev1, s));
    DeviceStats hs;
    GPO_CK(cudaMemcpyAsync(&hs, c->dStats, sizeof(hs), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaStreamSynchronize(s));
    if (stats) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c->ev0, c->ev1);
      stats->nodes = hs.nodes;
      stats->kernel_ms = ms;
    }
    return status_to_error(hs.status);
  }
  // a batch far too small to give every warp a position is split at the root
  if (o.root_split_plies >= 0 && depth >= 14) {
    int threads = o.threads_per_block > 0 ? o.threads_per_block : 128, top = 2, grid = 0;
    size_t smem = 0;
    GPO_CK(batched_plan(threads, depth, &top));
    GPO_CK(batched_grid(threads, top, c->sms, &grid, &smem));
    const long warps = static_cast<long>(grid) * (threads / 32);
    if (o.root_split_plies > 0 || static_cast<long>(n) * kSplitBelowWarpsDiv < warps) {
      const int rc = run_root_split(c, dP, dO, n, depth, dScore, dBest, dNodes, o, s, stats, warps,
                                    o.root_split_plies);
      if (rc != 1) return rc;  // 1: inputs the kernel must reject, solved unsplit below
    }
  }
  return run_batched(c, dP, dO, n, depth, dScore, dBest, dNodes, o, s, stats, true, true, nullptr);
}

// ---- CUDA graphs of a batched solve (repeated batches) ----
// The batched path without the learned ordering, the root split or the tail
// handoff is a fixed sequence of stream work: clear the counters, bucket,
// clear the table, search, copy the counters out.  For a caller that solves batch
// after batch in the same device arrays, that sequence is captured once into
// a CUDA graph and replayed: one graph launch instead of seven API calls
// and launches, and no host work between them.  The graph owns every buffer
// it touches, so solves through the other entry points (which may grow the
// context's buffers) never move memory under it.
struct GraphState {
  int device = -1;
  int n = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr;
  unsigned* perm = nullptr;
  unsigned* hist = nullptr;
  unsigned* cursor = nullptr;
  DeviceStats* stats = nullptr;
  DeviceStats* host_stats = nullptr;  // pinned: the replay's counters
  unsigned char* frames = nullptr;
  unsigned long long* table = nullptr;
  int table_bits = 0;
  int launches = 0;
};

void graph_free(GraphState* g) {
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->capture) cudaStreamDestroy(g->capture);
  cudaFree(g->perm);
  cudaFree(g->hist);
  cudaFree(g->cursor);
  cudaFree(g->stats);
  cudaFree(g->frames);
  cudaFree(g->table);
  cudaFreeHost(g->host_stats);
  delete g;
}

int graph_build(GraphState* g, const Context* c, const u64* dP, const u64* dO, int n, int depth,
                signed char* dScore, const gpo_options& o) {
  g->device = c->device;
  g->n = n;
  GPO_CK(cudaMalloc(&g->perm, static_cast<size_t>(n) * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&g->hist, 65 * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&g->cursor, 65 * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&g->stats, sizeof(DeviceStats)));
  GPO_CK(cudaMallocHost(&g->host_stats, sizeof(DeviceStats)));
  std::memset(g->host_stats, 0, sizeof(DeviceStats));
  BatchedArgs a = {};
  a.player = dP;
  a.opp = dO;
  a.perm = g->perm;
  a.n = n;
  a.depth = depth;
  a.score = dScore;
  a.stats = g->stats;
  a.ff = o.fastest_first_empties > 0 ? o.fastest_first_empties : kDefaultFF;
  a.stab_min = o.stability_min_empties > 0 ? o.stability_min_empties
                                           : (o.stability_min_empties < 0 ? 0 : kDefaultStabMin);
  a.stab_gate = kDefaultStabGate;
  a.help_min = o.help_min_empties > 0 ? o.help_min_empties
                                      : (o.help_min_empties < 0 ? 0 : kDefaultHelpMin);
  a.node_budget = o.node_budget;
  a.hard_nodes = o.hard_nodes > 0 ? static_cast<unsigned long long>(o.hard_nodes)
                                  : (o.hard_nodes < 0 ? 0ULL : kDefaultHardNodes);
  a.learned_min = 64;
  a.wait_limit_ns =
      static_cast<unsigned long long>(o.wait_limit_ms > 0 ? o.wait_limit_ms : 600000) * 1000000ULL;
  const int threads = o.threads_per_block > 0 ? o.threads_per_block : 128;
  GPO_CK(batched_plan(threads, depth, &a.smem_top));
  if (o.smem_frames < 0 || (o.smem_frames > 0 && o.smem_frames < depth - 2)) a.smem_top = 2;
  int grid = 0;
  size_t smem = 0;
  GPO_CK(batched_grid(threads, a.smem_top, c->sms, &grid, &smem));
  const long warps = static_cast<long>(grid) * (threads / 32);
  if (o.roots_per_warp > 0) {
    a.roots_per_warp = o.roots_per_warp;
  } else {
    const long per = (n + warps - 1) / warps;
    a.roots_per_warp = static_cast<int>(per < 1 ? 1 : (per > 32 ? 32 : per));
  }
  const size_t fbytes = batched_gframe_bytes(depth, a.smem_top, static_cast<size_t>(grid) * threads);
  if (fbytes) GPO_CK(cudaMalloc(&g->frames, fbytes));
  a.gframes = g->frames;
  if (o.use_table != 0) {
    g->table_bits = o.table_bits > 0 ? o.table_bits : default_table_bits(c);
    GPO_CK(cudaMalloc(&g->table, static_cast<size_t>(16) << g->table_bits));
    a.tt = g->table;
    a.tt_bits = g->table_bits;
    a.tt_min = o.table_min_empties > 0 ? o.table_min_empties : kDefaultTableMin;
  }
  GPO_CK(cudaStreamCreateWithFlags(&g->capture, cudaStreamNonBlocking));
  cudaStream_t s = g->capture;
  GPO_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaMemsetAsync(g->stats, 0, sizeof(DeviceStats), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(g->hist, 0, 65 * sizeof(unsigned), s);
  if (e == cudaSuccess) e = launch_bucket(dP, dO, n, depth, g->hist, g->cursor, g->perm, g->stats,
                                          c->sms, s);
  if (e == cudaSuccess && g->table)
    e = cudaMemsetAsync(g->table, 0, static_cast<size_t>(16) << g->table_bits, s);
  if (e == cudaSuccess) e = launch_batched_shape(a, grid, threads, smem, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g->host_stats, g->stats, sizeof(DeviceStats), cudaMemcpyDeviceToHost, s);
  cudaGraph_t graph = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
  g->graph = graph;
  if (e != cudaSuccess) return cuda_fail(e, "graph capture");
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
  GPO_CK(cudaGraphInstantiate(&g->exec, g->graph, 0));
  g->launches = 4;  // bucketing (3) and the search
  return GPO_OK;
}

int validate_call(const void* a, const void* b, const void* out, int n, int depth) {
  if (n < 0) return GPO_ERR_ARG;
  if (n > 0 && (!a || !b || !out)) return GPO_ERR_ARG;
  if (depth < 1 || depth > kMaxEmpties) return GPO_ERR_DEPTH;
  return GPO_OK;
}

}  // namespace
}  // namespace gpo

using namespace gpo;

extern "C" {

void gpo_default_options(gpo_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof(*opt));
  opt->method = GPO_METHOD_BATCHED;
  opt->use_table = -1;
  opt->use_learned = -1;
}

int solve_batch_ex(const uint64_t* player, const uint64_t* opp, int n, int depth, int8_t* score,
                   int8_t* best_move, uint64_t* nodes, const gpo_options* opt, gpo_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  int rc = validate_call(player, opp, score, n, depth);
  if (rc == GPO_OK) rc = check_options(opt);
  if (rc != GPO_OK) return rc;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (n == 0) return GPO_OK;
  std::lock_guard<std::mutex> lock(g_mutex);
  Context* c = nullptr;
  if ((rc = ensure_context(&c)) != GPO_OK) return rc;
  if ((rc = ensure_capacity(c, static_cast<size_t>(n))) != GPO_OK) return rc;
  const unsigned long long launches0 = c->launches;
  cudaStream_t s = c->stream;
  GPO_CK(cudaMemcpyAsync(c->dP, player, n * sizeof(u64), cudaMemcpyHostToDevice, s));
  GPO_CK(cudaMemcpyAsync(c->dO, opp, n * sizeof(u64), cudaMemcpyHostToDevice, s));
  rc = run_solve(c, c->dP, c->dO, n, depth, c->dScore, best_move ? c->dBest : nullptr,
                 nodes ? c->dNodes : nullptr, opt, stats, s);
  if (rc == GPO_ERR_CUDA || rc == GPO_ERR_NOMEM) return rc;
  GPO_CK(cudaMemcpyAsync(score, c->dScore, n, cudaMemcpyDeviceToHost, s));
  if (best_move) GPO_CK(cudaMemcpyAsync(best_move, c->dBest, n, cudaMemcpyDeviceToHost, s));
  if (nodes)
    GPO_CK(cudaMemcpyAsync(nodes, c->dNodes, n * sizeof(u64), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  if (stats) {
    stats->launches = c->launches - launches0;
    stats->total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int solve_batch(const uint64_t* player, const uint64_t* opp, int n, int depth, int8_t* score) {
  return solve_batch_ex(player, opp, n, depth, score, nullptr, nullptr, nullptr, nullptr);
}

int solve_batch_device(const uint64_t* d_player, const uint64_t* d_opp, int n, int depth,
                       int8_t* d_score, int8_t* d_best_move, uint64_t* d_nodes,
                       const gpo_options* opt, gpo_stats* stats, void* stream) {
  const auto t0 = std::chrono::steady_clock::now();
  int rc = validate_call(d_player, d_opp, d_score, n, depth);
  if (rc == GPO_OK) rc = check_options(opt);
  if (rc != GPO_OK) return rc;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (n == 0) return GPO_OK;
  std::lock_guard<std::mutex> lock(g_mutex);
  Context* c = nullptr;
  if ((rc = ensure_context(&c)) != GPO_OK) return rc;
  if ((rc = ensure_capacity(c, static_cast<size_t>(n))) != GPO_OK) return rc;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  const unsigned long long launches0 = c->launches;
  rc = run_solve(c, reinterpret_cast<const u64*>(d_player), reinterpret_cast<const u64*>(d_opp), n,
                 depth, reinterpret_cast<signed char*>(d_score),
                 reinterpret_cast<signed char*>(d_best_move),
                 reinterpret_cast<unsigned long long*>(d_nodes), opt, stats, s);
  if (stats) {
    stats->launches = c->launches - launches0;
    stats->total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int gpo_generate_device(uint64_t seed, uint64_t first, int n, int min_empties, int max_empties,
                        uint64_t* d_player, uint64_t* d_opp, void* stream) {
  if (n < 0 || (n > 0 && (!d_player || !d_opp))) return GPO_ERR_ARG;
  if (min_empties < 0 || max_empties > 60 || min_empties > max_empties) return GPO_ERR_ARG;
  if (seed >= (1ULL << 32)) return GPO_ERR_ARG;
  if (n == 0) return GPO_OK;
  std::lock_guard<std::mutex> lock(g_mutex);
  Context* c = nullptr;
  int rc = ensure_context(&c);
  if (rc != GPO_OK) return rc;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  GPO_CK(launch_generate(seed, first, n, min_empties, max_empties,
                         reinterpret_cast<u64*>(d_player), reinterpret_cast<u64*>(d_opp), s));
  GPO_CK(cudaStreamSynchronize(s));
  return GPO_OK;
}

int gpo_generate(uint64_t seed, uint64_t first, int n, int min_empties, int max_empties,
                 uint64_t* player, uint64_t* opp) {
  if (n < 0 || (n > 0 && (!player || !opp))) return GPO_ERR_ARG;
  if (min_empties < 0 || max_empties > 60 || min_empties > max_empties) return GPO_ERR_ARG;
  if (seed >= (1ULL << 32)) return GPO_ERR_ARG;
  if (n == 0) return GPO_OK;
  std::lock_guard<std::mutex> lock(g_mutex);
  Context* c = nullptr;
  int rc = ensure_context(&c);
  if (rc != GPO_OK) return rc;
  if ((rc = ensure_capacity(c, static_cast<size_t>(n))) != GPO_OK) return rc;
  cudaStream_t s = c->stream;
  GPO_CK(launch_generate(seed, first, n, min_empties, max_empties, c->dP, c->dO, s));
  GPO_CK(cudaMemcpyAsync(player, c->dP, n * sizeof(u64), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaMemcpyAsync(opp, c->dO, n * sizeof(u64), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  return GPO_OK;
}

void solve_shutdown(void) {
  std::lock_guard<std::mutex> lock(g_mutex);
  int cur = -1;
  cudaGetDevice(&cur);
  for (int d = 0; d < kMaxDevices; ++d) {
    if (!g_ctx[d]) continue;
    cudaSetDevice(d);
    free_context(g_ctx[d]);
    g_ctx[d] = nullptr;
  }
  if (cur >= 0) cudaSetDevice(cur);
}

int gpo_graph_create(const uint64_t* d_player, const uint64_t* d_opp, int n, int depth,
                     int8_t* d_score, const gpo_options* opt, gpo_graph** out) {
  if (!out) return GPO_ERR_ARG;
  *out = nullptr;
  int rc = validate_call(d_player, d_opp, d_score, n, depth);
  if (rc == GPO_OK) rc = check_options(opt);
  if (rc != GPO_OK) return rc;
  if (n == 0) return GPO_ERR_ARG;
  gpo_options o;
  gpo_default_options(&o);
  if (opt) o = *opt;
  if (o.method != GPO_METHOD_BATCHED || o.use_learned > 0) return GPO_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_mutex);
  Context* c = nullptr;
  if ((rc = ensure_context(&c)) != GPO_OK) return rc;
  GraphState* g = new GraphState();
  rc = graph_build(g, c, reinterpret_cast<const u64*>(d_player), reinterpret_cast<const u64*>(d_opp),
                   n, depth, reinterpret_cast<signed char*>(d_score), o);
  if (rc != GPO_OK) {
    graph_free(g);
    return rc;
  }
  *out = reinterpret_cast<gpo_graph*>(g);
  return GPO_OK;
}

int gpo_graph_launch(gpo_graph* graph, void* stream) {
  if (!graph) return GPO_ERR_ARG;
  GraphState* g = reinterpret_cast<GraphState*>(graph);
  int dev = -1;
  GPO_CK(cudaGetDevice(&dev));
  if (dev != g->device) return GPO_ERR_ARG;
  GPO_CK(cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)));
  return GPO_OK;
}

int gpo_graph_stats(gpo_graph* graph, gpo_stats* stats) {
  if (!graph || !stats) return GPO_ERR_ARG;
  const GraphState* g = reinterpret_cast<const GraphState*>(graph);
  const DeviceStats& hs = *g->host_stats;
  std::memset(stats, 0, sizeof(*stats));
  stats->nodes = hs.nodes;
  stats->table_probes = hs.tt_probes;
  stats->table_hits = hs.tt_hits;
  stats->table_updates = hs.tt_updates;
  stats->splits = hs.handouts;
  stats->stability_cuts = hs.stab_cuts;
  stats->table_bits = static_cast<uint64_t>(g->table_bits);
  stats->launches = static_cast<uint64_t>(g->launches);
  return status_to_error(hs.status);
}

void gpo_graph_destroy(gpo_graph* graph) {
  if (!graph) return;
  GraphState* g = reinterpret_cast<GraphState*>(graph);
  cudaStreamSynchronize(g->capture);
  graph_free(g);
}

const char* gpo_strerror(int status) {
  switch (status) {
    case GPO_OK: return "ok";
    case GPO_ERR_ARG: return "invalid argument";
    case GPO_ERR_DEPTH: return "depth out of range or a position has more empty squares than depth";
    case GPO_ERR_BOARD: return "a square is occupied by both sides";
    case GPO_ERR_CUDA: return "CUDA runtime error";
    case GPO_ERR_NOMEM: return "out of memory";
    case GPO_ERR_TIMEOUT: return "node budget or launch deadline exceeded";
    case GPO_ERR_INTERNAL: return "internal consistency check failed";
    case GPO_ERR_IO: return "file I/O error";
    default: return "unknown status";
  }
}

int gpo_device_info(char* name, int name_len, int* sm_count) {
  std::lock_guard<std::mutex> lock(g_mutex);
  Context* c = nullptr;
  const int rc = ensure_context(&c);
  if (rc != GPO_OK) return rc;
  if (name && name_len > 0) std::snprintf(name, static_cast<size_t>(name_len), "%s", c->name);
  if (sm_count) *sm_count = c->sms;
  return GPO_OK;
}

}  // extern "C"

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

struct Context {
  int device = -1;
  int sms = 0;
  char name[256] = {0};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  size_t cap = 0;
  u64* dP = nullptr;
  u64* dO = nullptr;
  signed char* dScore = nullptr;
  signed char* dBest = nullptr;
  unsigned long long* dNodes = nullptr;
  unsigned* dPerm = nullptr;
  unsigned* dHist = nullptr;    // 65 buckets
  // 65 bucket cursors during bucketing; between passes, [0] counts marked
  // positions and [1..3] the children sets of an expansion
  unsigned* dCursor = nullptr;
  DeviceStats* dStats = nullptr;
  unsigned char* dFrames = nullptr;  // batched kernel's global frame slots
  size_t frames_cap = 0;
  // work donation: mailboxes (33 per lane), queue records
  unsigned task_cap = 0;
  size_t mbox_cap = 0;
  unsigned* dMboxAcc = nullptr;
  unsigned* dMboxPend = nullptr;
  unsigned* dMboxCancel = nullptr;
  DonatedTask* dQueue = nullptr;
  unsigned* dReady = nullptr;
  unsigned* dConsumed = nullptr;
  unsigned* dPosTasks = nullptr;  // per position of a pass (capacity pass_cap)
  unsigned long long* dTable = nullptr;  // transposition table
  int table_bits = 0;
  u64* dLists = nullptr;  // learned root orders (capacity pass_cap)
  // dPerm, dPosTasks and dLists hold one entry per position of a search
  // pass; an expansion level can hold more positions than the call's input,
  // so they grow on their own capacity, checked by every pass.
  size_t pass_cap = 0;
  // second pass (hard positions)
  size_t second_cap = 0;
  unsigned* d2Idx = nullptr;
  u64* d2P = nullptr;
  u64* d2O = nullptr;
  signed char* d2Score = nullptr;
  signed char* d2Best = nullptr;
  unsigned long long* d2Nodes = nullptr;
  unsigned long long launches = 0;  // kernels launched since the context was made
};

constexpr unsigned kTaskCap = 1u << 20;  // queue records (a ring, reused within a call)

std::mutex g_mutex;
Context* g_ctx = nullptr;

int cuda_fail(cudaError_t e, const char* what) {
  std::fprintf(stderr, "gpuothello2: %s: %s (%s)\n", what, cudaGetErrorName(e), cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? GPO_ERR_NOMEM : GPO_ERR_CUDA;
}

#define GPO_CK(call)                                 \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

void free_donation(Context* c) {
  cudaFree(c->dMboxAcc);
  cudaFree(c->dMboxPend);
  cudaFree(c->dMboxCancel);
  cudaFree(c->dQueue);
  cudaFree(c->dReady);
  cudaFree(c->dConsumed);
  c->dConsumed = nullptr;
  c->dMboxAcc = c->dMboxPend = c->dMboxCancel = c->dReady = nullptr;
  c->dQueue = nullptr;
  c->task_cap = 0;
  c->mbox_cap = 0;
}

// Mailboxes for `lanes` grid threads and the record queue.
int ensure_donation(Context* c, size_t lanes) {
  const size_t mboxes = static_cast<size_t>(kMaxEmpties + 1) * lanes;
  if (c->task_cap == kTaskCap && c->mbox_cap >= mboxes) return GPO_OK;
  free_donation(c);
  GPO_CK(cudaMalloc(&c->dMboxAcc, mboxes * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&c->dMboxPend, mboxes * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&c->dMboxCancel, mboxes * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&c->dQueue, kTaskCap * sizeof(DonatedTask)));
  GPO_CK(cudaMalloc(&c->dReady, kTaskCap * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&c->dConsumed, kTaskCap * sizeof(unsigned)));
  c->task_cap = kTaskCap;
  c->mbox_cap = mboxes;
  return GPO_OK;
}

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
  free_donation(c);
  cudaFree(c->d2Idx);
  cudaFree(c->d2P);
  cudaFree(c->d2O);
  cudaFree(c->d2Score);
  cudaFree(c->d2Best);
  cudaFree(c->d2Nodes);
  c->d2Idx = nullptr;
  c->d2P = c->d2O = nullptr;
  c->d2Score = c->d2Best = nullptr;
  c->d2Nodes = nullptr;
  c->second_cap = 0;
  cudaFree(c->dPosTasks);
  c->dPosTasks = nullptr;
  cudaFree(c->dLists);
  c->dLists = nullptr;
  cudaFree(c->dFrames);
  c->dFrames = nullptr;
  c->frames_cap = 0;
  cudaFree(c->dP);
  cudaFree(c->dO);
  cudaFree(c->dScore);
  cudaFree(c->dBest);
  cudaFree(c->dNodes);
  cudaFree(c->dPerm);
  c->dP = c->dO = nullptr;
  c->dScore = c->dBest = nullptr;
  c->dNodes = nullptr;
  c->dPerm = nullptr;
  c->cap = 0;
  c->pass_cap = 0;
}

int ensure_context(Context** out) {
  if (!g_ctx) {
    int dev = 0;
    GPO_CK(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    GPO_CK(cudaGetDeviceProperties(&prop, dev));
    Context* c = new Context();
    c->device = dev;
    c->sms = prop.multiProcessorCount;
    std::snprintf(c->name, sizeof(c->name), "%s", prop.name);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&c->dHist, 65 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&c->dCursor, 65 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&c->dStats, sizeof(DeviceStats));
    if (e != cudaSuccess) {
      delete c;
      return cuda_fail(e, "context setup");
    }
    g_ctx = c;
  }
  *out = g_ctx;
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

// Per-position scratch of one search pass (queue order, outstanding
// subtrees, learned root orders) for n positions.  Called by every pass,
// after the previous pass has finished with the arrays.
int ensure_pass_scratch(Context* c, size_t n) {
  if (n <= c->pass_cap) return GPO_OK;
  cudaFree(c->dPerm);
  cudaFree(c->dPosTasks);
  cudaFree(c->dLists);
  c->dPerm = nullptr;
  c->dPosTasks = nullptr;
  c->dLists = nullptr;
  c->pass_cap = 0;
  size_t cap = 1024;
  while (cap < n) cap *= 2;
  GPO_CK(cudaMalloc(&c->dPerm, cap * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&c->dPosTasks, cap * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&c->dLists, cap * sizeof(u64)));
  c->pass_cap = cap;
  return GPO_OK;
}

int status_to_error(unsigned st) {
  if (st & kErrOverlap) return GPO_ERR_BOARD;
  if (st & kErrDepth) return GPO_ERR_DEPTH;
  if (st & (kErrBudget | kErrWait)) return GPO_ERR_TIMEOUT;
  if (st & (kErrInternal | kErrTable)) return GPO_ERR_INTERNAL;
  return GPO_OK;
}

int check_options(const gpo_options* opt) {
  if (!opt) return GPO_OK;
  if (opt->table_bits != 0 && (opt->table_bits < 16 || opt->table_bits > 31)) return GPO_ERR_ARG;
  if (opt->method != GPO_METHOD_BATCHED && opt->method != GPO_METHOD_PLAIN) return GPO_ERR_ARG;
  // the batched kernel is compiled for at most 256 threads per block
  if (opt->threads_per_block != 0 &&
      (opt->threads_per_block < 32 || opt->threads_per_block > 256 || opt->threads_per_block % 32))
    return GPO_ERR_ARG;
  return GPO_OK;
}

struct PassResult {
  DeviceStats hs = {};
  float ms = 0.f;  // search kernel time
  unsigned long long learned = 0;
};

struct PassConfig {
  unsigned long long budget;  // per-position node budget (0 = none)
  bool mark;                  // over budget: score -128 instead of an error
  bool split;                 // hand subtrees of hard positions to idle lanes
  bool clear_table;           // clear the transposition table first
  const signed char* alpha = nullptr;  // per-position search windows (null = full)
  const signed char* beta = nullptr;
};

// One batched pass over device arrays already in place: bucketing, learned
// root orders, the persistent search; waits for it and returns its status.
int run_pass(Context* c, const u64* dP, const u64* dO, int n, int depth, signed char* dScore,
             signed char* dBest, unsigned long long* dNodes, const gpo_options& o,
             const PassConfig& pc, cudaStream_t s, PassResult* pr) {
  const int rcs = ensure_pass_scratch(c, static_cast<size_t>(n));
  if (rcs != GPO_OK) return rcs;
  GPO_CK(cudaMemsetAsync(c->dStats, 0, sizeof(DeviceStats), s));
  GPO_CK(cudaMemsetAsync(c->dHist, 0, 65 * sizeof(unsigned), s));
  GPO_CK(launch_bucket(dP, dO, n, depth, c->dHist, c->dCursor, c->dPerm, c->dStats, c->sms, s));
  c->launches += 3;
  // Learned root orders for the positions with >= learned_min empties
  // (the front of the bucketed queue).
  const int lmin = o.learned_min_empties > 0 ? o.learned_min_empties : 14;
  const bool learned = (o.use_learned > 0 || (o.use_learned < 0 && mlp_loaded())) && depth >= lmin;
  long learned_count = 0;
  if (learned) {
    if (!mlp_loaded()) return GPO_ERR_ARG;
    unsigned hist[65];
    GPO_CK(cudaMemcpyAsync(hist, c->dHist, sizeof(hist), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaStreamSynchronize(s));
    for (int e = lmin; e <= 64; ++e) learned_count += hist[e];
    if (learned_count > 0) {
      unsigned launched = 0;
      const int rcl = mlp_order_roots(dP, dO, c->dPerm, learned_count, c->dLists, s, &launched);
      c->launches += launched;
      if (rcl != GPO_OK) return rcl;
      pr->learned = static_cast<unsigned long long>(learned_count);
    }
  }
  BatchedArgs a = {};
  a.player = dP;
  a.opp = dO;
  a.perm = c->dPerm;
  a.n = n;
  a.depth = depth;
  a.ff = o.fastest_first_empties > 0 ? o.fastest_first_empties : 9;
  a.score = dScore;
  a.best = dBest;
  a.nodes_out = dNodes;
  a.stats = c->dStats;
  a.node_budget = pc.budget;
  a.budget_mark = pc.mark ? 1 : 0;
  BatchedLaunch cfg;
  cfg.threads = o.threads_per_block > 0 ? o.threads_per_block : 128;
  GPO_CK(batched_plan(cfg.threads, depth, &a.smem_top));
  // slots 2..smem_top live in shared memory: a cap only lowers the tier
  if (o.smem_frames < 0)
    a.smem_top = 1;
  else if (o.smem_frames > 0 && a.smem_top > o.smem_frames + 1)
    a.smem_top = o.smem_frames + 1;
  cfg.grid = 0;
  size_t smem = 0;
  GPO_CK(batched_grid(cfg.threads, a.smem_top, c->sms, &cfg.grid, &smem));
  const size_t need = static_cast<size_t>(depth > a.smem_top ? depth - a.smem_top : 0) *
                      static_cast<size_t>(cfg.grid) * cfg.threads * 20;
  if (need > c->frames_cap) {
    cudaFree(c->dFrames);
    c->dFrames = nullptr;
    c->frames_cap = 0;
    GPO_CK(cudaMalloc(&c->dFrames, need));
    c->frames_cap = need;
  }
  a.gframes = c->dFrames;
  a.root_lists = learned_count > 0 ? c->dLists : nullptr;
  a.learned_min = lmin;
  if (pc.split) {
    const int rcd = ensure_donation(c, static_cast<size_t>(cfg.grid) * cfg.threads);
    if (rcd != GPO_OK) return rcd;
    a.donate_min = o.split_min_empties > 0 ? o.split_min_empties : 12;
    a.long_nodes = 1ULL << 21;
    a.pos_tasks = c->dPosTasks;
    // At most 32 handed-out subtrees per position: more lanes than that on
    // one position cost more in stale-window search than they save.
    a.max_tasks = 32;
    a.task_cap = c->task_cap;
    a.mbox_acc = c->dMboxAcc;
    a.mbox_pend = c->dMboxPend;
    a.mbox_cancel = c->dMboxCancel;
    a.queue = c->dQueue;
    a.ready = c->dReady;
    a.consumed = c->dConsumed;
    GPO_CK(cudaMemsetAsync(c->dPosTasks, 0, static_cast<size_t>(n) * sizeof(unsigned), s));
    GPO_CK(cudaMemsetAsync(c->dReady, 0, static_cast<size_t>(c->task_cap) * sizeof(unsigned), s));
    GPO_CK(cudaMemsetAsync(c->dConsumed, 0, static_cast<size_t>(c->task_cap) * sizeof(unsigned), s));
  }
  const bool table = o.use_table > 0;
  if (table) {
    const int bits = o.table_bits > 0 ? o.table_bits : 24;
    const int rct = ensure_table(c, bits);
    if (rct != GPO_OK) return rct;
    if (pc.clear_table) GPO_CK(cudaMemsetAsync(c->dTable, 0, static_cast<size_t>(16) << bits, s));
    a.tt = c->dTable;
    a.tt_bits = bits;
    a.tt_min = o.table_min_empties > 0 ? o.table_min_empties : 11;
  }
  a.root_alpha = pc.alpha;
  a.root_beta = pc.beta;
  a.wait_limit_ns =
      static_cast<unsigned long long>(o.wait_limit_ms > 0 ? o.wait_limit_ms : 600000) * 1000000ULL;
  if (dNodes) GPO_CK(cudaMemsetAsync(dNodes, 0, static_cast<size_t>(n) * sizeof(u64), s));
  GPO_CK(cudaEventRecord(c->ev0, s));
  GPO_CK(launch_batched(a, cfg, c->sms, s));
  c->launches += 1;
  GPO_CK(cudaEventRecord(c->ev1, s));
  GPO_CK(cudaMemcpyAsync(&pr->hs, c->dStats, sizeof(pr->hs), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  cudaEventElapsedTime(&pr->ms, c->ev0, c->ev1);
  return status_to_error(pr->hs.status);
}

int ensure_second(Context* c, size_t n) {
  if (n <= c->second_cap) return GPO_OK;
  cudaFree(c->d2Idx);
  cudaFree(c->d2P);
  cudaFree(c->d2O);
  cudaFree(c->d2Score);
  cudaFree(c->d2Best);
  cudaFree(c->d2Nodes);
  c->second_cap = 0;
  GPO_CK(cudaMalloc(&c->d2Idx, n * sizeof(unsigned)));
  GPO_CK(cudaMalloc(&c->d2P, n * sizeof(u64)));
  GPO_CK(cudaMalloc(&c->d2O, n * sizeof(u64)));
  GPO_CK(cudaMalloc(&c->d2Score, n));
  GPO_CK(cudaMalloc(&c->d2Best, n));
  GPO_CK(cudaMalloc(&c->d2Nodes, n * sizeof(u64)));
  c->second_cap = n;
  return GPO_OK;
}

// One level of the expansion: positions, their results, and (below the
// input level) their parent and move; with their search windows when the
// level is searched with windows (null = full window).
struct Level {
  const u64* P = nullptr;
  const u64* O = nullptr;
  const signed char* alpha = nullptr;
  const signed char* beta = nullptr;
  signed char* score = nullptr;
  signed char* best = nullptr;
  unsigned long long* nodes = nullptr;
  unsigned* parent = nullptr;
  unsigned char* move = nullptr;
  int n = 0;
  unsigned* idx = nullptr;  // marked (over budget) positions of this level
  int m = 0;
  unsigned* acc = nullptr;
  std::vector<void*> owned;
  ~Level() {
    for (void* p : owned) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T** p, size_t count) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), (count ? count : 1) * sizeof(T));
    if (e == cudaSuccess) owned.push_back(*p);
    return e;
  }
};

// Counters summed over every pass of a solve.
struct Totals {
  unsigned long long nodes = 0, probes = 0, hits = 0, updates = 0, learned = 0, splits = 0;
  double ms = 0.0;
  void add(const PassResult& r) {
    nodes += r.hs.nodes;
    probes += r.hs.tt_probes;
    hits += r.hs.tt_hits;
    updates += r.hs.tt_updates;
    learned += r.learned;
    ms += r.ms;
  }
  void write(gpo_stats* stats) const {
    if (!stats) return;
    stats->nodes = nodes;
    stats->table_probes = probes;
    stats->table_hits = hits;
    stats->table_updates = updates;
    stats->learned_calls = learned;
    stats->splits = splits;
    stats->kernel_ms = ms;
  }
};

constexpr int kExpandLevels = 6;
constexpr unsigned long long kLevelBudget = 1ULL << 22;

// Hard positions (over kLevelBudget nodes) are replaced by their children,
// solved as independent positions in the next pass (again with the budget,
// except in the last level); values combine bottom-up as the max of the
// children's negated scores.  No lane ever waits for another, and every
// child is an ordinary solve, so a hard position spreads over 10x, 100x,
// ... lanes without the stale-window cost of splitting a running search.
// With windows (dAlpha/dBeta), each position is searched with its window and
// a child inherits its parent's window negated and swapped; the max of the
// children's fail-soft values is then the parent's fail-soft value.
int run_expanded(Context* c, const u64* dP, const u64* dO, int n, const signed char* dAlpha,
                 const signed char* dBeta, int depth, signed char* dScore, signed char* dBest,
                 unsigned long long* dNodes, const gpo_options& o, bool clear_table, Totals* t,
                 cudaStream_t s) {
  if (n == 0) return GPO_OK;
  Level lv[kExpandLevels];
  lv[0].P = dP;
  lv[0].O = dO;
  lv[0].alpha = dAlpha;
  lv[0].beta = dBeta;
  lv[0].score = dScore;
  lv[0].best = dBest;
  lv[0].nodes = dNodes;
  lv[0].n = n;
  int rc = GPO_OK;
  int last = 0;
  for (int k = 0; k < kExpandLevels; ++k) {
    Level& L = lv[k];
    const bool final_level = k == kExpandLevels - 1;
    PassConfig pc;
    pc.budget = final_level ? 0 : (o.expand_budget > 0 ? o.expand_budget : kLevelBudget);
    pc.mark = !final_level;
    pc.split = false;
    pc.clear_table = clear_table && k == 0;
    pc.alpha = L.alpha;
    pc.beta = L.beta;
    PassResult r;
    rc = run_pass(c, L.P, L.O, L.n, depth, L.score, L.best, L.nodes, o, pc, s, &r);
    t->add(r);
    last = k;
    if (rc != GPO_OK || final_level) break;
    // over-budget positions of this level
    GPO_CK(L.alloc(&L.idx, static_cast<size_t>(L.n)));
    GPO_CK(launch_collect_marked(L.score, L.n, L.idx, c->dCursor, s));
    c->launches += 1;
    unsigned m = 0;
    GPO_CK(cudaMemcpyAsync(&m, c->dCursor, sizeof(m), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaStreamSynchronize(s));
    L.m = static_cast<int>(m);
    if (m == 0) break;
    // their children form the next level
    Level& C = lv[k + 1];
    const size_t cap = static_cast<size_t>(m) * 33;
    u64 *cP = nullptr, *cO = nullptr;
    signed char *ca = nullptr, *cb = nullptr;
    GPO_CK(C.alloc(&cP, cap));
    GPO_CK(C.alloc(&cO, cap));
    GPO_CK(C.alloc(&C.parent, cap));
    GPO_CK(C.alloc(&C.move, cap));
    GPO_CK(C.alloc(&C.score, cap));
    if (L.nodes) GPO_CK(C.alloc(&C.nodes, cap));
    if (L.alpha) {
      GPO_CK(C.alloc(&ca, cap));
      GPO_CK(C.alloc(&cb, cap));
    }
    GPO_CK(cudaMemsetAsync(c->dCursor + 1, 0, sizeof(unsigned), s));
    GPO_CK(launch_expand(L.P, L.O, L.idx, L.m, cP, cO, C.parent, C.move, c->dCursor + 1,
                         static_cast<unsigned>(cap), L.alpha, L.beta, ca, cb, s));
    c->launches += 1;
    unsigned cn = 0;
    GPO_CK(cudaMemcpyAsync(&cn, c->dCursor + 1, sizeof(cn), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaStreamSynchronize(s));
    if (cn > cap) return GPO_ERR_INTERNAL;
    C.P = cP;
    C.O = cO;
    C.alpha = ca;
    C.beta = cb;
    C.n = static_cast<int>(cn);
    t->splits += cn;
  }
  // combine from the deepest level up
  for (int k = last; k >= 1 && rc == GPO_OK; --k) {
    Level& C = lv[k];
    Level& L = lv[k - 1];
    GPO_CK(L.alloc(&L.acc, static_cast<size_t>(L.n)));
    GPO_CK(cudaMemsetAsync(L.acc, 0, static_cast<size_t>(L.n) * sizeof(unsigned), s));
    GPO_CK(launch_combine(C.score, C.parent, C.move, C.nodes, C.n, L.acc, L.nodes, s));
    GPO_CK(launch_finalize(L.idx, L.m, L.acc, L.score, L.best, s));
    c->launches += 2;
  }
  GPO_CK(cudaStreamSynchronize(s));
  return rc;
}

// Principal-variation-first expansion (expand_windows = 1).  The first pass
// is the default one; a hard position's children are then searched in the
// order alpha-beta would use: the first child in fastest-first order with
// a full window (A), which fixes a bound on the parent; the other children
// with a null window around that bound (B), which only tells whether each
// beats it; the children that do, again with the window above the bound
// (C).  Each set is solved by run_expanded, so a hard child is expanded in
// turn with its window.  The parent's value is the max over A, B and C of
// the negated values of A and C (C's are exact, and a B child outside C is
// worth no more than A's bound).
int run_pvs(Context* c, const u64* dP, const u64* dO, int n, int depth, signed char* dScore,
            signed char* dBest, unsigned long long* dNodes, const gpo_options& o, Totals* t,
            cudaStream_t s) {
  Level top;  // owns this function's buffers
  PassConfig pc;
  pc.budget = o.expand_budget > 0 ? o.expand_budget : kLevelBudget;
  pc.mark = true;
  pc.split = false;
  pc.clear_table = true;
  PassResult r;
  int rc = run_pass(c, dP, dO, n, depth, dScore, dBest, dNodes, o, pc, s, &r);
  t->add(r);
  if (rc != GPO_OK) return rc;
  unsigned* idx = nullptr;
  GPO_CK(top.alloc(&idx, static_cast<size_t>(n)));
  GPO_CK(launch_collect_marked(dScore, n, idx, c->dCursor, s));
  c->launches += 1;
  unsigned mu = 0;
  GPO_CK(cudaMemcpyAsync(&mu, c->dCursor, sizeof(mu), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  const int m = static_cast<int>(mu);
  if (m == 0) return GPO_OK;

  // A: one first child per marked position; B: the others
  const size_t capb = static_cast<size_t>(m) * 32;
  u64 *aP, *aO, *bP, *bO;
  unsigned *apar, *bpar;
  unsigned char *amov, *bmov;
  signed char *asc, *bsc, *bound, *ba, *bb;
  unsigned long long *anod = nullptr, *bnod = nullptr;
  GPO_CK(top.alloc(&aP, m));
  GPO_CK(top.alloc(&aO, m));
  GPO_CK(top.alloc(&apar, m));
  GPO_CK(top.alloc(&amov, m));
  GPO_CK(top.alloc(&asc, m));
  GPO_CK(top.alloc(&bP, capb));
  GPO_CK(top.alloc(&bO, capb));
  GPO_CK(top.alloc(&bpar, capb));
  GPO_CK(top.alloc(&bmov, capb));
  GPO_CK(top.alloc(&bsc, capb));
  GPO_CK(top.alloc(&ba, capb));
  GPO_CK(top.alloc(&bb, capb));
  GPO_CK(top.alloc(&bound, static_cast<size_t>(n)));
  if (dNodes) {
    GPO_CK(top.alloc(&anod, m));
    GPO_CK(top.alloc(&bnod, capb));
  }
  GPO_CK(cudaMemsetAsync(c->dCursor + 1, 0, sizeof(unsigned), s));
  GPO_CK(launch_expand_first(dP, dO, idx, m, aP, aO, apar, amov, bP, bO, bpar, bmov,
                             c->dCursor + 1, static_cast<unsigned>(capb), s));
  c->launches += 1;
  unsigned nbu = 0;
  GPO_CK(cudaMemcpyAsync(&nbu, c->dCursor + 1, sizeof(nbu), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  if (nbu > capb) return GPO_ERR_INTERNAL;
  const int nb = static_cast<int>(nbu);
  t->splits += static_cast<unsigned long long>(m) + nbu;

  rc = run_expanded(c, aP, aO, m, nullptr, nullptr, depth, asc, nullptr, anod, o, false, t, s);
  if (rc != GPO_OK) return rc;
  GPO_CK(launch_pvs_bound(asc, apar, m, bound, s));
  c->launches += 1;

  int nc = 0;
  u64 *cP = nullptr, *cO = nullptr;
  unsigned* cpar = nullptr;
  unsigned char* cmov = nullptr;
  signed char *csc = nullptr, *ca = nullptr, *cb = nullptr;
  unsigned long long* cnod = nullptr;
  if (nb > 0) {
    GPO_CK(launch_pvs_window(bpar, nb, bound, ba, bb, s));
    c->launches += 1;
    rc = run_expanded(c, bP, bO, nb, ba, bb, depth, bsc, nullptr, bnod, o, false, t, s);
    if (rc != GPO_OK) return rc;
    GPO_CK(top.alloc(&cP, nb));
    GPO_CK(top.alloc(&cO, nb));
    GPO_CK(top.alloc(&cpar, nb));
    GPO_CK(top.alloc(&cmov, nb));
    GPO_CK(top.alloc(&csc, nb));
    GPO_CK(top.alloc(&ca, nb));
    GPO_CK(top.alloc(&cb, nb));
    if (dNodes) GPO_CK(top.alloc(&cnod, nb));
    GPO_CK(cudaMemsetAsync(c->dCursor + 2, 0, sizeof(unsigned), s));
    GPO_CK(launch_pvs_research(bP, bO, bpar, bmov, bsc, nb, bound, cP, cO, cpar, cmov, ca, cb,
                               c->dCursor + 2, s));
    c->launches += 1;
    unsigned ncu = 0;
    GPO_CK(cudaMemcpyAsync(&ncu, c->dCursor + 2, sizeof(ncu), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaStreamSynchronize(s));
    nc = static_cast<int>(ncu);
    t->splits += ncu;
    rc = run_expanded(c, cP, cO, nc, ca, cb, depth, csc, nullptr, cnod, o, false, t, s);
    if (rc != GPO_OK) return rc;
  }

  // The parent's value and move come from A and C only: a B child that did
  // not beat the bound is worth at most the bound (its result is only a
  // bound, so its move must not win a tie), and one that did is in C with
  // its exact value.  B still adds its node counts (into a discarded max).
  unsigned *acc = nullptr, *acc_b = nullptr;
  GPO_CK(top.alloc(&acc, static_cast<size_t>(n)));
  GPO_CK(cudaMemsetAsync(acc, 0, static_cast<size_t>(n) * sizeof(unsigned), s));
  GPO_CK(launch_combine(asc, apar, amov, anod, m, acc, dNodes, s));
  c->launches += 1;
  if (nb > 0 && dNodes) {
    GPO_CK(top.alloc(&acc_b, static_cast<size_t>(n)));
    GPO_CK(launch_combine(bsc, bpar, bmov, bnod, nb, acc_b, dNodes, s));
    c->launches += 1;
  }
  if (nc > 0) {
    GPO_CK(launch_combine(csc, cpar, cmov, cnod, nc, acc, dNodes, s));
    c->launches += 1;
  }
  GPO_CK(launch_finalize(idx, m, acc, dScore, dBest, s));
  c->launches += 1;
  GPO_CK(cudaStreamSynchronize(s));
  return GPO_OK;
}

// Recursive principal-variation-first expansion (expand_windows = 2): every
// expanded position, at every level, searches its first child before its
// siblings.  A position (with its window) gets one budgeted pass; if it is
// marked, its first child is solved by this same function with the
// position's window negated and swapped, which gives a bound; a bound at or
// above beta cuts the position off (its siblings are never searched, as in
// alpha-beta at a cut node); otherwise the siblings get the null window
// above a' = max(alpha, bound), and when the position's window is wider than
// that (a PV-type node), the siblings that beat a' are searched again for
// their values.  Each of these sets recurses one level deeper; the last
// level is searched without a budget.  The position's fail-soft value is the
// max over its first child, the siblings (see pvs_siblings_kernel for which
// of them count) and the re-searched ones.
int run_pvs_rec(Context* c, const u64* dP, const u64* dO, int n, const signed char* dAlpha,
                const signed char* dBeta, int depth, signed char* dScore, signed char* dBest,
                unsigned long long* dNodes, const gpo_options& o, int level, bool clear_table,
                Totals* t, cudaStream_t s) {
  if (n == 0) return GPO_OK;
  const bool final_level = level >= kExpandLevels - 1;
  PassConfig pc;
  pc.budget = final_level ? 0 : (o.expand_budget > 0 ? o.expand_budget : kLevelBudget);
  pc.mark = !final_level;
  pc.split = false;
  pc.clear_table = clear_table;
  pc.alpha = dAlpha;
  pc.beta = dBeta;
  PassResult r;
  int rc = run_pass(c, dP, dO, n, depth, dScore, dBest, dNodes, o, pc, s, &r);
  t->add(r);
  if (rc != GPO_OK || final_level) return rc;

  Level mem;  // owns this level's buffers
  unsigned* idx = nullptr;
  GPO_CK(mem.alloc(&idx, static_cast<size_t>(n)));
  GPO_CK(launch_collect_marked(dScore, n, idx, c->dCursor, s));
  c->launches += 1;
  unsigned mu = 0;
  GPO_CK(cudaMemcpyAsync(&mu, c->dCursor, sizeof(mu), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  const int m = static_cast<int>(mu);
  if (m == 0) return GPO_OK;

  // first children (A, at the parent's slot) and their siblings (B)
  const size_t capb = static_cast<size_t>(m) * 32;
  u64 *aP, *aO, *bP, *bO;
  unsigned *apar, *bpar;
  unsigned char *amov, *bmov;
  signed char *asc, *bound, *aa = nullptr, *ab = nullptr;
  unsigned long long *anod = nullptr;
  GPO_CK(mem.alloc(&aP, m));
  GPO_CK(mem.alloc(&aO, m));
  GPO_CK(mem.alloc(&apar, m));
  GPO_CK(mem.alloc(&amov, m));
  GPO_CK(mem.alloc(&asc, m));
  GPO_CK(mem.alloc(&bP, capb));
  GPO_CK(mem.alloc(&bO, capb));
  GPO_CK(mem.alloc(&bpar, capb));
  GPO_CK(mem.alloc(&bmov, capb));
  GPO_CK(mem.alloc(&bound, static_cast<size_t>(n)));
  if (dNodes) GPO_CK(mem.alloc(&anod, m));
  GPO_CK(cudaMemsetAsync(c->dCursor + 1, 0, sizeof(unsigned), s));
  GPO_CK(launch_expand_first(dP, dO, idx, m, aP, aO, apar, amov, bP, bO, bpar, bmov,
                             c->dCursor + 1, static_cast<unsigned>(capb), s));
  c->launches += 1;
  unsigned nbu = 0;
  GPO_CK(cudaMemcpyAsync(&nbu, c->dCursor + 1, sizeof(nbu), cudaMemcpyDeviceToHost, s));
  GPO_CK(cudaStreamSynchronize(s));
  if (nbu > capb) return GPO_ERR_INTERNAL;
  const int nb = static_cast<int>(nbu);
  t->splits += static_cast<unsigned long long>(m);
  if (dAlpha) {
    GPO_CK(mem.alloc(&aa, m));
    GPO_CK(mem.alloc(&ab, m));
    GPO_CK(launch_child_window(apar, m, dAlpha, dBeta, aa, ab, s));
    c->launches += 1;
  }
  rc = run_pvs_rec(c, aP, aO, m, aa, ab, depth, asc, nullptr, anod, o, level + 1, false, t, s);
  if (rc != GPO_OK) return rc;
  GPO_CK(launch_pvs_bound(asc, apar, m, bound, s));
  c->launches += 1;

  // siblings with null windows, then the re-searches
  int ns = 0, nc = 0;
  u64 *sP = nullptr, *sO = nullptr, *cP = nullptr, *cO = nullptr;
  unsigned *spar = nullptr, *cpar = nullptr;
  unsigned char *smov = nullptr, *sflag = nullptr, *sskip = nullptr, *cmov = nullptr;
  signed char *ssc = nullptr, *sa = nullptr, *sb = nullptr, *csc = nullptr, *ca = nullptr,
              *cb = nullptr;
  unsigned long long *snod = nullptr, *cnod = nullptr;
  if (nb > 0) {
    GPO_CK(mem.alloc(&sP, nb));
    GPO_CK(mem.alloc(&sO, nb));
    GPO_CK(mem.alloc(&spar, nb));
    GPO_CK(mem.alloc(&smov, nb));
    GPO_CK(mem.alloc(&ssc, nb));
    GPO_CK(mem.alloc(&sa, nb));
    GPO_CK(mem.alloc(&sb, nb));
    GPO_CK(mem.alloc(&sflag, nb));
    GPO_CK(mem.alloc(&sskip, nb));
    if (dNodes) GPO_CK(mem.alloc(&snod, nb));
    GPO_CK(cudaMemsetAsync(c->dCursor + 2, 0, sizeof(unsigned), s));
    GPO_CK(launch_pvs_siblings(bP, bO, bpar, bmov, nb, dAlpha, dBeta, bound, sP, sO, spar, smov,
                               sa, sb, sflag, sskip, c->dCursor + 2, s));
    c->launches += 1;
    unsigned nsu = 0;
    GPO_CK(cudaMemcpyAsync(&nsu, c->dCursor + 2, sizeof(nsu), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaStreamSynchronize(s));
    ns = static_cast<int>(nsu);
    t->splits += nsu;
    rc = run_pvs_rec(c, sP, sO, ns, sa, sb, depth, ssc, nullptr, snod, o, level + 1, false, t, s);
    if (rc != GPO_OK) return rc;
    if (ns > 0) {
      GPO_CK(mem.alloc(&cP, ns));
      GPO_CK(mem.alloc(&cO, ns));
      GPO_CK(mem.alloc(&cpar, ns));
      GPO_CK(mem.alloc(&cmov, ns));
      GPO_CK(mem.alloc(&csc, ns));
      GPO_CK(mem.alloc(&ca, ns));
      GPO_CK(mem.alloc(&cb, ns));
      if (dNodes) GPO_CK(mem.alloc(&cnod, ns));
      GPO_CK(cudaMemsetAsync(c->dCursor + 3, 0, sizeof(unsigned), s));
      GPO_CK(launch_pvs_research2(sP, sO, spar, smov, ssc, sflag, ns, dAlpha, dBeta, bound, cP, cO,
                                  cpar, cmov, ca, cb, c->dCursor + 3, s));
      c->launches += 1;
      unsigned ncu = 0;
      GPO_CK(cudaMemcpyAsync(&ncu, c->dCursor + 3, sizeof(ncu), cudaMemcpyDeviceToHost, s));
      GPO_CK(cudaStreamSynchronize(s));
      nc = static_cast<int>(ncu);
      t->splits += ncu;
      rc = run_pvs_rec(c, cP, cO, nc, ca, cb, depth, csc, nullptr, cnod, o, level + 1, false, t,
                       s);
      if (rc != GPO_OK) return rc;
    }
  }

  unsigned* acc = nullptr;
  GPO_CK(mem.alloc(&acc, static_cast<size_t>(n)));
  GPO_CK(cudaMemsetAsync(acc, 0, static_cast<size_t>(n) * sizeof(unsigned), s));
  GPO_CK(launch_combine(asc, apar, amov, anod, m, acc, dNodes, s));
  c->launches += 1;
  if (ns > 0) {
    GPO_CK(launch_combine_masked(ssc, spar, smov, snod, sskip, ns, acc, dNodes, s));
    c->launches += 1;
  }
  if (nc > 0) {
    GPO_CK(launch_combine(csc, cpar, cmov, cnod, nc, acc, dNodes, s));
    c->launches += 1;
  }
  GPO_CK(launch_finalize(idx, m, acc, dScore, dBest, s));
  c->launches += 1;
  GPO_CK(cudaStreamSynchronize(s));
  return GPO_OK;
}

// Runs the solve pipeline on device arrays already in place.  Batched
// method: a first pass gives every position a node budget; the few hard
// positions that exceed it are solved again in a second pass in which idle
// lanes split them (their first-pass search is discarded, the table keeps
// what it learned).  With a caller node budget, or splitting off, one pass.
int run_solve(Context* c, const u64* dP, const u64* dO, int n, int depth, signed char* dScore,
              signed char* dBest, unsigned long long* dNodes, const gpo_options* opt,
              gpo_stats* stats, cudaStream_t s) {
  gpo_options o;
  gpo_default_options(&o);
  if (opt) o = *opt;
  if (o.method == GPO_METHOD_PLAIN) {
    GPO_CK(cudaMemsetAsync(c->dStats, 0, sizeof(DeviceStats), s));
    GPO_CK(cudaEventRecord(c->ev0, s));
    GPO_CK(launch_plain(dP, dO, n, depth, dScore, dNodes, c->dStats, s));
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
  // split_min_empties: 0 (default) = expand hard positions into their
  // children level by level; > 0 = hand subtrees of hard positions to idle
  // lanes inside the kernel (second pass); < 0 = one pass, no splitting.
  if (o.split_min_empties == 0 && o.node_budget == 0) {
    Totals t;
    int rc;
    if (o.expand_windows >= 2)
      rc = run_pvs_rec(c, dP, dO, n, nullptr, nullptr, depth, dScore, dBest, dNodes, o, 0, true,
                       &t, s);
    else if (o.expand_windows == 1)
      rc = run_pvs(c, dP, dO, n, depth, dScore, dBest, dNodes, o, &t, s);
    else
      rc = run_expanded(c, dP, dO, n, nullptr, nullptr, depth, dScore, dBest, dNodes, o, true, &t,
                        s);
    t.write(stats);
    return rc;
  }
  const bool split = o.split_min_empties > 0;
  const bool two_pass = split && o.node_budget == 0;
  PassConfig p1;
  p1.budget = two_pass ? (1ULL << 22) : o.node_budget;
  p1.mark = two_pass;
  p1.split = split && !two_pass;
  p1.clear_table = true;
  PassResult r1;
  int rc = run_pass(c, dP, dO, n, depth, dScore, dBest, dNodes, o, p1, s, &r1);
  PassResult r2;
  if (rc == GPO_OK && two_pass) {
    unsigned count = 0;
    GPO_CK(ensure_second(c, static_cast<size_t>(n)) == GPO_OK ? cudaSuccess : cudaErrorMemoryAllocation);
    GPO_CK(launch_collect_marked(dScore, n, c->d2Idx, c->dCursor, s));
    c->launches += 1;
    GPO_CK(cudaMemcpyAsync(&count, c->dCursor, sizeof(count), cudaMemcpyDeviceToHost, s));
    GPO_CK(cudaStreamSynchronize(s));
    if (count > 0) {
      const int m = static_cast<int>(count);
      GPO_CK(launch_gather(dP, dO, c->d2Idx, m, c->d2P, c->d2O, s));
      c->launches += 1;
      PassConfig p2;
      p2.budget = 0;
      p2.mark = false;
      p2.split = true;
      p2.clear_table = false;
      rc = run_pass(c, c->d2P, c->d2O, m, depth, c->d2Score, dBest ? c->d2Best : nullptr,
                    dNodes ? c->d2Nodes : nullptr, o, p2, s, &r2);
      if (rc == GPO_OK || rc == GPO_ERR_TIMEOUT) {
        GPO_CK(launch_scatter_scores(c->d2Score, c->d2Best, c->d2Nodes, c->d2Idx, m, dScore,
                                     dBest, dNodes, s));
        c->launches += 1;
        GPO_CK(cudaStreamSynchronize(s));
      }
    }
  }
  if (stats) {
    stats->nodes = r1.hs.nodes + r2.hs.nodes;
    stats->table_probes = r1.hs.tt_probes + r2.hs.tt_probes;
    stats->table_hits = r1.hs.tt_hits + r2.hs.tt_hits;
    stats->table_updates = r1.hs.tt_updates + r2.hs.tt_updates;
    stats->learned_calls = r1.learned + r2.learned;
    stats->splits = r1.hs.donations + r2.hs.donations;
    stats->kernel_ms = r1.ms + r2.ms;
  }
  return rc;
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
  if (!g_ctx) return;
  Context* c = g_ctx;
  cudaStreamSynchronize(c->stream);
  free_buffers(c);
  cudaFree(c->dTable);
  cudaFree(c->dHist);
  cudaFree(c->dCursor);
  cudaFree(c->dStats);
  cudaEventDestroy(c->ev0);
  cudaEventDestroy(c->ev1);
  cudaStreamDestroy(c->stream);
  delete c;
  g_ctx = nullptr;
}

const char* gpo_strerror(int status) {
  switch (status) {
    case GPO_OK: return "ok";
    case GPO_ERR_ARG: return "invalid argument";
    case GPO_ERR_DEPTH: return "depth out of range or a position has more empty squares than depth";
    case GPO_ERR_BOARD: return "a square is occupied by both sides";
    case GPO_ERR_CUDA: return "CUDA runtime error";
    case GPO_ERR_NOMEM: return "out of memory";
    case GPO_ERR_TIMEOUT: return "node budget or wait limit exceeded";
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

// The batched search kernel's own source (gpuothello2_gb300/csrc/batched.cu)
// run on the CPU under the SIMT emulation of tests/simt/simt_prelude.h (test
// infrastructure only; the product never links this file).
//
// emu_batched() runs batched_kernel as one block of `warps` x 32 CPU threads
// over n positions, with the buffers the C-ABI layer would give it: the
// empties-descending queue order, the frame tiers, the donation mailboxes
// and record ring, the transposition table and learned root lists.  Tests
// compare its scores with the oracle and exercise the code paths a GPU run
// takes (in-kernel donation across warps, the table, node budgets).
#include <algorithm>
#include <memory>
#include <numeric>
#include <thread>
#include <vector>

#include "../gpuothello2_gb300/csrc/batched.cu"

thread_local simt_uint3 threadIdx, blockIdx;
simt_uint3 blockDim, gridDim;
thread_local SimtWarp* simt_warp = nullptr;
SimtBarrier* simt_block = nullptr;
std::mutex simt_cas128_mutex;

namespace gpo {
// dynamic shared memory of the one emulated block: the ray table and up to
// 31 frame slots of 20 bytes for 128 threads
constexpr size_t kEmuSmemWords = (kRayBytes + 128 * 31 * kFrameBytes) / 8 + 8;
alignas(16) u64 smem_raw[kEmuSmemWords];
}  // namespace gpo

extern "C" {

struct EmuOptions {
  int warps;                        // 1..4
  int ff;                           // fastest-first threshold (0 = 9)
  int smem_slots;                   // frame slots in shared memory (0 = none)
  int donate_min;                   // in-kernel donation from nodes with this many empties (0 = off)
  unsigned long long long_nodes;    // root size after which it hands out moves unasked
  unsigned max_tasks;               // outstanding subtrees per position
  unsigned long long node_budget;   // per position, 0 = none
  int budget_mark;                  // over budget: score -128 instead of an error
  int tt_bits;                      // 0 = no table
  int tt_min;
  const unsigned long long* root_lists;  // learned root orders per position, or null
  int learned_min;
};

// stats: nodes, table probes, hits, updates, donations, cancels, status
int emu_batched(const unsigned long long* P, const unsigned long long* O, int n, int depth,
                const EmuOptions* opt, signed char* score, signed char* best,
                unsigned long long* nodes, unsigned long long* stats) {
  using namespace gpo;
  const int warps = opt->warps;
  if (warps < 1 || warps > 4 || n < 0 || depth < 1 || depth > kMaxEmpties) return -1;
  const int T = warps * 32;
  std::vector<unsigned> perm(static_cast<size_t>(n));
  std::iota(perm.begin(), perm.end(), 0u);
  std::stable_sort(perm.begin(), perm.end(), [&](unsigned a, unsigned b) {
    return __builtin_popcountll(P[a] | O[a]) < __builtin_popcountll(P[b] | O[b]);
  });
  BatchedArgs a = {};
  a.player = P;
  a.opp = O;
  a.perm = perm.data();
  a.n = n;
  a.depth = depth;
  a.ff = opt->ff > 0 ? opt->ff : 9;
  a.score = score;
  a.best = best;
  a.nodes_out = nodes;
  DeviceStats st = {};
  a.stats = &st;
  a.node_budget = opt->node_budget;
  a.budget_mark = opt->budget_mark;
  int top = opt->smem_slots > 0 ? opt->smem_slots + 1 : 1;
  if (top > depth) top = depth;
  if (top > 32) top = 32;
  a.smem_top = top;
  const size_t gslots = static_cast<size_t>(depth > top ? depth - top : 0);
  std::vector<u64> gframes((gslots * kFrameBytes * T) / 8 + 1);
  a.gframes = reinterpret_cast<unsigned char*>(gframes.data());
  const size_t mboxes = static_cast<size_t>(kMaxEmpties + 1) * T;
  std::vector<unsigned> acc(mboxes), pend(mboxes), cancel(mboxes), pos_tasks(n + 1);
  const unsigned task_cap = 4096;
  std::vector<DonatedTask> queue(task_cap);
  std::vector<unsigned> ready(task_cap), consumed(task_cap);
  if (opt->donate_min > 0) {
    a.donate_min = opt->donate_min;
    a.long_nodes = opt->long_nodes ? opt->long_nodes : (1ULL << 21);
    a.pos_tasks = pos_tasks.data();
    a.max_tasks = opt->max_tasks ? opt->max_tasks : 32;
    a.task_cap = task_cap;
    a.mbox_acc = acc.data();
    a.mbox_pend = pend.data();
    a.mbox_cancel = cancel.data();
    a.queue = queue.data();
    a.ready = ready.data();
    a.consumed = consumed.data();
  }
  std::vector<u64> table;
  if (opt->tt_bits > 0) {
    table.assign(static_cast<size_t>(2) << opt->tt_bits, 0);
    a.tt = table.data();
    a.tt_bits = opt->tt_bits;
    a.tt_min = opt->tt_min > 0 ? opt->tt_min : 11;
  }
  a.root_lists = opt->root_lists;
  a.learned_min = opt->learned_min > 0 ? opt->learned_min : 14;
  a.wait_limit_ns = 600ULL * 1000000000ULL;
  const size_t smem = kRayBytes + static_cast<size_t>(T) * (top >= 2 ? top - 1 : 0) * kFrameBytes;
  if (smem > sizeof(smem_raw)) return -1;

  blockDim = {static_cast<unsigned>(T), 1, 1};
  gridDim = {1, 1, 1};
  SimtBarrier block(T);
  simt_block = &block;
  std::vector<std::unique_ptr<SimtBarrier>> bars;
  std::vector<SimtWarp> ws(warps);
  for (int w = 0; w < warps; ++w) {
    bars.emplace_back(new SimtBarrier(32));
    ws[w].bar = bars.back().get();
  }
  std::vector<std::thread> threads;
  for (int t = 0; t < T; ++t) {
    threads.emplace_back([&, t] {
      threadIdx = {static_cast<unsigned>(t), 0, 0};
      blockIdx = {0, 0, 0};
      simt_warp = &ws[t / 32];
      batched_kernel(a);
    });
  }
  for (auto& th : threads) th.join();
  stats[0] = st.nodes;
  stats[1] = st.tt_probes;
  stats[2] = st.tt_hits;
  stats[3] = st.tt_updates;
  stats[4] = st.donations;
  stats[5] = st.cancels;
  stats[6] = st.status;
  return 0;
}

}  // extern "C"

// The batched search kernel's own source (gpuothello2_gb300/csrc/batched.cu)
// run on the CPU under the SIMT emulation of tests/simt/simt_prelude.h (test
// infrastructure only; the product never links this file).
//
// emu_batched() runs batched_kernel as one block of `warps` x 32 CPU threads
// over n positions, with the buffers the C-ABI layer would give it: the
// empties-descending queue order, the frame placements, the transposition
// table and a learned order table.  Tests compare its scores with the oracle
// and exercise the code paths a GPU run takes (helping between the lanes
// of a warp, the table, the stability cutoff, node budgets).
#include <algorithm>
#include <memory>
#include <numeric>
#include <thread>
#include <vector>

#include "batched_emu.cu"

thread_local simt_uint3 threadIdx, blockIdx;
simt_uint3 blockDim, gridDim;
thread_local SimtWarp* simt_warp = nullptr;
SimtBarrier* simt_block = nullptr;
std::mutex simt_cas128_mutex;

namespace gpo {
// dynamic shared memory of the one emulated block: the ray table, the
// split-node state and up to 30 frame slots for 128 threads
constexpr size_t kEmuSmemWords = (kTableBytes + 128 * (kSplitBytes + 30 * kFrameBytes)) / 8 + 8;
alignas(16) u64 smem_raw[kEmuSmemWords];
}  // namespace gpo

extern "C" {

struct EmuOptions {
  int warps;                        // 1..4
  int ff;                           // fastest-first threshold (0 = 6)
  int shared_frames;                // 1: frame slots in shared memory, 0: in the global array
  int help_min;                     // helping from nodes with this many empties (0 = off)
  int roots_per_warp;               // input positions per warp (0 = 32)
  int stab_min;                     // stability cutoff (0 = off)
  int stab_gate;
  unsigned long long node_budget;   // per position, 0 = none
  int tt_bits;                      // 0 = no table
  int tt_min;
  const unsigned long long* order_table;  // learned order table, or null
  int order_bits;
  int learned_min;
};

// stats: nodes, table probes, hits, updates, handouts, stability cuts, status
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
  a.ff = opt->ff > 0 ? opt->ff : 6;
  a.score = score;
  a.best = best;
  a.nodes_out = nodes;
  DeviceStats st = {};
  a.stats = &st;
  a.node_budget = opt->node_budget;
  a.help_min = opt->help_min;
  a.roots_per_warp = opt->roots_per_warp > 0 ? opt->roots_per_warp : 32;
  a.stab_min = opt->stab_min;
  a.stab_gate = opt->stab_gate;
  a.smem_top = opt->shared_frames ? depth : 2;
  std::vector<u64> gframes(batched_gframe_bytes(depth, a.smem_top, static_cast<size_t>(T)) / 8 + 1);
  a.gframes = reinterpret_cast<unsigned char*>(gframes.data());
  std::vector<u64> table;
  if (opt->tt_bits > 0) {
    table.assign(static_cast<size_t>(2) << opt->tt_bits, 0);
    a.tt = table.data();
    a.tt_bits = opt->tt_bits;
    a.tt_min = opt->tt_min > 0 ? opt->tt_min : 7;
  }
  a.order_table = opt->order_table;
  a.order_bits = opt->order_bits;
  a.learned_min = opt->learned_min > 0 ? opt->learned_min : 14;
  a.wait_limit_ns = 600ULL * 1000000000ULL;
  const size_t smem = batched_smem_bytes(T, a.smem_top);
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
  stats[4] = st.handouts;
  stats[5] = st.stab_cuts;
  stats[6] = st.status;
  return 0;
}

}  // extern "C"

// Batched solver: one persistent launch over a device work queue of
// positions ordered by empty count (most empties first), one thread per
// position at a time, each lane refilling itself from the queue as soon as
// its position is solved.
//
// Search (same values as the reference's negamax, different tree):
//   - nodes with >= ff empties: fastest-first order, kept as a sorted move
//     list per level (the role of the reference's UpperNode list,
//     solver.cu:78-93);
//   - nodes below ff: parity/corner order straight from the move mask;
//   - a child with <= 4 empties is solved inline by Small<N> (search.cuh);
//   - fail-soft negamax with in-place passes (solver.cu:57-73, 214-221,
//     246-256 semantics).
//
// Frames hold only what cannot be recomputed: the remaining-move mask, the
// flips of the move being searched (to undo it) and a packed word (move
// square, alpha, beta, best, passed).  They live in shared memory,
// interleaved by thread ([level][thread]) so a warp touching one level hits
// 32 consecutive words, or in local memory (kSmemStack = false).
#include "common.cuh"
#include "kernels.h"
#include "search.cuh"

namespace gpo {

constexpr int kUpperSlots = kMaxEmpties;  // sorted-list levels (local memory)

__device__ __forceinline__ unsigned pack_meta(int sq, int alpha, int beta, int best, int passed) {
  return static_cast<unsigned>(sq) | (static_cast<unsigned>(alpha & 0xff) << 6) |
         (static_cast<unsigned>(beta & 0xff) << 14) | (static_cast<unsigned>(best & 0xff) << 22) |
         (static_cast<unsigned>(passed) << 30);
}

// Sorted fastest-first list for the node (P, O) with move mask `moves`.
__device__ __forceinline__ int build_ff_list(u64 P, u64 O, u64 moves, unsigned char* list) {
  unsigned char key[kMaxEmpties];
  int n = 0;
  while (moves) {
    const u64 bit = moves & (0ULL - moves);
    moves ^= bit;
    const int sq = ctz64(bit);
    const int k = ff_key(P, O, sq, bit);
    int j = n++;
    while (j > 0 && key[j - 1] > k) {
      key[j] = key[j - 1];
      list[j] = list[j - 1];
      --j;
    }
    key[j] = static_cast<unsigned char>(k);
    list[j] = static_cast<unsigned char>(sq);
  }
  return n;
}

template <bool kSmemStack>
__global__ void batched_kernel(BatchedArgs args) {
  extern __shared__ u64 smem_u64[];
  const int B = blockDim.x;
  const int t = threadIdx.x;
  const int L = args.levels;
  u64* sM = smem_u64;
  u64* sF = smem_u64 + L * B;
  unsigned* sX = reinterpret_cast<unsigned*>(smem_u64 + 2 * L * B);
  u64 lM[kSmemStack ? 1 : kMaxEmpties];
  u64 lF[kSmemStack ? 1 : kMaxEmpties];
  unsigned lX[kSmemStack ? 1 : kMaxEmpties];
  unsigned char ulist[kUpperSlots][kMaxEmpties];
  unsigned char uidx_s[kUpperSlots], ucnt_s[kUpperSlots];

  const unsigned lane = t & 31;
  const unsigned lane_lt = (1u << lane) - 1u;
  unsigned long long total_nodes = 0;

  bool busy = false, exhausted = false;
  int pos = 0;
  u64 P = 0, O = 0, moves = 0;
  int alpha = 0, beta = 0, best = 0, passed = 0, E = 0, level = 0, uidx = 0, ucnt = 0;
  int rootbest = kMoveNoneDev;
  unsigned long long nodes = 0;

  for (;;) {
    // ---- refill idle lanes from the queue (one atomic per warp) ----
    const unsigned need = __ballot_sync(0xffffffffu, !busy && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned base = 0;
      if (static_cast<int>(lane) == leader) base = atomicAdd(&args.stats->next, __popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!busy && !exhausted) {
        const unsigned k = base + __popc(need & lane_lt);
        if (k < static_cast<unsigned>(args.n)) {
          pos = static_cast<int>(args.perm[k]);
          P = args.player[pos];
          O = args.opp[pos];
          E = 64 - popc(P | O);
          nodes = 1;
          alpha = -64;
          beta = 64;
          best = -65;
          passed = 0;
          level = 0;
          rootbest = kMoveNoneDev;
          moves = gpo_mobility(P, O);
          busy = true;
          if ((P & O) || E > args.depth) {  // rejected input: flagged, not searched
            atomicOr(&args.stats->status, (P & O) ? kErrOverlap : kErrDepth);
            args.score[pos] = 0;
            if (args.best) args.best[pos] = kMoveNoneDev;
            if (args.nodes_out) args.nodes_out[pos] = 0;
            busy = false;
          } else if (!moves) {
            const u64 om = gpo_mobility(O, P);
            if (!om) {
              args.score[pos] = static_cast<signed char>(gpo_final(P, O));
              if (args.best) args.best[pos] = kMoveNoneDev;
              if (args.nodes_out) args.nodes_out[pos] = nodes;
              total_nodes += nodes;
              busy = false;
            } else {
              const u64 tmp = P;
              P = O;
              O = tmp;
              alpha = -64;
              beta = 64;
              passed = 1;
              moves = om;
              ++nodes;
              rootbest = kMovePassDev;
            }
          }
          if (busy && E >= args.ff) {
            ucnt = build_ff_list(P, O, moves, ulist[0]);
            uidx = 0;
          }
        } else {
          exhausted = true;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, busy) == 0) break;
    if (!busy) continue;

    // ---- one search step ----
    const bool upper = E >= args.ff;
    int sq = -1;
    if (alpha < beta) {
      if (upper) {
        if (uidx < ucnt) sq = ulist[level][uidx++];
      } else if (moves) {
        const u64 bit = pick_parity(moves, ~(P | O));
        moves ^= bit;
        sq = ctz64(bit);
      }
    }
    if (sq >= 0) {
      const u64 bit = 1ULL << sq;
      const u64 f = gpo_flip(P, O, sq);
      const u64 cP = O ^ f, cO = P ^ f ^ bit;
      const int lo = alpha > best ? alpha : best;
      int v;
      bool pushed = false;
      if (E - 1 <= kSmallMax) {
        v = -small_solve(E - 1, cP, cO, -beta, -lo, nodes);
      } else {
        ++nodes;
        const u64 cm = gpo_mobility(cP, cO);
        u64 om = 0;
        if (!cm) om = gpo_mobility(cO, cP);
        if (!cm && !om) {
          v = -gpo_final(cP, cO);
        } else {
          if (level >= L) {  // unreachable when frames cover maxE - kSmallMax levels
            atomicOr(&args.stats->status, kErrInternal);
            busy = false;
            exhausted = true;
            continue;
          }
          const unsigned meta = pack_meta(sq, alpha, beta, best, passed);
          if (kSmemStack) {
            sM[level * B + t] = moves;
            sF[level * B + t] = f;
            sX[level * B + t] = meta;
          } else {
            lM[level] = moves;
            lF[level] = f;
            lX[level] = meta;
          }
          if (upper && level < kUpperSlots) {
            uidx_s[level] = static_cast<unsigned char>(uidx);
            ucnt_s[level] = static_cast<unsigned char>(ucnt);
          }
          ++level;
          --E;
          best = -65;
          if (cm) {
            P = cP;
            O = cO;
            alpha = -beta;
            beta = -lo;
            passed = 0;
            moves = cm;
          } else {  // the child passes at once: same side to move, same window
            P = cO;
            O = cP;
            alpha = lo;  // beta unchanged
            passed = 1;
            moves = om;
            ++nodes;
          }
          if (E >= args.ff && level < kUpperSlots) {
            ucnt = build_ff_list(P, O, moves, ulist[level]);
            uidx = 0;
          }
          pushed = true;
          if (args.node_budget && nodes > args.node_budget) {
            atomicOr(&args.stats->status, kErrBudget);
            args.score[pos] = 0;
            if (args.best) args.best[pos] = kMoveNoneDev;
            if (args.nodes_out) args.nodes_out[pos] = nodes;
            total_nodes += nodes;
            busy = false;
          }
        }
      }
      if (!pushed) {
        if (v > best) {
          best = v;
          if (level == 0 && !passed) rootbest = sq;
          if (best > alpha) alpha = best;
        }
      }
      continue;
    }

    // ---- node finished: return its value to the parent ----
    const int r = passed ? -best : best;
    if (level == 0) {
      args.score[pos] = static_cast<signed char>(r);
      if (args.best) args.best[pos] = static_cast<signed char>(rootbest);
      if (args.nodes_out) args.nodes_out[pos] = nodes;
      total_nodes += nodes;
      busy = false;
      continue;
    }
    if (passed) {  // back to the orientation the node was created in
      const u64 tmp = P;
      P = O;
      O = tmp;
    }
    --level;
    ++E;
    u64 f;
    unsigned meta;
    if (kSmemStack) {
      moves = sM[level * B + t];
      f = sF[level * B + t];
      meta = sX[level * B + t];
    } else {
      moves = lM[level];
      f = lF[level];
      meta = lX[level];
    }
    const int psq = static_cast<int>(meta & 63u);
    alpha = static_cast<signed char>((meta >> 6) & 0xff);
    beta = static_cast<signed char>((meta >> 14) & 0xff);
    best = static_cast<signed char>((meta >> 22) & 0xff);
    passed = static_cast<int>((meta >> 30) & 1u);
    if (E >= args.ff && level < kUpperSlots) {
      uidx = uidx_s[level];
      ucnt = ucnt_s[level];
    }
    {
      const u64 bit = 1ULL << psq;
      const u64 pP = O ^ f ^ bit, pO = P ^ f;
      P = pP;
      O = pO;
    }
    const int v = -r;
    if (v > best) {
      best = v;
      if (level == 0 && !passed) rootbest = psq;
      if (best > alpha) alpha = best;
    }
  }
  warp_add(&args.stats->nodes, total_nodes);
}

int batched_levels(int depth) {
  const int l = depth - kSmallMax - 1;
  return l > 1 ? l : 1;
}

cudaError_t launch_batched(const BatchedArgs& args, BatchedLaunch& cfg, int sms, cudaStream_t s) {
  const int threads = cfg.threads > 0 ? cfg.threads : 128;
  const size_t smem = cfg.smem_stack ? static_cast<size_t>(threads) * args.levels * 20 : 0;
  auto kernel = cfg.smem_stack ? batched_kernel<true> : batched_kernel<false>;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  cfg.grid = per_sm * sms;
  cfg.smem = smem;
  kernel<<<cfg.grid, threads, smem, s>>>(args);
  return cudaGetLastError();
}

}  // namespace gpo

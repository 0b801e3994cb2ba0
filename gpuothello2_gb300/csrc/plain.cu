// Plain thread-per-board solver: one thread searches one position with the
// reference's exact tree, so its scores and its per-position node counts can
// be checked one-for-one against the reference-order oracle.
//
// Tree (solver.cu:75-283, node.cuh:5-74):
//   - "upper" plies 0 .. depth-10 order the legal moves by the opponent's
//     move count after the move, stably, from the empty-scan order
//     (corners first, then lowest square) (solver.cu:78-93);
//   - deeper "lower" plies take the legal moves in the empty-scan order
//     (node.cuh:21-28, solver.cu:244-270); the reference tries every empty
//     square and skips the ones that flip nothing, which visits the same
//     children in the same order as walking the legal-move mask;
//   - fail-soft negamax: result = max(result, v), alpha = max(alpha, result),
//     stop when alpha >= beta (node.cuh:70-73, solver.cu:146-149);
//   - a side without moves passes in place with the window negated and
//     swapped; a second pass scores the position; a parent takes +result from
//     a passed child and -result otherwise (solver.cu:57-73, 162-165, 171,
//     183, 200, 214-221, 246-256).
//
// GB300 layout: one thread per position over the whole grid (the reference
// runs n/32 threads, solver.cu:321, 331); lower frames in shared memory,
// interleaved by thread so a warp's accesses to one level hit distinct banks;
// upper frames (rarely touched) in per-thread local memory.
#include "common.cuh"
#include "kernels.h"

namespace gpo {

constexpr int kPlainLower = 10;  // lower_stack_depth + 1 (solver.cu:9, 331)
constexpr int kPlainBlock = 128;

struct PlainUpper {
  u64 P, O;
  int alpha, beta, result, idx, n, passed;
  unsigned char list[kMaxEmpties];
};

// Legal moves of an upper node in the reference's order.
__device__ __forceinline__ int plain_upper_moves(u64 P, u64 O, unsigned char* list,
                                                 const u64* rays) {
  unsigned char key[kMaxEmpties];
  int n = 0;
  const u64 moves = gpo_mobility(P, O);
  for (int part = 0; part < 2; ++part) {
    u64 m = part == 0 ? (moves & kCorners) : (moves & ~kCorners);
    while (m) {
      const int sq = ctz64(m);
      m &= m - 1;
      const u64 bit = 1ULL << sq;
      const u64 f = gpo_flip(P, O, sq, rays);
      const int k = popc(gpo_mobility(O ^ f, P ^ f ^ bit));
      int j = n++;
      while (j > 0 && key[j - 1] > k) {
        key[j] = key[j - 1];
        list[j] = list[j - 1];
        --j;
      }
      key[j] = static_cast<unsigned char>(k);
      list[j] = static_cast<unsigned char>(sq);
    }
  }
  return n;
}

__device__ __forceinline__ u64 scan_pick(u64 moves) {
  const u64 c = moves & kCorners;
  return c ? (c & (0ULL - c)) : (moves & (0ULL - moves));
}

__global__ void __launch_bounds__(kPlainBlock)
plain_kernel(const u64* __restrict__ player, const u64* __restrict__ opp, int n, int depth,
             signed char* __restrict__ score, unsigned long long* __restrict__ nodes_out,
             DeviceStats* __restrict__ stats, unsigned long long limit_ns) {
  __shared__ u64 sP[kPlainLower][kPlainBlock];
  __shared__ u64 sO[kPlainLower][kPlainBlock];
  __shared__ u64 sM[kPlainLower][kPlainBlock];
  __shared__ int sMeta[kPlainLower][kPlainBlock];
  __shared__ __align__(16) u64 rays[256];
  PlainUpper up[kMaxEmpties - 8];
  gpo_build_rays(rays);
  // One deadline for the launch: the first block to start stamps the time.
  if (threadIdx.x == 0) atomicCAS(&stats->t0, 0ULL, gpo_global_ns());
  __syncthreads();
  const unsigned long long deadline = *reinterpret_cast<volatile unsigned long long*>(&stats->t0) + limit_ns;

  const int t = threadIdx.x;
  const int i = blockIdx.x * blockDim.x + t;
  unsigned long long nodes = 0;
  if (i < n) {
    u64 P = player[i], O = opp[i];
    const int empties = 64 - popc(P | O);
    if ((P & O) != 0) {
      atomicOr(&stats->status, kErrOverlap);
    } else if (empties > depth) {
      atomicOr(&stats->status, kErrDepth);
    } else {
      const int U = depth > 10 ? depth - 9 : 1;  // number of upper plies
      int level = 0;
      int alpha = -64, beta = 64, result = -64, passed = 0, found = 0, idx = 0, cnt = 0;
      u64 moves = 0;
      cnt = plain_upper_moves(P, O, up[0].list, rays);
      nodes = 1;
      for (;;) {
        if ((nodes & 4095) == 0 && gpo_global_ns() > deadline) {  // past the launch deadline
          atomicOr(&stats->status, kErrWait);
          break;
        }
        // Each pass either pushes a child / passes in place (continue) or
        // falls through to the commit at the bottom.
        if (level < U) {
          if (idx == cnt) {
            if (cnt == 0) {
              if (passed) {
                result = gpo_final(P, O);
              } else {
                const u64 tmp = P;
                P = O;
                O = tmp;
                const int a = alpha;
                alpha = -beta;
                beta = -a;
                result = -64;
                passed = 1;
                ++nodes;
                cnt = plain_upper_moves(P, O, up[level].list, rays);
                idx = 0;
                continue;
              }
            }
          } else if (alpha < beta) {
            const int sq = up[level].list[idx++];
            const u64 bit = 1ULL << sq;
            const u64 f = gpo_flip(P, O, sq, rays);
            PlainUpper& fr = up[level];
            fr.P = P; fr.O = O; fr.alpha = alpha; fr.beta = beta; fr.result = result;
            fr.idx = idx; fr.n = cnt; fr.passed = passed;
            const u64 nP = O ^ f, nO = P ^ f ^ bit;
            P = nP; O = nO;
            const int a = alpha;
            alpha = -beta;
            beta = -a;
            passed = 0;
            ++level;
            ++nodes;
            if (level < U) {
              result = -64;
              idx = 0;
              cnt = plain_upper_moves(P, O, up[level].list, rays);
            } else {
              result = -127;
              found = 0;
              moves = gpo_mobility(P, O);
            }
            continue;
          }
        } else {
          if (!moves) {
            if (found) {
              // all moves searched
            } else if (passed) {
              result = gpo_final(P, O);
            } else {
              const u64 tmp = P;
              P = O;
              O = tmp;
              const int a = alpha;
              alpha = -beta;
              beta = -a;
              result = -127;
              passed = 1;
              ++nodes;
              moves = gpo_mobility(P, O);
              continue;
            }
          } else if (alpha < beta) {
            const u64 bit = scan_pick(moves);
            moves ^= bit;
            found = 1;
            const int sq = ctz64(bit);
            const u64 f = gpo_flip(P, O, sq, rays);
            const int l = level - U;
            if (l >= kPlainLower) {  // depth >= empties makes this unreachable
              atomicOr(&stats->status, kErrInternal);
              break;
            }
            sP[l][t] = P;
            sO[l][t] = O;
            sM[l][t] = moves;
            sMeta[l][t] = (alpha & 0xff) | ((beta & 0xff) << 8) | ((result & 0xff) << 16) |
                          (passed << 24) | (found << 25);
            const u64 nP = O ^ f, nO = P ^ f ^ bit;
            P = nP; O = nO;
            const int a = alpha;
            alpha = -beta;
            beta = -a;
            result = -127;
            passed = 0;
            found = 0;
            ++level;
            ++nodes;
            moves = gpo_mobility(P, O);
            continue;
          }
        }
        // commit: hand this node's value to its parent
        const int v = passed ? result : -result;
        if (level == 0) {
          score[i] = static_cast<signed char>(passed ? -result : result);
          break;
        }
        --level;
        if (level < U) {
          const PlainUpper& fr = up[level];
          P = fr.P; O = fr.O; alpha = fr.alpha; beta = fr.beta; result = fr.result;
          idx = fr.idx; cnt = fr.n; passed = fr.passed;
        } else {
          const int l = level - U;
          P = sP[l][t];
          O = sO[l][t];
          moves = sM[l][t];
          const int m = sMeta[l][t];
          alpha = static_cast<signed char>(m & 0xff);
          beta = static_cast<signed char>((m >> 8) & 0xff);
          result = static_cast<signed char>((m >> 16) & 0xff);
          passed = (m >> 24) & 1;
          found = (m >> 25) & 1;
        }
        if (v > result) result = v;
        if (result > alpha) alpha = result;
      }
    }
    if (nodes_out) nodes_out[i] = nodes;
  }
  warp_add(&stats->nodes, nodes);
}

cudaError_t launch_plain(const u64* player, const u64* opp, int n, int depth, signed char* score,
                         unsigned long long* nodes_out, DeviceStats* stats,
                         unsigned long long limit_ns, cudaStream_t s) {
  const int grid = (n + kPlainBlock - 1) / kPlainBlock;
  plain_kernel<<<grid, kPlainBlock, 0, s>>>(player, opp, n, depth, score, nodes_out, stats,
                                            limit_ns);
  return cudaGetLastError();
}

}  // namespace gpo

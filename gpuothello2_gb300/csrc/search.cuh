// Search building blocks of the batched solver: the exact solver for the
// last few empties and the move pickers.  The reference has no such
// specialisation (its lower nodes try every empty square, solver.cu:244-270);
// these change node counts and speed only, never a score.
#pragma once
#include "common.cuh"

namespace gpo {

constexpr u64 kXSquares = 0x0042000000004200ULL;  // B2, G2, B7, G7

// Exact negamax value of (P, O) with exactly N empty squares, fail-soft in
// (alpha, beta).  One loop per side: the side to move tries its moves; if it
// has none the other side moves (a pass), and if neither can move the game
// is over.  Counts every position examined, pass frames included.
template <int N>
struct Small {
  static __device__ __forceinline__ int solve(u64 P, u64 O, int alpha, int beta,
                                              unsigned long long& nodes) {
    ++nodes;
    const u64 empty = ~(P | O);
    u64 me = P, you = O;
    int a = alpha, b = beta;
    int best = -65;
    int side = 0;
    for (;;) {
      u64 it = empty;
      while (it) {
        const u64 bit = it & (0ULL - it);
        it ^= bit;
        const u64 f = gpo_flip(me, you, ctz64(bit));
        if (!f) continue;
        const int lo = a > best ? a : best;
        const int v = -Small<N - 1>::solve(you ^ f, me ^ f ^ bit, -b, -lo, nodes);
        if (v > best) {
          best = v;
          if (v >= b) break;
        }
      }
      if (best > -65 || side) break;
      // the side to move has no move: pass
      side = 1;
      ++nodes;
      const u64 t = me;
      me = you;
      you = t;
      const int ta = a;
      a = -b;
      b = -ta;
    }
    if (best == -65) return gpo_final(P, O);  // neither side can move
    return side ? -best : best;
  }
};

template <>
struct Small<1> {
  static __device__ __forceinline__ int solve(u64 P, u64 O, int, int,
                                              unsigned long long& nodes) {
    ++nodes;
    return gpo_solve1(P, O, ctz64(~(P | O)));
  }
};

template <>
struct Small<0> {
  static __device__ __forceinline__ int solve(u64 P, u64 O, int, int,
                                              unsigned long long& nodes) {
    ++nodes;
    return gpo_final(P, O);
  }
};

// Runtime dispatch for a child with `e` <= kSmallMax empties.
constexpr int kSmallMax = 4;
__device__ __forceinline__ int small_solve(int e, u64 P, u64 O, int alpha, int beta,
                                           unsigned long long& nodes) {
  switch (e) {
    case 4: return Small<4>::solve(P, O, alpha, beta, nodes);
    case 3: return Small<3>::solve(P, O, alpha, beta, nodes);
    case 2: return Small<2>::solve(P, O, alpha, beta, nodes);
    case 1: return Small<1>::solve(P, O, alpha, beta, nodes);
    default: return Small<0>::solve(P, O, alpha, beta, nodes);
  }
}

// Move choice below the fastest-first threshold: corners, then squares in
// quadrants holding an odd number of empties (the last move of a region is
// then ours), avoiding the X-squares next to an empty corner; lowest square
// breaks ties.
__device__ __forceinline__ u64 pick_parity(u64 moves, u64 empty) {
  const u64 q0 = 0x000000000f0f0f0fULL, q1 = 0x00000000f0f0f0f0ULL;
  const u64 q2 = 0x0f0f0f0f00000000ULL, q3 = 0xf0f0f0f000000000ULL;
  const u64 odd = ((popc(empty & q0) & 1) ? q0 : 0ULL) | ((popc(empty & q1) & 1) ? q1 : 0ULL) |
                  ((popc(empty & q2) & 1) ? q2 : 0ULL) | ((popc(empty & q3) & 1) ? q3 : 0ULL);
  u64 c = moves & kCorners;
  if (c) return c & (0ULL - c);
  c = moves & odd & ~kXSquares;
  if (c) return c & (0ULL - c);
  c = moves & ~kXSquares;
  if (c) return c & (0ULL - c);
  return moves & (0ULL - moves);
}

// Fastest-first key of a move: the opponent's reply count after it, with
// corners first on ties.  Lower keys are searched first.
__device__ __forceinline__ int ff_key(u64 P, u64 O, int sq, u64 bit) {
  const u64 f = gpo_flip(P, O, sq);
  const int k = popc(gpo_mobility(O ^ f, P ^ f ^ bit)) * 2;
  return (bit & kCorners) ? k : k + 1;
}

}  // namespace gpo

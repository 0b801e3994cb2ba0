// Bitboard primitives for the endgame search (device side).
//
// Square numbering follows the reference: square = row*8 + col, A1 = bit 0
// (main.cu:31-39).  A position is (P, O): discs of the side to move and of
// the other side.
//
//   gpo_mobility   legal-move mask            (board.cu:56-78 semantics)
//   gpo_flip       discs flipped by a move    (board.cu:28-54 semantics)
//   gpo_final      disc difference at game end, empties to the winner
//                                             (board.cuh:7-18)
//
// The ray geometry constants are the squares k*s (k = 1..7) reached from
// square 0 by steps s = 1, 7, 8, 9 ("up", toward higher bits) and the mirror
// set 63 - k*s ("down", toward lower bits).  Horizontal and diagonal runs can
// only flank interior discs, so the opponent set is clipped to columns B..G
// for those lines; every scan then stops at an edge column at the latest and
// the masks need no per-square clipping.
#pragma once
#include <cstdint>

namespace gpo {

typedef unsigned long long u64;

__device__ __forceinline__ int popc(u64 x) { return __popcll(x); }

// ---- mobility ----
// One line direction with step S: discs of O (masked by M) reachable from P
// by one or more steps, propagated with a doubling pass (runs are at most 6
// long), then moved one more step onto the landing square.
template <int S>
__device__ __forceinline__ u64 mob_dir(u64 P, u64 M) {
  u64 l = M & (P << S);
  u64 r = M & (P >> S);
  l |= M & (l << S);
  r |= M & (r >> S);
  const u64 pl = M & (M << S);
  const u64 pr = pl >> S;
  l |= pl & (l << (2 * S));
  r |= pr & (r >> (2 * S));
  l |= pl & (l << (2 * S));
  r |= pr & (r >> (2 * S));
  return (l << S) | (r >> S);
}

__device__ __forceinline__ u64 gpo_mobility(u64 P, u64 O) {
  const u64 Oi = O & 0x7e7e7e7e7e7e7e7eULL;
  const u64 m = mob_dir<1>(P, Oi) | mob_dir<7>(P, Oi) | mob_dir<9>(P, Oi) | mob_dir<8>(P, O);
  return m & ~(P | O);
}

// ---- flip ----
// Up ray (higher bits): the first square along the ray that is not an
// opponent disc is found with a carry: (Om | ~ray) + 1 clears every bit
// below it and sets it.  Down ray (lower bits): the first such square is
// the highest set bit of ~Om & ray.
__device__ __forceinline__ u64 flip_up(u64 P, u64 Om, u64 ray) {
  const u64 outflank = ((Om | ~ray) + 1) & ray & P;
  return outflank ? ((outflank - 1) & ray) : 0ULL;
}

__device__ __forceinline__ u64 flip_down(u64 P, u64 Om, u64 ray) {
  const u64 stop = ~Om & ray;
  const u64 top = stop ? (0x8000000000000000ULL >> __clzll(stop)) : 0ULL;
  const u64 outflank = top & P;
  return (0ULL - outflank - outflank) & ray;  // ray squares above outflank
}

__device__ __forceinline__ u64 gpo_flip(u64 P, u64 O, int sq) {
  const u64 Oi = O & 0x7e7e7e7e7e7e7e7eULL;
  const int dn = 63 - sq;
  u64 f = flip_up(P, O, 0x0101010101010100ULL << sq);
  f |= flip_up(P, Oi, 0x00000000000000feULL << sq);
  f |= flip_up(P, Oi, 0x0002040810204080ULL << sq);
  f |= flip_up(P, Oi, 0x8040201008040200ULL << sq);
  f |= flip_down(P, O, 0x0080808080808080ULL >> dn);
  f |= flip_down(P, Oi, 0x7f00000000000000ULL >> dn);
  f |= flip_down(P, Oi, 0x0102040810204000ULL >> dn);
  f |= flip_down(P, Oi, 0x0040201008040201ULL >> dn);
  return f;
}

// Exact final score: disc difference with the empties awarded to the
// winner (board.cuh:7-18).
__device__ __forceinline__ int gpo_final(u64 P, u64 O) {
  const int pc = popc(P), oc = popc(O);
  return pc == oc ? 0 : (pc > oc ? 64 - 2 * oc : 2 * pc - 64);
}

// Score after the last empty square `sq` is filled (or passed on).  With one
// empty the disc difference after a move follows from the flip count alone.
__device__ __forceinline__ int gpo_solve1(u64 P, u64 O, int sq) {
  int n = popc(gpo_flip(P, O, sq));
  if (n) return 2 * (popc(P) + n + 1) - 64;
  n = popc(gpo_flip(O, P, sq));
  if (n) return 64 - 2 * (popc(O) + n + 1);
  return gpo_final(P, O);
}

}  // namespace gpo

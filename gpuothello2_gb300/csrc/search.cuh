// Search building blocks of the batched solver: the move picker below the
// fastest-first threshold and the packed ordered-move list.  They change
// node counts and speed only, never a score.
#pragma once
#include "common.cuh"

namespace gpo {

constexpr u64 kXSquares = 0x0042000000004200ULL;  // B2, G2, B7, G7

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

// ---- packed fastest-first list ----
// One 64-bit word holds a node's best five moves in ascending key order:
// entries of 12 bits (key: 6 high bits, square: 6 low bits) at bits 0..59,
// an empty entry being all ones; bits 60..62 index the next entry to
// search; bit 63 records that the node has more than five moves (the rest
// are searched afterwards from the move mask).  Keeping the list in the
// frame's move word means no per-thread local memory is touched.
constexpr u64 kListEmpty = 0x0FFFFFFFFFFFFFFFULL;
constexpr u64 kListBody = (1ULL << 60) - 1;
constexpr u64 kListOverflow = 1ULL << 63;

__device__ __forceinline__ u64 list_insert(u64 lst, int key, int sq) {
  int j = 0;
#pragma unroll
  for (int i = 0; i < 5; ++i) j += static_cast<int>((lst >> (12 * i + 6)) & 63) <= key;
  if (j >= 5) return lst | kListOverflow;
  const u64 body = lst & kListBody;
  const u64 low = body & ((1ULL << (12 * j)) - 1);
  const u64 high = body >> (12 * j);
  const bool pushed_out = ((body >> 48) & 0xFFF) != 0xFFF;
  const u64 e = (static_cast<u64>(key) << 6) | static_cast<u64>(sq);
  const u64 nb = (low | (e << (12 * j)) | (high << (12 * (j + 1)))) & kListBody;
  return nb | (lst & ~kListBody) | (pushed_out ? kListOverflow : 0ULL);
}

__device__ __forceinline__ int list_index(u64 lst) { return static_cast<int>((lst >> 60) & 7); }

// Next entry (0xFFF when the five slots are used up or empty).
__device__ __forceinline__ int list_peek(u64 lst) {
  const int i = list_index(lst);
  return i < 5 ? static_cast<int>((lst >> (12 * i)) & 0xFFF) : 0xFFF;
}

// Squares held by the list.
__device__ __forceinline__ u64 list_squares(u64 lst) {
  u64 m = 0;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const int e = static_cast<int>((lst >> (12 * i)) & 0xFFF);
    if (e != 0xFFF) m |= 1ULL << (e & 63);
  }
  return m;
}

}  // namespace gpo

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
// Mobility: horizontal and diagonal runs can only flank interior discs, so
// the opponent set is clipped to columns B..G for those lines and no shift
// can carry a run across the board edge.
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
// Rays toward higher bits ("up": +8, +1, +7, +9) use a carry: the first
// square along the ray that is not an opponent disc is the lowest set bit of
// (Om | ~ray) + 1 within the ray.  Rays toward lower bits are the up rays of
// the mirrored square 63 - sq on the bit-reversed board (reversing the bit
// order rotates the board by 180 degrees, which maps south/west/south-east/
// south-west onto north/east/north-west/north-east), so all eight directions
// use the carry form.
//
// `rays` is the per-square up-ray table built by gpo_build_rays (in shared
// memory): rays[4*sq + k] for k = 0..3 = the squares beyond sq toward +8,
// +1, +7, +9.  Loading it runs on the load/store pipe, which the search
// leaves idle, instead of four variable 64-bit shifts on the integer pipe.
__device__ __forceinline__ u64 flip_up(u64 P, u64 Om, u64 ray) {
  const u64 outflank = ((Om | ~ray) + 1) & ray & P;
  return outflank ? ((outflank - 1) & ray) : 0ULL;
}

// The table's rays stop at the board edge, so no column mask is needed.
__device__ __forceinline__ u64 flip_up4(u64 P, u64 O, const u64* r) {
  const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(r);
  const ulonglong2 b = *reinterpret_cast<const ulonglong2*>(r + 2);
  return flip_up(P, O, a.x) | flip_up(P, O, a.y) | flip_up(P, O, b.x) | flip_up(P, O, b.y);
}

__device__ __forceinline__ u64 gpo_flip(u64 P, u64 O, int sq, const u64* rays) {
  const u64 up = flip_up4(P, O, rays + 4 * sq);
  const u64 dn = flip_up4(__brevll(P), __brevll(O), rays + 4 * (63 - sq));
  return up | __brevll(dn);
}

// Fills the 64 x 4 up-ray table (256 words) cooperatively; the caller
// synchronises the block afterwards.
__device__ __forceinline__ void gpo_build_rays(u64* rays) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    const int sq = i >> 2, k = i & 3;
    const int dr = k == 1 ? 0 : 1;
    const int dc = k == 0 ? 0 : (k == 1 ? 1 : (k == 2 ? -1 : 1));
    u64 m = 0;
    int r = sq / 8 + dr, c = sq % 8 + dc;
    while (r >= 0 && r < 8 && c >= 0 && c < 8) {
      m |= 1ULL << (r * 8 + c);
      r += dr;
      c += dc;
    }
    rays[i] = m;
  }
}

// Exact final score: disc difference with the empties awarded to the
// winner (board.cuh:7-18).
__device__ __forceinline__ int gpo_final(u64 P, u64 O) {
  const int pc = popc(P), oc = popc(O);
  return pc == oc ? 0 : (pc > oc ? 64 - 2 * oc : 2 * pc - 64);
}

// ---- flip counts at the last empty square ----
// With one empty square s, every other square holds a disc, so along each
// line through s the discs of one side are the complement of the other's:
// the discs X flips by playing s follow from X's 8-bit pattern on the line
// alone (the runs of non-X squares next to s that end at an X disc).
// cnt[pos * 256 + x] holds that count for an 8-square line with X pattern x
// and s at position pos.  The lines are gathered into 8-bit patterns:
//   row:       bit c = square (r, c);
//   column:    ((X >> c) & 0x0101..01) * 0x0102040810204080 >> 56, bit k =
//              square (k, c) (the partial products land on distinct bits);
//   diagonals: (X & mask) * 0x0101..01 >> 56, bit c = the diagonal's square
//              in column c.
// A diagonal shorter than 8 squares reads 0 (not X) past its ends, which is
// harmless: a run reaching past the board edge ends at no X disc.
// dmask[2 * s] / dmask[2 * s + 1]: the squares of s's a1-h8 and a8-h1
// diagonals.  Both tables are built once per block (gpo_build_last).
__device__ __forceinline__ void gpo_build_last(unsigned char* cnt, u64* dmask) {
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) {
    const int pos = i >> 8, x = i & 255;
    int n = 0, k = 0;
    for (int j = pos + 1; j < 8; ++j) {  // toward higher positions
      if ((x >> j) & 1) {
        n += k;
        break;
      }
      ++k;
    }
    k = 0;
    for (int j = pos - 1; j >= 0; --j) {  // toward lower positions
      if ((x >> j) & 1) {
        n += k;
        break;
      }
      ++k;
    }
    cnt[i] = static_cast<unsigned char>(n);
  }
  for (int i = threadIdx.x; i < 128; i += blockDim.x) {
    const int sq = i >> 1, r = sq >> 3, c = sq & 7;
    u64 m = 0;
    for (int rr = 0; rr < 8; ++rr) {
      const int cc = (i & 1) ? (r + c - rr) : (c - r + rr);  // a8-h1 : a1-h8
      if (cc >= 0 && cc < 8) m |= 1ULL << (rr * 8 + cc);
    }
    dmask[i] = m;
  }
}

__device__ __forceinline__ int gpo_last_count(u64 X, int s, const unsigned char* cnt,
                                              const u64* dmask) {
  const int r = s >> 3, c = s & 7;
  const unsigned row = static_cast<unsigned>(X >> (8 * r)) & 0xffu;
  const unsigned col =
      static_cast<unsigned>((((X >> c) & 0x0101010101010101ULL) * 0x0102040810204080ULL) >> 56);
  const unsigned d9 = static_cast<unsigned>(((X & dmask[2 * s]) * 0x0101010101010101ULL) >> 56);
  const unsigned d7 = static_cast<unsigned>(((X & dmask[2 * s + 1]) * 0x0101010101010101ULL) >> 56);
  return cnt[c * 256 + row] + cnt[r * 256 + col] + cnt[c * 256 + d9] + cnt[c * 256 + d7];
}

// ---- stable discs ----
// A subset of the discs of `O` that no sequence of moves can flip: a disc is
// kept when, along each of the four line directions, its line is full, it
// sits on the board edge across that direction, or a neighbour along it is
// already kept.  Such a disc cannot be flipped along that line (a flip needs
// an empty square to play on and a bracketing disc on the far side, and the
// kept neighbour would have to flip with it).  Sound after any number of
// rounds, so the loop is bounded; it stops early when nothing is added.
// The side to move can then score at most 64 - 2 * popc(result).
__device__ __forceinline__ u64 gpo_stable(u64 O, u64 occ) {
  constexpr u64 notA = 0xfefefefefefefefeULL, notH = 0x7f7f7f7f7f7f7f7fULL;
  constexpr u64 notAB = 0xfcfcfcfcfcfcfcfcULL, notGH = 0x3f3f3f3f3f3f3f3fULL;
  constexpr u64 notAD = 0xf0f0f0f0f0f0f0f0ULL, notEH = 0x0f0f0f0f0f0f0f0fULL;
  constexpr u64 colAH = 0x8181818181818181ULL, row18 = 0xff000000000000ffULL;
  constexpr u64 edge = colAH | row18;
  // full rows: bit 8r survives the three folds only if the whole byte is set
  u64 h = occ & (occ >> 1);
  h &= h >> 2;
  h &= h >> 4;
  h = (h & 0x0101010101010101ULL) * 0xffULL;
  // full columns: bit c of row 0 survives only if the whole column is set
  u64 v = occ & (occ >> 8);
  v &= v >> 16;
  v &= v >> 32;
  v = (v & 0xffULL) * 0x0101010101010101ULL;
  // diagonals: spread the empty squares along each diagonal (1, 2, 4 steps);
  // squares never reached lie on full diagonals
  u64 e9 = ~occ, e7 = ~occ;
  e9 |= ((e9 << 9) & notA) | ((e9 >> 9) & notH);
  e9 |= ((e9 << 18) & notAB) | ((e9 >> 18) & notGH);
  e9 |= ((e9 << 36) & notAD) | ((e9 >> 36) & notEH);
  e7 |= ((e7 << 7) & notH) | ((e7 >> 7) & notA);
  e7 |= ((e7 << 14) & notGH) | ((e7 >> 14) & notAB);
  e7 |= ((e7 << 28) & notEH) | ((e7 >> 28) & notAD);
  const u64 H = h | colAH, V = v | row18, D9 = ~e9 | edge, D7 = ~e7 | edge;
  u64 st = 0;
  for (int i = 0; i < 8; ++i) {
    const u64 n = O & (H | ((st << 1) & notA) | ((st >> 1) & notH)) & (V | (st << 8) | (st >> 8)) &
                  (D9 | ((st << 9) & notA) | ((st >> 9) & notH)) &
                  (D7 | ((st << 7) & notH) | ((st >> 7) & notA));
    if (n == st) break;
    st = n;
  }
  return st;
}

// Score after the last empty square `sq` is filled (or passed on).  With one
// empty the disc difference after a move follows from the flip count alone.
__device__ __forceinline__ int gpo_solve1(u64 P, u64 O, int sq, const u64* rays) {
  int n = popc(gpo_flip(P, O, sq, rays));
  if (n) return 2 * (popc(P) + n + 1) - 64;
  n = popc(gpo_flip(O, P, sq, rays));
  if (n) return 64 - 2 * (popc(O) + n + 1);
  return gpo_final(P, O);
}

}  // namespace gpo

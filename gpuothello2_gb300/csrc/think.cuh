// Think mode: the pattern evaluator and the depth-limited search, written
// once for the device and the host.  The CUDA kernels in think.cu call these
// functions per thread; the same source compiles as plain C++ (no
// __CUDACC__), which lets the CPU tests check this exact search and
// evaluator against the oracle without a GPU.  Nothing in the product runs
// the host instantiation.
//
// Evaluator (replaces Evaluator, eval.cuh:5-17, eval.cu:12-141).  A feature
// is a square mask with a table of 3^k floats (k = its square count) indexed
// by the base-3 number whose digit j is 0 (empty), 1 (side to move) or 2
// (other side) on the mask's j-th lowest square.  The reference computes
// that index with a bit extract and a base-3 lookup (eval.cu:107-113); here
// it is a sum of per-byte tables: for each byte of the board a feature
// covers, a 256-entry table maps the byte's discs to their base-3 digit
// weights, so one feature costs one or two lookups per side in shared
// memory and one gather from the L2-resident value tables.  The board is
// scored in the reference's 8 symmetries and order: for each of 4 rotations
// the board as is, then transposed, features in file order, summed in
// float in exactly that order, plus the offset, clamped to [-64, 64]
// (eval.cu:129-141) -- so the float result is bit-identical.
//
// Search (replaces think_kernel, thinker.cu:12-376).  depth-3 "upper"
// plies order the legal moves by the opponent's reply count after the move,
// stably, from the corners-first scan (thinker.cu:18-33), start at -65 and
// record the move of each raising commit (thinker.cu:97-103); the last 3
// plies take the legal moves corners first, then lowest square
// (node.cuh:21-28); a move at the last ply is scored round(eval) of the
// position reached (thinker.cu:200-204, 324-326) and a game that ends
// earlier is scored exactly.  Fail-soft; a side without moves passes in
// place with the window negated (no ply consumed); a parent takes +value
// from a passed child and -value otherwise.  The root's best move is 64
// when the root passed (thinker.cu:167-170).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GPO_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#define GPO_HD inline
#endif

namespace gpo {
namespace think {

typedef unsigned long long u64;

constexpr int kMaxFeatures = 32;
constexpr int kMaxPairs = 64;        // (feature, board byte) digit tables in all
constexpr int kMaxFeatureBits = 12;  // 3^12 values per feature at most
constexpr int kMinDepth = 4;         // depth - 3 upper plies must exist (thinker.cu:8, 362)
constexpr int kMaxDepth = 24;
constexpr int kMaxMoves = 64;
constexpr int kMovePass = 64;
constexpr int kMoveNone = 65;
constexpr u64 kCornerMask = 0x8100000000000081ULL;

struct EvalMeta {
  int nf;                                    // features
  int npairs;                                // digit tables
  float offset;
  unsigned value_off[kMaxFeatures];          // first value of feature j
  unsigned char pair_begin[kMaxFeatures + 1];  // tables of feature j: [begin[j], begin[j+1])
  unsigned char pair_byte[kMaxPairs];        // board byte each table reads
};

// ---- bit helpers ----
GPO_HD int popc(u64 x) {
#ifdef __CUDA_ARCH__
  return __popcll(x);
#else
  return __builtin_popcountll(x);
#endif
}

GPO_HD int lowest_square(u64 x) {  // x != 0
#ifdef __CUDA_ARCH__
  return __ffsll(static_cast<long long>(x)) - 1;
#else
  return __builtin_ctzll(x);
#endif
}

// Row r -> row 7-r (a byte reversal).
GPO_HD u64 flip_rows(u64 x) {
#ifdef __CUDA_ARCH__
  const unsigned lo = static_cast<unsigned>(x), hi = static_cast<unsigned>(x >> 32);
  return (static_cast<u64>(__byte_perm(lo, 0, 0x0123)) << 32) | __byte_perm(hi, 0, 0x0123);
#else
  return __builtin_bswap64(x);
#endif
}

// Exchanges the bits selected by `low` with the bits d places above them.
GPO_HD u64 swap_bits(u64 x, u64 low, int d) {
  const u64 t = (x ^ (x >> d)) & low;
  return x ^ t ^ (t << d);
}

// Square (r, c) -> (c, r): swap the off-diagonal 4x4 blocks, then the 2x2
// blocks inside each 4x4 block, then single squares inside each 2x2 block.
GPO_HD u64 transpose(u64 x) {
  x = swap_bits(x, 0x00000000F0F0F0F0ULL, 28);
  x = swap_bits(x, 0x0000CCCC0000CCCCULL, 14);
  return swap_bits(x, 0x00AA00AA00AA00AAULL, 7);
}

// Shift of a disc set one square in direction d (E, W, N, S, NE, NW, SE,
// SW), dropping discs that leave the board.
GPO_HD u64 step(u64 x, int d) {
  const u64 not_a = 0xFEFEFEFEFEFEFEFEULL, not_h = 0x7F7F7F7F7F7F7F7FULL;
  switch (d) {
    case 0: return (x << 1) & not_a;
    case 1: return (x >> 1) & not_h;
    case 2: return x << 8;
    case 3: return x >> 8;
    case 4: return (x << 9) & not_a;
    case 5: return (x << 7) & not_h;
    case 6: return (x >> 7) & not_a;
    default: return (x >> 9) & not_h;
  }
}

GPO_HD u64 mobility(u64 P, u64 O) {
  const u64 empty = ~(P | O);
  u64 moves = 0;
  for (int d = 0; d < 8; ++d) {
    u64 x = step(P, d) & O;
    for (int k = 0; k < 5; ++k) x |= step(x, d) & O;
    moves |= step(x, d) & empty;
  }
  return moves;
}

GPO_HD u64 flips(u64 P, u64 O, int sq) {
  u64 f = 0;
  for (int d = 0; d < 8; ++d) {
    u64 run = 0, x = step(1ULL << sq, d);
    while (x & O) {
      run |= x;
      x = step(x, d);
    }
    if (x & P) f |= run;
  }
  return f;
}

GPO_HD int final_score(u64 P, u64 O) {
  const int p = popc(P), o = popc(O);
  if (p == o) return 0;
  return p > o ? 64 - 2 * o : 2 * p - 64;
}

// ---- evaluator ----
template <class T>
GPO_HD T load_ro(const T* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

GPO_HD unsigned feature_index(u64 me, u64 op, const EvalMeta& m, const unsigned* digits, int j) {
  unsigned idx = 0;
  for (int k = m.pair_begin[j]; k < m.pair_begin[j + 1]; ++k) {
    const int sh = 8 * m.pair_byte[k];
    const unsigned* t = digits + 256 * k;
    idx += t[(me >> sh) & 0xFF] + 2u * t[(op >> sh) & 0xFF];
  }
  return idx;
}

GPO_HD float evaluate(u64 me, u64 op, const EvalMeta& m, const unsigned* digits,
                      const float* values) {
  float score = 0.0f;
  for (int r = 0; r < 4; ++r) {
    const u64 tme = transpose(me), top = transpose(op);
    for (int j = 0; j < m.nf; ++j) {
      const float* v = values + m.value_off[j];
      score += load_ro(v + feature_index(me, op, m, digits, j));
      score += load_ro(v + feature_index(tme, top, m, digits, j));
    }
    me = flip_rows(tme);
    op = flip_rows(top);
  }
  const float s = score + m.offset;
  return s > 64.0f ? 64.0f : (s < -64.0f ? -64.0f : s);
}

GPO_HD int leaf_value(u64 me, u64 op, const EvalMeta& m, const unsigned* digits,
                      const float* values) {
  return static_cast<int>(roundf(evaluate(me, op, m, digits, values)));
}

// ---- search ----
struct Frame {
  u64 P, O, moves;  // moves: lower plies, the legal moves not yet tried
  int alpha, beta, result;
  int passed, idx, n, best;
};

// Legal moves of an upper node in the reference's order; returns the count.
GPO_HD int upper_moves(u64 P, u64 O, unsigned char* list) {
  unsigned char key[kMaxMoves];
  int n = 0;
  const u64 legal = mobility(P, O);
  for (int part = 0; part < 2; ++part) {
    u64 m = part == 0 ? (legal & kCornerMask) : (legal & ~kCornerMask);
    while (m) {
      const int sq = lowest_square(m);
      m &= m - 1;
      const u64 bit = 1ULL << sq;
      const u64 f = flips(P, O, sq);
      const int k = popc(mobility(O ^ f, P ^ f ^ bit));
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

GPO_HD u64 scan_pick(u64 moves) {
  const u64 c = moves & kCornerMask;
  return c ? (c & (0ULL - c)) : (moves & (0ULL - moves));
}

// Searches one position to `depth` plies (kMinDepth..kMaxDepth) with the
// caller's frames (depth of them) and move lists (depth - 3 rows of
// kMaxMoves).  Returns the value for the side to move; *best = its move
// (64 = pass); *nodes = root, children, pass frames and leaves.
GPO_HD int search(u64 P0, u64 O0, int depth, const EvalMeta& m, const unsigned* digits,
                  const float* values, Frame* fr, unsigned char (*lists)[kMaxMoves], int* best,
                  unsigned long long* nodes_out) {
  enum { OPEN, STEP, COMMIT };
  const int upper = depth - 3;
  unsigned long long nodes = 0;
  int level = 0, state = OPEN, score = 0;
  u64 P = P0, O = O0;
  int alpha = -64, beta = 64;
  for (;;) {
    Frame& f = fr[level];
    if (state == OPEN) {
      ++nodes;
      f.P = P;
      f.O = O;
      f.alpha = alpha;
      f.beta = beta;
      f.passed = 0;
      f.best = kMoveNone;
      state = STEP;
      bool none;
      if (level < upper) {
        f.result = -65;
        f.idx = 0;
        f.n = upper_moves(P, O, lists[level]);
        none = f.n == 0;
      } else {
        f.result = -32767;
        f.moves = mobility(P, O);
        none = f.moves == 0;
      }
      if (none) {  // pass in place
        ++nodes;
        f.passed = 1;
        f.P = O;
        f.O = P;
        f.alpha = -beta;
        f.beta = -alpha;
        if (level < upper) {
          f.result = -65;
          f.n = upper_moves(f.P, f.O, lists[level]);
          none = f.n == 0;
        } else {
          f.moves = mobility(f.P, f.O);
          none = f.moves == 0;
        }
        if (none) {  // neither side can move: the game is over
          f.result = final_score(f.P, f.O);
          state = COMMIT;
        }
      }
      continue;
    }
    if (state == STEP) {
      int sq = -1;
      if (level < upper) {
        if (f.idx < f.n && f.alpha < f.beta) sq = lists[level][f.idx++];
      } else if (f.moves && f.alpha < f.beta) {
        const u64 bit = scan_pick(f.moves);
        f.moves ^= bit;
        sq = lowest_square(bit);
      }
      if (sq < 0) {
        state = COMMIT;
        continue;
      }
      const u64 bit = 1ULL << sq;
      const u64 fl = flips(f.P, f.O, sq);
      const u64 cP = f.O ^ fl, cO = f.P ^ fl ^ bit;
      if (level == depth - 1) {  // the position reached is a leaf
        ++nodes;
        const int v = -leaf_value(cP, cO, m, digits, values);
        if (v > f.result) f.result = v;
        if (f.result > f.alpha) f.alpha = f.result;
        continue;
      }
      P = cP;
      O = cO;
      alpha = -f.beta;
      beta = -f.alpha;
      ++level;
      state = OPEN;
      continue;
    }
    // COMMIT: hand this node's value to its parent
    const int v = f.passed ? f.result : -f.result;
    if (level == 0) {
      score = f.passed ? -f.result : f.result;
      *best = f.passed ? kMovePass : f.best;
      break;
    }
    --level;
    Frame& g = fr[level];
    if (level < upper) {
      if (v > g.result) {
        g.result = v;
        g.best = lists[level][g.idx - 1];
        if (g.result > g.alpha) g.alpha = g.result;
      }
    } else {
      if (v > g.result) g.result = v;
      if (g.result > g.alpha) g.alpha = g.result;
    }
    state = STEP;
  }
  *nodes_out = nodes;
  return score;
}

}  // namespace think
}  // namespace gpo

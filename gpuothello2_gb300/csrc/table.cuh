// Lock-free transposition table with 128-bit CAS entries (the role of the
// reference's Table, table.cuh:16-66 / table.cu:36-86, whose call sites are
// commented out in its search, solver.cu:119-144, 182).
//
// 2^bits entries of 16 bytes in 2^(bits-1) buckets of two (one 32-byte
// sector).  A position may sit in either entry of its bucket; a store for a
// new position takes an empty entry, else evicts the entry whose position has
// fewer empty squares (a smaller subtree, cheaper to search again; the
// second entry on a tie).  Tens of thousands of searches run at once and
// share the table, so without this preference the many entries of small
// subtrees would keep evicting the few of large ones; one entry of a bucket
// takes the churn while the other keeps the larger subtree.  Every store
// evicts something, so entries of finished positions never block a bucket.
//
// Key: a bijective map of the position (P, O) to two words, cheap to
// compute: x = P * K1 (odd K1, invertible mod 2^64) and
// y = (O ^ rotl(x, 32)) * K2 (invertible in O for a given x).  The high
// bits - 1 bits of y index the bucket (the high bits of a product depend on
// every bit of its factor, so on every square of both sides); an entry
// stores x and the remaining low bits of y, which with the bucket index give
// back (P, O) exactly: no false hits, unlike a truncated hash, for any
// bits >= 17.  The inverse map also gives a stored entry's empty count for
// the eviction choice, so none is stored.  Entry: word 0 = x, word 1 =
// (y low bits) << 16 | (lower + 64) << 8 | (upper + 64).  All zero = empty; a
// position whose entry would be all zero is simply never found (a miss is
// always safe).
//
// Entries are read and written only with atom.global.cas.b128, so a reader
// never sees half of one write and half of another.  A read is a CAS of
// zero by zero (it can only rewrite an empty entry with itself); a write
// retries a few times and then gives up -- the table is a cache.
#pragma once
#include "common.cuh"

namespace gpo {

constexpr u64 kTTK1 = 0x9E3779B97F4A7C15ULL, kTTK1inv = 0xF1DE83E19937733DULL;
constexpr u64 kTTK2 = 0xD6E8FEB86659FD93ULL, kTTK2inv = 0xCFEE444D8B59A89BULL;

struct TTKey {
  u64 x, y;
};

__device__ __forceinline__ u64 tt_rot32(u64 v) { return (v << 32) | (v >> 32); }

__device__ __forceinline__ TTKey tt_key(u64 P, u64 O) {
  const u64 x = P * kTTK1;
  return TTKey{x, (O ^ tt_rot32(x)) * kTTK2};
}

// bucket index (the high bits - 1 bits of y) and tag (the rest of y)
__device__ __forceinline__ size_t tt_bucket(const TTKey& k, int bits) {
  return static_cast<size_t>(k.y >> (65 - bits));
}
__device__ __forceinline__ u64 tt_tag(const TTKey& k, int bits) {
  return (k.y << (bits - 1)) >> (bits - 1);
}

// Empty squares of the position an entry of bucket b holds (the key map
// inverted).
__device__ __forceinline__ int tt_entry_empties(u64 w0, u64 w1, size_t b, int bits) {
  const u64 y = (static_cast<u64>(b) << (65 - bits)) | (w1 >> 16);
  const u64 P = w0 * kTTK1inv;
  const u64 O = (y * kTTK2inv) ^ tt_rot32(w0);
  return 64 - popc(P | O);
}

__device__ __forceinline__ void tt_cas128(u64* addr, u64 c0, u64 c1, u64 v0, u64 v1, u64& o0,
                                          u64& o1) {
#ifdef GPO_SIMT_EMU  // the CPU emulation of the search used by the tests
  gpo_emu_cas128(addr, c0, c1, v0, v1, o0, o1);
#else
  asm volatile(
      "{\n\t.reg .b128 c, v, d;\n\t"
      "mov.b128 c, {%2, %3};\n\t"
      "mov.b128 v, {%4, %5};\n\t"
      "atom.global.cas.b128 d, [%6], c, v;\n\t"
      "mov.b128 {%0, %1}, d;\n\t}"
      : "=l"(o0), "=l"(o1)
      : "l"(c0), "l"(c1), "l"(v0), "l"(v1), "l"(addr)
      : "memory");
#endif
}

__device__ __forceinline__ bool tt_same(const TTKey& k, int bits, u64 w0, u64 w1) {
  return w0 == k.x && (w1 >> 16) == tt_tag(k, bits) && (w0 | w1) != 0;
}

// Bounds stored for the position, or false.
__device__ __forceinline__ bool tt_probe(u64* table, int bits, const TTKey& k, int& lower,
                                         int& upper) {
  u64* e = table + 4 * tt_bucket(k, bits);
  for (int j = 0; j < 2; ++j) {
    u64 w0, w1;
    tt_cas128(e + 2 * j, 0, 0, 0, 0, w0, w1);
    if (tt_same(k, bits, w0, w1)) {
      lower = static_cast<int>((w1 >> 8) & 0xff) - 64;
      upper = static_cast<int>(w1 & 0xff) - 64;
      return true;
    }
  }
  return false;
}

// Records lower <= value <= upper for the position, merging with what its
// entry already holds; otherwise takes an empty entry of the bucket or
// evicts the one with fewer empties.
__device__ __forceinline__ bool tt_store(u64* table, int bits, const TTKey& k, int lower,
                                         int upper) {
  const size_t b = tt_bucket(k, bits);
  u64* bucket = table + 4 * b;
  const u64 tag = tt_tag(k, bits) << 16;
  u64 a0, a1, b0, b1;
  tt_cas128(bucket, 0, 0, 0, 0, a0, a1);
  tt_cas128(bucket + 2, 0, 0, 0, 0, b0, b1);
  int j;
  u64 c0, c1;
  if (tt_same(k, bits, a0, a1)) {
    j = 0;
  } else if (tt_same(k, bits, b0, b1)) {
    j = 1;
  } else if ((a0 | a1) == 0) {
    j = 0;
  } else if ((b0 | b1) == 0) {
    j = 1;
  } else {
    j = tt_entry_empties(a0, a1, b, bits) < tt_entry_empties(b0, b1, b, bits) ? 0 : 1;
  }
  c0 = j ? b0 : a0;
  c1 = j ? b1 : a1;
  u64* e = bucket + 2 * j;
  for (int attempt = 0; attempt < 4; ++attempt) {
    int lo = lower, up = upper;
    if (tt_same(k, bits, c0, c1)) {
      const int ol = static_cast<int>((c1 >> 8) & 0xff) - 64;
      const int ou = static_cast<int>(c1 & 0xff) - 64;
      if (ol > lo) lo = ol;
      if (ou < up) up = ou;
      if (lo > up) {  // cannot happen for exact searches; keep the new bounds
        lo = lower;
        up = upper;
      }
    }
    const u64 v1 = tag | (static_cast<u64>(lo + 64) << 8) | static_cast<u64>(up + 64);
    u64 o0, o1;
    tt_cas128(e, c0, c1, k.x, v1, o0, o1);
    if (o0 == c0 && o1 == c1) return true;
    c0 = o0;
    c1 = o1;
  }
  return false;
}

}  // namespace gpo

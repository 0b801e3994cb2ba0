// Lock-free transposition table with 128-bit CAS entries (the role of the
// reference's Table, table.cuh:16-66 / table.cu:36-86, whose call sites are
// commented out in its search, solver.cu:119-144, 182).
//
// Key: a bijective map of the position (P, O) to two words, cheap to
// compute: x = P * K1 (odd K1, invertible mod 2^64) and
// y = (O ^ rotl(x, 32)) * K2 (invertible in O for a given x).  The high
// `bits` bits of y index the table (the high bits of a product depend on
// every bit of its factor, so on every square of both sides); the entry
// stores x and the low 64 - bits bits of y, which with the index give back
// (P, O) exactly: no false hits, unlike a truncated hash, for any
// bits >= 16.  Entry: word 0 = x, word 1 = (y low bits) << 16 |
// (lower + 64) << 8 | (upper + 64).  All zero = empty; a position whose
// entry would be all zero is simply never found (a miss is always safe).
//
// Entries are read and written only with atom.global.cas.b128, so a reader
// never sees half of one write and half of another.  A read is a CAS of
// zero by zero (it can only rewrite an empty entry with itself); a write
// retries a few times and then gives up -- the table is a cache.
#pragma once
#include "common.cuh"

namespace gpo {

struct TTKey {
  u64 x, y;
};

__device__ __forceinline__ TTKey tt_key(u64 P, u64 O) {
  const u64 x = P * 0x9E3779B97F4A7C15ULL;
  const u64 r = (x << 32) | (x >> 32);
  return TTKey{x, (O ^ r) * 0xD6E8FEB86659FD93ULL};
}

__device__ __forceinline__ size_t tt_index(const TTKey& k, int bits) {
  return static_cast<size_t>(k.y >> (64 - bits));
}
__device__ __forceinline__ u64 tt_tag(const TTKey& k, int bits) {
  return (k.y << bits) >> bits;  // the low 64 - bits bits of y
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
  u64* e = table + 2 * tt_index(k, bits);
  u64 w0, w1;
  tt_cas128(e, 0, 0, 0, 0, w0, w1);
  if (!tt_same(k, bits, w0, w1)) return false;
  lower = static_cast<int>((w1 >> 8) & 0xff) - 64;
  upper = static_cast<int>(w1 & 0xff) - 64;
  return true;
}

// Records lower <= value <= upper for the position, merging with what the
// entry already holds for it; replaces an entry of another position.
__device__ __forceinline__ bool tt_store(u64* table, int bits, const TTKey& k, int lower,
                                         int upper) {
  u64* e = table + 2 * tt_index(k, bits);
  const u64 tag = tt_tag(k, bits) << 16;
  u64 c0 = 0, c1 = 0;
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

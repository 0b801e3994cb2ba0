// Lock-free transposition table with 128-bit CAS entries (the role of the
// reference's Table, table.cuh:16-66 / table.cu:36-86, whose call sites are
// commented out in its search, solver.cu:119-144, 182).
//
// Key: a bijective 128-bit mix (three Feistel rounds) of the position
// (P, O).  Its low `bits` bits index the table; the remaining 128 - bits bits
// are stored, so an entry names exactly one position (no false hits, unlike
// a truncated hash) as long as bits >= 16.  Entry: word 0 = mix high half,
// word 1 = (mix low half >> bits) << 16 | (lower + 64) << 8 | (upper + 64).
// All zero = empty.
//
// Entries are read and written only with atom.global.cas.b128, so a reader
// never sees half of one write and half of another.  A read is a CAS of
// zero by zero (it can only rewrite an empty entry with itself); a write
// retries a few times and then gives up -- the table is a cache.
#pragma once
#include "common.cuh"

namespace gpo {

__device__ __forceinline__ u64 tt_mix64(u64 x) {
  x ^= x >> 31;
  x *= 0x7fb5d329728ea185ULL;
  x ^= x >> 27;
  x *= 0x81dadef4bc2dd44dULL;
  x ^= x >> 33;
  return x;
}

struct TTKey {
  u64 hi, lo;
};

__device__ __forceinline__ TTKey tt_key(u64 P, u64 O) {
  u64 a = P, b = O;
  b ^= tt_mix64(a);
  a ^= tt_mix64(b);
  b ^= tt_mix64(a);
  return TTKey{a, b};
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
  return w0 == k.hi && (w1 >> 16) == (k.lo >> bits) && (w0 | w1) != 0;
}

// Bounds stored for the position, or false.
__device__ __forceinline__ bool tt_probe(u64* table, int bits, const TTKey& k, int& lower,
                                         int& upper) {
  u64* e = table + 2 * (k.lo & ((1ULL << bits) - 1));
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
  u64* e = table + 2 * (k.lo & ((1ULL << bits) - 1));
  const u64 tag = (k.lo >> bits) << 16;
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
    tt_cas128(e, c0, c1, k.hi, v1, o0, o1);
    if (o0 == c0 && o1 == c1) return true;
    c0 = o0;
    c1 = o1;
  }
  return false;
}

}  // namespace gpo

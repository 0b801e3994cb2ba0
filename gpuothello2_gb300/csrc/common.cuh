// Shared definitions for the solver kernels and the C-ABI layer.
#pragma once
#include <cstdint>

#include "bitboard.cuh"

namespace gpo {

// Largest empty count a position may have (stack sizing).  Every kernel
// rejects a position with more empties than the call's depth, and the
// C-ABI rejects depth > GPO_MAX_EMPTIES.
constexpr int kMaxEmpties = 32;

constexpr u64 kCorners = 0x8100000000000081ULL;

// Best-move codes (the reference's hand::PASS / hand::NOMOVE, alphabeta.cuh:7-10).
constexpr int kMovePassDev = 64;
constexpr int kMoveNoneDev = 65;
// Score of a position the batched kernel handed back unsolved (tail handoff):
// outside every real score's range [-64, 64].
constexpr int kUnsolvedDev = -128;

// Error bits set by kernels in the device status word (host maps them to
// the negative GPO_ERR_* codes of the C-ABI).
enum : unsigned int {
  kErrDepth = 1u << 0,     // a position has more empties than `depth`
  kErrOverlap = 1u << 1,   // a square is set in both bitboards
  kErrBudget = 1u << 2,    // a search hit the per-position node budget
  kErrTable = 1u << 3,     // a table update gave up after its retry limit
  kErrInternal = 1u << 4,  // stack index out of range (never expected)
  kErrWait = 1u << 5,      // the search launch ran past its deadline
};

// Per-launch device counters (one instance in device memory per context).
struct DeviceStats {
  unsigned long long nodes;
  unsigned long long tt_probes;
  unsigned long long tt_hits;
  unsigned long long tt_updates;
  unsigned long long learned_calls;
  unsigned long long handouts;   // moves of split nodes searched by helper lanes
  unsigned long long stab_cuts;  // nodes closed by the stability cutoff
  unsigned int status;
  unsigned int next;             // work-queue cursor of the persistent kernel
  unsigned int done;             // input positions finished (solved, rejected or handed back)
  unsigned int handed;           // input positions handed back unsolved (tail handoff)
  unsigned long long t0;         // plain kernel: global timer at its first block's start
};

// The GPU's global nanosecond timer (launch deadlines).
__device__ __forceinline__ unsigned long long gpo_global_ns() {
#ifdef GPO_SIMT_EMU  // the CPU emulation of the kernels used by the tests
  return gpo_emu_ns();
#else
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
#endif
}

__device__ __forceinline__ int ctz64(u64 x) { return __ffsll(static_cast<long long>(x)) - 1; }

// Warp-level sum of a 64-bit counter, one atomic per warp.  Must be called
// by all 32 lanes of the warp together (kernels call it after their loops,
// where every lane has arrived).
__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

}  // namespace gpo

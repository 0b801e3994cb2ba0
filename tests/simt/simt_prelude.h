// SIMT emulation of CUDA kernels on the CPU (test infrastructure only).
//
// Force-included ahead of a kernel source compiled as host C++: every CUDA
// thread of one block runs as a std::thread; warp collectives (__ballot_sync,
// __any_sync, __shfl_sync, __shfl_down_sync) meet at a per-warp barrier, so
// the 32 lanes of a warp agree on every collective exactly as on the GPU;
// __syncthreads is a block barrier; atomics are the compiler's __atomic
// builtins on the same addresses; dynamic shared memory is one array for
// the block (the emulation runs a grid of one block).  The two inline-PTX
// sites of the solver (the global timer and the 128-bit CAS) take host
// versions under GPO_SIMT_EMU.
//
// This lets the tests run the batched search kernel's own source on a
// machine without a GPU and check it against the oracle.  It is not a
// performance model and it never runs in the product.
#pragma once
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <algorithm>
#include <thread>

#define GPO_SIMT_EMU 1
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __launch_bounds__(...)
#define __shared__
#define __align__(n) __attribute__((aligned(n)))

struct simt_uint3 {
  unsigned x, y, z;
};
extern thread_local simt_uint3 threadIdx, blockIdx;
extern simt_uint3 blockDim, gridDim;

struct alignas(16) ulonglong2 {
  unsigned long long x, y;
};

// Phase-counting barrier whose waiters yield the CPU: the emulation runs
// more threads than cores, and a sleeping (futex) barrier makes every
// collective cost several scheduler round trips.
struct SimtBarrier {
  explicit SimtBarrier(int parties) : n(parties) {}
  void arrive_and_wait() {
    const unsigned ph = phase.load(std::memory_order_acquire);
    if (count.fetch_add(1, std::memory_order_acq_rel) == n - 1) {
      count.store(0, std::memory_order_relaxed);
      phase.fetch_add(1, std::memory_order_acq_rel);
    } else {
      while (phase.load(std::memory_order_acquire) == ph) std::this_thread::yield();
    }
  }
  const int n;
  std::atomic<int> count{0};
  std::atomic<unsigned> phase{0};
};

struct SimtWarp {
  SimtBarrier* bar;
  unsigned long long slot[32];
};
extern thread_local SimtWarp* simt_warp;
extern SimtBarrier* simt_block;

inline unsigned long long simt_gather(unsigned long long v, int src) {
  SimtWarp& w = *simt_warp;
  w.slot[threadIdx.x & 31] = v;
  w.bar->arrive_and_wait();
  const unsigned long long r = w.slot[src & 31];
  w.bar->arrive_and_wait();
  return r;
}

inline unsigned __ballot_sync(unsigned, int pred) {
  SimtWarp& w = *simt_warp;
  w.slot[threadIdx.x & 31] = pred ? 1 : 0;
  w.bar->arrive_and_wait();
  unsigned r = 0;
  for (int i = 0; i < 32; ++i)
    if (w.slot[i]) r |= 1u << i;
  w.bar->arrive_and_wait();
  return r;
}
inline int __any_sync(unsigned mask, int pred) { return __ballot_sync(mask, pred) != 0; }
inline unsigned __shfl_sync(unsigned, unsigned v, int src) {
  return static_cast<unsigned>(simt_gather(v, src));
}
inline unsigned long long __shfl_down_sync(unsigned, unsigned long long v, unsigned d) {
  const int lane = threadIdx.x & 31;
  const int src = lane + static_cast<int>(d) < 32 ? lane + static_cast<int>(d) : lane;
  return simt_gather(v, src);
}
inline unsigned long long __shfl_sync(unsigned, unsigned long long v, int src) {
  return simt_gather(v, src);
}
inline int __shfl_sync(unsigned, int v, int src) {
  return static_cast<int>(static_cast<unsigned>(simt_gather(static_cast<unsigned>(v), src)));
}
inline void __syncwarp(unsigned = 0xffffffffu) { simt_warp->bar->arrive_and_wait(); }
inline void __syncthreads() { simt_block->arrive_and_wait(); }
inline void __threadfence() { __atomic_thread_fence(__ATOMIC_SEQ_CST); }
inline void __nanosleep(unsigned) { std::this_thread::yield(); }

inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __popcll(unsigned long long x) { return __builtin_popcountll(x); }
inline int __ffs(int x) { return __builtin_ffs(x); }
inline int __ffsll(long long x) { return __builtin_ffsll(x); }
inline int __clz(int x) { return x ? __builtin_clz(static_cast<unsigned>(x)) : 32; }
using std::min;
using std::max;
inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b) {
  return static_cast<unsigned long long>((static_cast<unsigned __int128>(a) * b) >> 64);
}
inline unsigned long long __brevll(unsigned long long x) {
  unsigned long long r = 0;
  for (int i = 0; i < 64; ++i) r |= ((x >> i) & 1ULL) << (63 - i);
  return r;
}
template <class T>
inline T __ldcg(const T* p) {
  return __atomic_load_n(p, __ATOMIC_SEQ_CST);
}

inline unsigned atomicAdd(unsigned* p, unsigned v) {
  return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);
}
inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) {
  return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);
}
inline unsigned atomicSub(unsigned* p, unsigned v) {
  return __atomic_fetch_sub(p, v, __ATOMIC_SEQ_CST);
}
inline unsigned atomicOr(unsigned* p, unsigned v) {
  return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST);
}
inline unsigned atomicExch(unsigned* p, unsigned v) {
  return __atomic_exchange_n(p, v, __ATOMIC_SEQ_CST);
}
inline unsigned atomicCAS(unsigned* p, unsigned cmp, unsigned v) {
  __atomic_compare_exchange_n(p, &cmp, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return cmp;
}
inline unsigned long long atomicCAS(unsigned long long* p, unsigned long long cmp,
                                    unsigned long long v) {
  __atomic_compare_exchange_n(p, &cmp, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return cmp;
}
inline unsigned atomicMax(unsigned* p, unsigned v) {
  unsigned old = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (old < v &&
         !__atomic_compare_exchange_n(p, &old, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
  }
  return old;
}

// host versions of the two inline-PTX sites
inline unsigned long long gpo_emu_ns() {
  return static_cast<unsigned long long>(std::chrono::duration_cast<std::chrono::nanoseconds>(
      std::chrono::steady_clock::now().time_since_epoch()).count());
}
extern std::mutex simt_cas128_mutex;
inline void gpo_emu_cas128(unsigned long long* addr, unsigned long long c0, unsigned long long c1,
                           unsigned long long v0, unsigned long long v1, unsigned long long& o0,
                           unsigned long long& o1) {
  std::lock_guard<std::mutex> lock(simt_cas128_mutex);
  o0 = addr[0];
  o1 = addr[1];
  if (o0 == c0 && o1 == c1) {
    addr[0] = v0;
    addr[1] = v1;
  }
}

// ---- kernel launches ----
// Runs `body` as one block of `threads` CPU threads (block index `b` of a
// grid of `grid`): each thread gets its thread index, its warp's barrier
// and the block barrier.  Blocks of an ordinary launch run one after
// another, so a kernel's static __shared__ arrays are the block's.
#include <functional>
#include <memory>
#include <tuple>
#include <vector>

inline void simt_run_block(unsigned b, unsigned grid, unsigned threads,
                           const std::function<void()>& body) {
  blockDim = {threads, 1, 1};
  gridDim = {grid, 1, 1};
  SimtBarrier block(static_cast<int>(threads));
  simt_block = &block;
  const unsigned warps = (threads + 31) / 32;
  std::vector<std::unique_ptr<SimtBarrier>> bars;
  std::vector<SimtWarp> ws(warps);
  for (unsigned w = 0; w < warps; ++w) {
    bars.emplace_back(new SimtBarrier(32));
    ws[w].bar = bars.back().get();
  }
  std::vector<std::thread> ts;
  for (unsigned t = 0; t < threads; ++t) {
    ts.emplace_back([&, t] {
      threadIdx = {t, 0, 0};
      blockIdx = {b, 0, 0};
      simt_warp = &ws[t / 32];
      body();
    });
  }
  for (auto& th : ts) th.join();
}

struct SimtCfg {
  unsigned grid, block;
};
template <class G, class B, class... Rest>
inline SimtCfg simt_cfg(G grid, B block, Rest...) {
  return SimtCfg{static_cast<unsigned>(grid), static_cast<unsigned>(block)};
}

template <class... KP, class... A>
inline void simt_launch(void (*kernel)(KP...), SimtCfg c, A&&... a) {
  std::tuple<KP...> args(std::forward<A>(a)...);
  for (unsigned b = 0; b < c.grid; ++b)
    simt_run_block(b, c.grid, c.block, [&] { std::apply(kernel, args); });
}

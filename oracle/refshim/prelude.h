/*
 * Host prelude for compiling the reference solver's CUDA sources as plain
 * C++ on the CPU (test infrastructure only; nothing here ships).
 *
 * The reference search (solver.cu:1-311, board.cu, node.cuh, table.cu) is
 * written as CUDA device code but uses no device-only feature except thread
 * indices, shared-memory declarations, a few intrinsics and 32/64-bit
 * atomics.  Force-included ahead of those files (g++ -include prelude.h),
 * this header maps each of them onto a single-threaded host equivalent so
 * that the reference's own state machine runs unchanged on one CPU thread:
 *
 *   - __host__/__device__/__global__/__shared__/__constant__ expand to
 *     nothing, so kernels become ordinary functions;
 *   - threadIdx/blockIdx/blockDim/gridDim are process globals set by the
 *     harness (one block of one thread, so the kernel's per-block atomic
 *     fetch hands out problems 0,1,2,... in order);
 *   - atomics, __threadfence and __syncthreads are the sequential no-race
 *     versions;
 *   - the CUDA runtime calls used by the host halves of those files
 *     (cudaMalloc*, cudaMemcpy, cudaMemset, streams) are backed by malloc.
 *
 * The evaluator and think-mode search (eval.cu, thinker.cu) are compiled
 * the same way; eval.cu with __CUDA_ARCH__ defined, so that its device
 * branch (the software bit-extract loop and __ldg loads, eval.cu:67-79,
 * 115-139) is the code emulated, as on the GPU.
 *
 * The device intrinsics __popcll/__clzll are only reached through
 * `#ifdef __CUDA_ARCH__` branches or solver.cu:85; they are restated with
 * the GCC builtins and clz(0) defined as 64.
 */
#pragma once
#include <algorithm>
#include <cassert>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#define __host__
#define __device__
#define __global__
#define __shared__
#define __constant__
#define __forceinline__ inline

using std::max;
using std::min;
/* CUDA's math headers also overload min/max for mixed double/float
 * arguments, returning double; the evaluator's clamp (eval.cu:140) uses
 * them.  Same-type calls still resolve to std::min/std::max. */
inline double max(double a, double b) { return a > b ? a : b; }
inline double min(double a, double b) { return a < b ? a : b; }

/* Read-only-cache load (eval.cu:119-136): a plain load on one CPU thread. */
template <class T>
inline T __ldg(const T* p) {
  return *p;
}

struct refshim_dim3 {
  unsigned int x, y, z;
};
extern refshim_dim3 threadIdx, blockIdx, blockDim, gridDim;

inline int __popcll(unsigned long long x) { return __builtin_popcountll(x); }

/* __clzll(0) is 64 on the device, and the one place the reference shifts by
 * its result (board.cu:33, `0x8000000000000000ULL >> __clzll(...)`) then
 * relies on the PTX rule that a 64-bit logical shift by 64 or more yields 0.
 * In host C++ that shift is undefined (x86 masks the count to 0), so the
 * count is returned as a small type whose `>>` applies the PTX rule.
 * board.cu is compiled with __CUDA_ARCH__ defined so that its device branch
 * -- the code the GPU runs -- is the one emulated; its host branch calls
 * __builtin_clzll(0), which is undefined, when a whole ray is opponent discs. */
struct refshim_clz {
  int n;
  operator int() const { return n; }
};
inline refshim_clz __clzll(long long x) {
  return refshim_clz{x == 0 ? 64 : __builtin_clzll(static_cast<unsigned long long>(x))};
}
inline unsigned long long operator>>(unsigned long long x, refshim_clz c) {
  return c.n >= 64 ? 0ULL : (x >> c.n);
}

inline unsigned int atomicAdd(unsigned int* p, unsigned int v) {
  unsigned int old = *p;
  *p = old + v;
  return old;
}
inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) {
  unsigned long long old = *p;
  *p = old + v;
  return old;
}
inline int atomicCAS(int* p, int cmp, int val) {
  int old = *p;
  if (old == cmp) *p = val;
  return old;
}
inline int atomicExch(int* p, int val) {
  int old = *p;
  *p = val;
  return old;
}
inline void __threadfence() {}
inline void __syncthreads() {}

/* Minimal CUDA runtime surface used by solver.cu:313-348 and table.cu. */
typedef int cudaError_t;
typedef void* cudaStream_t;
enum refshim_memcpy_kind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3
};
static const cudaError_t cudaSuccess = 0;
static const cudaError_t cudaErrorNotReady = 600;

inline cudaError_t cudaMalloc(void** p, size_t n) {
  *p = std::calloc(n ? n : 1, 1);
  return *p ? cudaSuccess : 2;
}
inline cudaError_t cudaMallocManaged(void** p, size_t n) { return cudaMalloc(p, n); }
inline cudaError_t cudaFree(void* p) {
  std::free(p);
  return cudaSuccess;
}
inline cudaError_t cudaMemset(void* p, int v, size_t n) {
  std::memset(p, v, n);
  return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, int) {
  std::memcpy(d, s, n);
  return cudaSuccess;
}
inline cudaError_t cudaStreamCreate(cudaStream_t* s) {
  *s = nullptr;
  return cudaSuccess;
}
inline cudaError_t cudaStreamDestroy(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaStreamQuery(cudaStream_t) { return cudaSuccess; }

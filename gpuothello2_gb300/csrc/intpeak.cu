// INT32 issue-rate microbenchmark: the integer-ALU roofline denominator.
//
// The search is bound by 32-bit integer logic/shift/add instructions (a
// 64-bit bitboard operation is two of them).  This kernel issues long
// chains of independent lop3.b32 (3-input logic) or add.u32 instructions
// from every thread of a full grid and reports instructions per second.
// Built as its own small library (libgpo_intpeak.so); not part of the
// solver's C ABI.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

template <int kOp>
__global__ void int_chain_kernel(unsigned seed, unsigned* sink) {
  unsigned a[kChains];
  const unsigned b = seed * 0x9E3779B9u + threadIdx.x, c = seed ^ blockIdx.x;
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = seed + k * 7919u + threadIdx.x;
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
      if (kOp == 0)
        asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[k]) : "r"(b), "r"(c));
      else
        asm volatile("add.u32 %0, %0, %1;" : "+r"(a[k]) : "r"(b));
    }
  }
  unsigned x = 0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) x ^= a[k];
  if (x == 0x12345678u) sink[0] = x;  // keeps the chains alive
}

}  // namespace

extern "C" int gpo_int_peak(int op, double* ops_per_s, double* ms_out) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  unsigned* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(unsigned)) != cudaSuccess) return -1;
  const int threads = 256, blocks = sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&](unsigned s) {
    if (op == 0)
      int_chain_kernel<0><<<blocks, threads>>>(s, sink);
    else
      int_chain_kernel<1><<<blocks, threads>>>(s, sink);
  };
  for (int w = 0; w < 3; ++w) launch(w);
  cudaEventRecord(e0);
  const int reps = 10;
  for (int r = 0; r < reps; ++r) launch(100 + r);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const double ops = static_cast<double>(blocks) * threads * kChains * kIters * reps;
  *ops_per_s = ops / (ms * 1e-3);
  if (ms_out) *ms_out = ms / reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

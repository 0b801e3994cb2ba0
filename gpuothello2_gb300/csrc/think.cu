// Think mode and the pattern evaluator on the GPU, and their C ABI.
// Replaces BatchedThinkTask / think_kernel (thinker.cuh:9-29,
// thinker.cu:336-389) and Evaluator (eval.cuh:5-17, eval.cu:12-141); the
// search and evaluation themselves are in think.cuh.
//
// Layout: one thread per position.  Each block first copies the evaluator's
// metadata and its per-byte digit tables (npairs x 1 KB) into shared
// memory; the value tables (3^k floats per feature, about 1.4 MB for a
// 13-pattern set) stay in global memory and are read through the read-only
// path, so after the first leaves they are served from L2.  Search frames
// live in per-thread local memory (depth x 48 B plus depth-3 move lists of
// 64 B).  Positions are independent: no waits, no atomics but the status
// word.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gpuothello2.h"
#include "common.cuh"
#include "evalfile.h"
#include "think.cuh"

namespace gpo {
namespace {

using think::EvalMeta;

constexpr int kThinkBlock = 128;

__device__ void load_eval(const EvalMeta* meta, const unsigned* digits, EvalMeta* s_meta,
                          unsigned* s_digits) {
  if (threadIdx.x == 0) *s_meta = *meta;
  const int words = meta->npairs * 256;
  for (int i = threadIdx.x; i < words; i += blockDim.x) s_digits[i] = digits[i];
  __syncthreads();
}

__global__ void __launch_bounds__(kThinkBlock)
eval_kernel(const u64* __restrict__ player, const u64* __restrict__ opp, int n,
            const EvalMeta* __restrict__ meta, const unsigned* __restrict__ digits,
            const float* __restrict__ values, float* __restrict__ out,
            unsigned* __restrict__ status) {
  extern __shared__ unsigned s_digits[];
  __shared__ EvalMeta s_meta;
  load_eval(meta, digits, &s_meta, s_digits);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const u64 P = player[i], O = opp[i];
  if (P & O) {  // a base-3 digit would be 3: outside the tables
    atomicOr(status, kErrOverlap);
    out[i] = 0.0f;
    return;
  }
  out[i] = think::evaluate(P, O, s_meta, s_digits, values);
}

__global__ void __launch_bounds__(kThinkBlock)
think_kernel(const u64* __restrict__ player, const u64* __restrict__ opp, int n, int depth,
             const EvalMeta* __restrict__ meta, const unsigned* __restrict__ digits,
             const float* __restrict__ values, signed char* __restrict__ score,
             signed char* __restrict__ best, unsigned long long* __restrict__ nodes_out,
             unsigned long long* __restrict__ nodes_total, unsigned* __restrict__ status) {
  extern __shared__ unsigned s_digits[];
  __shared__ EvalMeta s_meta;
  load_eval(meta, digits, &s_meta, s_digits);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long nodes = 0;
  if (i < n) {
    const u64 P = player[i], O = opp[i];
    if (P & O) {
      atomicOr(status, kErrOverlap);
      score[i] = 0;
      if (best) best[i] = think::kMoveNone;
    } else {
      think::Frame fr[think::kMaxDepth];
      unsigned char lists[think::kMaxDepth - 3][think::kMaxMoves];
      int bm = think::kMoveNone;
      const int v = think::search(P, O, depth, s_meta, s_digits, values, fr, lists, &bm, &nodes);
      score[i] = static_cast<signed char>(v);
      if (best) best[i] = static_cast<signed char>(bm);
    }
    if (nodes_out) nodes_out[i] = nodes;
  }
  if (nodes) atomicAdd(nodes_total, nodes);
}

// Evaluator and buffers of the think entry points (their own lock and
// stream: think mode never runs inside a solve call).
struct ThinkState {
  bool loaded = false;
  int npairs = 0;
  EvalMeta* dMeta = nullptr;
  unsigned* dDigits = nullptr;
  float* dValues = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  size_t cap = 0;
  u64* dP = nullptr;
  u64* dO = nullptr;
  signed char* dScore = nullptr;
  signed char* dBest = nullptr;
  unsigned long long* dNodes = nullptr;
  float* dEval = nullptr;
  unsigned long long* dTotal = nullptr;
  unsigned* dStatus = nullptr;
};

std::mutex g_think_mutex;
ThinkState g_think;

int fail(cudaError_t e) { return e == cudaErrorMemoryAllocation ? GPO_ERR_NOMEM : GPO_ERR_CUDA; }

#define TH_CK(call)                               \
  do {                                            \
    const cudaError_t e_ = (call);                \
    if (e_ != cudaSuccess) return fail(e_);       \
  } while (0)

int ensure_think(size_t n) {
  ThinkState& t = g_think;
  if (!t.stream) {
    TH_CK(cudaStreamCreateWithFlags(&t.stream, cudaStreamNonBlocking));
    TH_CK(cudaEventCreate(&t.ev0));
    TH_CK(cudaEventCreate(&t.ev1));
    TH_CK(cudaMalloc(&t.dTotal, sizeof(unsigned long long)));
    TH_CK(cudaMalloc(&t.dStatus, sizeof(unsigned)));
  }
  if (n <= t.cap) return GPO_OK;
  cudaFree(t.dP);
  cudaFree(t.dO);
  cudaFree(t.dScore);
  cudaFree(t.dBest);
  cudaFree(t.dNodes);
  cudaFree(t.dEval);
  t.dP = t.dO = nullptr;
  t.dScore = t.dBest = nullptr;
  t.dNodes = nullptr;
  t.dEval = nullptr;
  t.cap = 0;
  size_t cap = 1024;
  while (cap < n) cap *= 2;
  TH_CK(cudaMalloc(&t.dP, cap * sizeof(u64)));
  TH_CK(cudaMalloc(&t.dO, cap * sizeof(u64)));
  TH_CK(cudaMalloc(&t.dScore, cap));
  TH_CK(cudaMalloc(&t.dBest, cap));
  TH_CK(cudaMalloc(&t.dNodes, cap * sizeof(unsigned long long)));
  TH_CK(cudaMalloc(&t.dEval, cap * sizeof(float)));
  t.cap = cap;
  return GPO_OK;
}

size_t eval_smem(int npairs) { return static_cast<size_t>(npairs) * 256 * sizeof(unsigned); }

int status_error(unsigned st) { return (st & kErrOverlap) ? GPO_ERR_BOARD : GPO_OK; }

}  // namespace
}  // namespace gpo

using namespace gpo;

extern "C" {

int gpo_eval_load(const uint64_t* features, int n_features, const double* values, double offset) {
  think::EvalHost h;
  const int rc = think::build_eval(features, n_features, values, offset, &h);
  if (rc != GPO_OK) return rc;
  std::lock_guard<std::mutex> lock(g_think_mutex);
  int r = ensure_think(0);
  if (r != GPO_OK) return r;
  ThinkState& t = g_think;
  cudaFree(t.dMeta);
  cudaFree(t.dDigits);
  cudaFree(t.dValues);
  t.dMeta = nullptr;
  t.dDigits = nullptr;
  t.dValues = nullptr;
  t.loaded = false;
  TH_CK(cudaMalloc(&t.dMeta, sizeof(EvalMeta)));
  TH_CK(cudaMalloc(&t.dDigits, h.digits.size() * sizeof(unsigned) + sizeof(unsigned)));
  TH_CK(cudaMalloc(&t.dValues, h.values.size() * sizeof(float)));
  TH_CK(cudaMemcpy(t.dMeta, &h.meta, sizeof(EvalMeta), cudaMemcpyHostToDevice));
  if (!h.digits.empty())
    TH_CK(cudaMemcpy(t.dDigits, h.digits.data(), h.digits.size() * sizeof(unsigned),
                     cudaMemcpyHostToDevice));
  TH_CK(cudaMemcpy(t.dValues, h.values.data(), h.values.size() * sizeof(float),
                   cudaMemcpyHostToDevice));
  t.npairs = h.meta.npairs;
  t.loaded = true;
  return GPO_OK;
}

int gpo_eval_load_files(const char* features_path, const char* values_path) {
  std::vector<uint64_t> masks;
  int rc = think::read_feature_file(features_path, &masks);
  if (rc != GPO_OK) return rc;
  std::vector<double> values;
  double offset = 0.0;
  rc = think::read_value_file(values_path, masks, &values, &offset);
  if (rc != GPO_OK) return rc;
  return gpo_eval_load(masks.data(), static_cast<int>(masks.size()), values.data(), offset);
}

int gpo_evaluate(const uint64_t* player, const uint64_t* opp, int n, float* value) {
  if (n < 0 || (n > 0 && (!player || !opp || !value))) return GPO_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_think_mutex);
  ThinkState& t = g_think;
  if (!t.loaded) return GPO_ERR_ARG;
  if (n == 0) return GPO_OK;
  const int r = ensure_think(static_cast<size_t>(n));
  if (r != GPO_OK) return r;
  cudaStream_t s = t.stream;
  TH_CK(cudaMemcpyAsync(t.dP, player, n * sizeof(u64), cudaMemcpyHostToDevice, s));
  TH_CK(cudaMemcpyAsync(t.dO, opp, n * sizeof(u64), cudaMemcpyHostToDevice, s));
  TH_CK(cudaMemsetAsync(t.dStatus, 0, sizeof(unsigned), s));
  const size_t smem = eval_smem(t.npairs);
  TH_CK(cudaFuncSetAttribute(eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem)));
  eval_kernel<<<(n + kThinkBlock - 1) / kThinkBlock, kThinkBlock, smem, s>>>(
      t.dP, t.dO, n, t.dMeta, t.dDigits, t.dValues, t.dEval, t.dStatus);
  TH_CK(cudaGetLastError());
  unsigned st = 0;
  TH_CK(cudaMemcpyAsync(value, t.dEval, n * sizeof(float), cudaMemcpyDeviceToHost, s));
  TH_CK(cudaMemcpyAsync(&st, t.dStatus, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  TH_CK(cudaStreamSynchronize(s));
  return status_error(st);
}

int think_batch(const uint64_t* player, const uint64_t* opp, int n, int depth, int8_t* score,
                int8_t* best_move, uint64_t* nodes, gpo_stats* stats) {
  if (n < 0 || (n > 0 && (!player || !opp || !score))) return GPO_ERR_ARG;
  if (depth < think::kMinDepth || depth > think::kMaxDepth) return GPO_ERR_DEPTH;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  std::lock_guard<std::mutex> lock(g_think_mutex);
  ThinkState& t = g_think;
  if (!t.loaded) return GPO_ERR_ARG;
  if (n == 0) return GPO_OK;
  const int r = ensure_think(static_cast<size_t>(n));
  if (r != GPO_OK) return r;
  cudaStream_t s = t.stream;
  TH_CK(cudaMemcpyAsync(t.dP, player, n * sizeof(u64), cudaMemcpyHostToDevice, s));
  TH_CK(cudaMemcpyAsync(t.dO, opp, n * sizeof(u64), cudaMemcpyHostToDevice, s));
  TH_CK(cudaMemsetAsync(t.dStatus, 0, sizeof(unsigned), s));
  TH_CK(cudaMemsetAsync(t.dTotal, 0, sizeof(unsigned long long), s));
  const size_t smem = eval_smem(t.npairs);
  TH_CK(cudaFuncSetAttribute(think_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem)));
  TH_CK(cudaEventRecord(t.ev0, s));
  think_kernel<<<(n + kThinkBlock - 1) / kThinkBlock, kThinkBlock, smem, s>>>(
      t.dP, t.dO, n, depth, t.dMeta, t.dDigits, t.dValues, t.dScore,
      best_move ? t.dBest : nullptr, nodes ? t.dNodes : nullptr, t.dTotal, t.dStatus);
  TH_CK(cudaGetLastError());
  TH_CK(cudaEventRecord(t.ev1, s));
  unsigned st = 0;
  unsigned long long total = 0;
  TH_CK(cudaMemcpyAsync(score, t.dScore, n, cudaMemcpyDeviceToHost, s));
  if (best_move) TH_CK(cudaMemcpyAsync(best_move, t.dBest, n, cudaMemcpyDeviceToHost, s));
  if (nodes)
    TH_CK(cudaMemcpyAsync(nodes, t.dNodes, n * sizeof(u64), cudaMemcpyDeviceToHost, s));
  TH_CK(cudaMemcpyAsync(&st, t.dStatus, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  TH_CK(cudaMemcpyAsync(&total, t.dTotal, sizeof(total), cudaMemcpyDeviceToHost, s));
  TH_CK(cudaStreamSynchronize(s));
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t.ev0, t.ev1);
    stats->nodes = total;
    stats->kernel_ms = ms;
    stats->launches = 1;
  }
  return status_error(st);
}

}  // extern "C"

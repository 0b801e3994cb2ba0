// Learned move orderer: a small MLP trained on the GPU by the kernels in
// this file and used to order the root moves of deep positions.
//
//   input  192 features: the side to move's discs (64), the other side's
//          discs (64), the legal-move mask (64), as 0/1
//   hidden 256 ReLU, 256 ReLU;  output 64 move logits (masked to legal moves)
//   BF16 weights and activations on the tensor cores, FP32 accumulation,
//   FP32 master weights for the Adam update.
//
// Labels are the best moves returned by the solver itself (solve_batch_ex's
// best_move).  The orderer only changes which move is searched first, so
// scores stay exact; it replaces the fastest-first probes at the nodes with
// >= learned_min_empties empties in the top two plies of the search (see
// the learned order table below).
//
// Every product (forward, the two input-gradient and three weight-gradient
// products of backward) is one generic kernel: C = A * B with arbitrary
// element strides, mma.sync.m16n8k16 BF16 -> FP32, one 32x32 tile per warp,
// fused epilogue (bias, ReLU, or the ReLU derivative of a stored
// activation).  The network is tiny next to the search; these products are
// not on the solver's hot path.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gpuothello2.h"
#include "common.cuh"
#include "kernels.h"
#include "table.cuh"

namespace gpo {

typedef __nv_bfloat16 bf16;

namespace {

__device__ __forceinline__ unsigned pack_bf16(bf16 lo, bf16 hi) {
  return static_cast<unsigned>(__bfloat16_as_ushort(lo)) |
         (static_cast<unsigned>(__bfloat16_as_ushort(hi)) << 16);
}

__device__ __forceinline__ void mma_bf16(float* d, const unsigned* a, const unsigned* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

enum : int { EPI_NONE = 0, EPI_BIAS_RELU = 1, EPI_BIAS = 2, EPI_RELU_MASK = 3 };

// C[m][n] = sum_k A(m, k) B(k, n); A(m, k) = A[m*sam + k*sak], B(k, n) =
// B[k*sbk + n*sbn].  M, N multiples of 32, K a multiple of 16.
// Epilogue: EPI_BIAS(_RELU) adds bias[n] (then ReLU); EPI_RELU_MASK keeps
// the value only where act[m][n] > 0 (the ReLU derivative).  Writes FP32
// (cf, row stride N) and/or BF16 (cb, row stride N).
__global__ void gemm_bf16_kernel(const bf16* __restrict__ A, long sam, long sak,
                                 const bf16* __restrict__ B, long sbk, long sbn, int M, int N,
                                 int K, int epi, const float* __restrict__ bias,
                                 const bf16* __restrict__ act, float* __restrict__ cf,
                                 bf16* __restrict__ cb) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int tiles_n = N / 32;
  const int tile = blockIdx.x * (blockDim.x >> 5) + warp;
  if (tile >= (M / 32) * tiles_n) return;
  const int m0 = (tile / tiles_n) * 32, n0 = (tile % tiles_n) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
  const int r = lane >> 2, c = (lane & 3) * 2;
  for (int k0 = 0; k0 < K; k0 += 16) {
    unsigned a[2][4], b[4][2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const long r0 = m0 + i * 16 + r, r1 = r0 + 8;
      const long k = k0 + c;
      a[i][0] = pack_bf16(A[r0 * sam + k * sak], A[r0 * sam + (k + 1) * sak]);
      a[i][1] = pack_bf16(A[r1 * sam + k * sak], A[r1 * sam + (k + 1) * sak]);
      a[i][2] = pack_bf16(A[r0 * sam + (k + 8) * sak], A[r0 * sam + (k + 9) * sak]);
      a[i][3] = pack_bf16(A[r1 * sam + (k + 8) * sak], A[r1 * sam + (k + 9) * sak]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long n = n0 + j * 8 + r;
      const long k = k0 + c;
      b[j][0] = pack_bf16(B[k * sbk + n * sbn], B[(k + 1) * sbk + n * sbn]);
      b[j][1] = pack_bf16(B[(k + 8) * sbk + n * sbn], B[(k + 9) * sbk + n * sbn]);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i], b[j]);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const long m = m0 + i * 16 + r + (q >= 2 ? 8 : 0);
        const long n = n0 + j * 8 + c + (q & 1);
        float v = acc[i][j][q];
        if (epi == EPI_BIAS || epi == EPI_BIAS_RELU) v += bias[n];
        if (epi == EPI_BIAS_RELU) v = v > 0.f ? v : 0.f;
        if (epi == EPI_RELU_MASK && !(__bfloat162float(act[m * N + n]) > 0.f)) v = 0.f;
        if (cf) cf[m * N + n] = v;
        if (cb) cb[m * N + n] = __float2bfloat16(v);
      }
}

// Features of rows 0..n-1 (rows n..rows-1 are zero padding) and legal masks.
__global__ void features_kernel(const u64* __restrict__ P, const u64* __restrict__ O, int n,
                                int rows, bf16* __restrict__ X, u64* __restrict__ legal) {
  const int i = blockIdx.x;
  if (i >= rows) return;
  u64 p = 0, o = 0, m = 0;
  if (i < n) {
    p = P[i];
    o = O[i];
    m = gpo_mobility(p, o);
  }
  if (threadIdx.x == 0 && legal) legal[i] = m;
  for (int f = threadIdx.x; f < 192; f += blockDim.x) {
    const u64 w = f < 64 ? p : (f < 128 ? o : m);
    X[static_cast<long>(i) * 192 + f] = __float2bfloat16(static_cast<float>((w >> (f & 63)) & 1));
  }
}

// Masked softmax cross-entropy over the legal moves; d = (softmax - onehot)
// / batch.  Rows without a legal move or without a label (label >= 64) get
// zero gradient and no loss.
__global__ void xent_kernel(const float* __restrict__ logits, const u64* __restrict__ legal,
                            const signed char* __restrict__ label, int rows, float inv_batch,
                            bf16* __restrict__ dlogits, float* __restrict__ loss_sum,
                            unsigned* __restrict__ correct, unsigned* __restrict__ counted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  const u64 m = legal[i];
  const int y = label ? label[i] : -1;
  const bool use = m && y >= 0 && y < 64 && ((m >> y) & 1);
  float mx = -1e30f;
  int arg = -1;
  for (int k = 0; k < 64; ++k)
    if ((m >> k) & 1) {
      const float z = logits[static_cast<long>(i) * 64 + k];
      if (z > mx) {
        mx = z;
        arg = k;
      }
    }
  float s = 0.f;
  for (int k = 0; k < 64; ++k)
    if ((m >> k) & 1) s += __expf(logits[static_cast<long>(i) * 64 + k] - mx);
  for (int k = 0; k < 64; ++k) {
    float g = 0.f;
    if (use && ((m >> k) & 1)) {
      const float pk = __expf(logits[static_cast<long>(i) * 64 + k] - mx) / s;
      g = (pk - (k == y ? 1.f : 0.f)) * inv_batch;
    }
    dlogits[static_cast<long>(i) * 64 + k] = __float2bfloat16(g);
  }
  if (use) {
    atomicAdd(loss_sum, -(logits[static_cast<long>(i) * 64 + y] - mx - __logf(s)));
    atomicAdd(counted, 1u);
    if (arg == y) atomicAdd(correct, 1u);
  }
}

// out[n] = sum over rows of D[row][n] (bias gradients).
__global__ void colsum_kernel(const bf16* __restrict__ D, int rows, int N, float* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += __bfloat162float(D[static_cast<long>(r) * N + n]);
  out[n] = s;
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, bf16* __restrict__ wb,
                            int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16(wi);
}

__global__ void to_bf16_kernel(const float* __restrict__ a, bf16* __restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = __float2bfloat16(a[i]);
}

// Packed fastest-first style list (search.cuh format) of the five legal
// moves with the highest logits, for the batched kernel's roots.
__global__ void order_kernel(const float* __restrict__ logits, const u64* __restrict__ legal,
                             int n, u64* __restrict__ lists) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  u64 m = legal[i];
  u64 lst = 0x0FFFFFFFFFFFFFFFULL;
  int cnt = 0;
  const int total = __popcll(m);
  for (int slot = 0; slot < 5 && m; ++slot) {
    float best = -1e30f;
    int arg = 0;
    for (u64 t = m; t; t &= t - 1) {
      const int k = __ffsll(static_cast<long long>(t)) - 1;
      const float z = logits[static_cast<long>(i) * 64 + k];
      if (z > best) {
        best = z;
        arg = k;
      }
    }
    m &= ~(1ULL << arg);
    const u64 e = (static_cast<u64>(slot) << 6) | static_cast<u64>(arg);
    lst = (lst & ~(0xFFFULL << (12 * slot))) | (e << (12 * slot));
    ++cnt;
  }
  if (total > cnt) lst |= 1ULL << 63;
  lists[i] = lst;
}

// ---- parameter block layout (FP32 or BF16, same order) ----
constexpr int kIn = 192, kH = 256, kOut = 64;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kH, kW2 = kB1 + kH, kB2 = kW2 + kH * kH,
              kW3 = kB2 + kH, kB3 = kW3 + kH * kOut, kParams = kB3 + kOut;

struct Net {
  float* w = nullptr;   // FP32 master
  bf16* wb = nullptr;   // BF16 copy
  float* g = nullptr;   // gradients
  float* m = nullptr;   // Adam moments
  float* v = nullptr;
  int rows = 0;         // activation capacity
  bf16* X = nullptr;
  bf16* H1 = nullptr;
  bf16* H2 = nullptr;
  float* Z = nullptr;   // logits
  bf16* D3 = nullptr;
  bf16* D2 = nullptr;
  bf16* D1 = nullptr;
  u64* legal = nullptr;
  u64* P = nullptr;
  u64* O = nullptr;
  signed char* y = nullptr;
  float* loss = nullptr;
  unsigned* cnt = nullptr;  // correct, counted
};

#define MLP_CK(call)                                                                   \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      std::fprintf(stderr, "gpuothello2 mlp: %s: %s\n", #call, cudaGetErrorString(e_)); \
      return e_ == cudaErrorMemoryAllocation ? GPO_ERR_NOMEM : GPO_ERR_CUDA;          \
    }                                                                                  \
  } while (0)

void net_free(Net& t) {
  void* ptrs[] = {t.w, t.wb, t.g, t.m, t.v, t.X, t.H1, t.H2, t.Z, t.D3, t.D2, t.D1, t.legal,
                  t.P, t.O, t.y, t.loss, t.cnt};
  for (void* p : ptrs) cudaFree(p);
  t = Net();
}

int net_alloc(Net& t, int rows, bool train) {
  MLP_CK(cudaMalloc(&t.w, kParams * sizeof(float)));
  MLP_CK(cudaMalloc(&t.wb, kParams * sizeof(bf16)));
  if (train) {
    MLP_CK(cudaMalloc(&t.g, kParams * sizeof(float)));
    MLP_CK(cudaMalloc(&t.m, kParams * sizeof(float)));
    MLP_CK(cudaMalloc(&t.v, kParams * sizeof(float)));
    MLP_CK(cudaMemset(t.m, 0, kParams * sizeof(float)));
    MLP_CK(cudaMemset(t.v, 0, kParams * sizeof(float)));
    MLP_CK(cudaMalloc(&t.D3, static_cast<size_t>(rows) * kOut * sizeof(bf16)));
    MLP_CK(cudaMalloc(&t.D2, static_cast<size_t>(rows) * kH * sizeof(bf16)));
    MLP_CK(cudaMalloc(&t.D1, static_cast<size_t>(rows) * kH * sizeof(bf16)));
    MLP_CK(cudaMalloc(&t.y, rows));
  }
  t.rows = rows;
  MLP_CK(cudaMalloc(&t.X, static_cast<size_t>(rows) * kIn * sizeof(bf16)));
  MLP_CK(cudaMalloc(&t.H1, static_cast<size_t>(rows) * kH * sizeof(bf16)));
  MLP_CK(cudaMalloc(&t.H2, static_cast<size_t>(rows) * kH * sizeof(bf16)));
  MLP_CK(cudaMalloc(&t.Z, static_cast<size_t>(rows) * kOut * sizeof(float)));
  MLP_CK(cudaMalloc(&t.legal, static_cast<size_t>(rows) * sizeof(u64)));
  MLP_CK(cudaMalloc(&t.P, static_cast<size_t>(rows) * sizeof(u64)));
  MLP_CK(cudaMalloc(&t.O, static_cast<size_t>(rows) * sizeof(u64)));
  MLP_CK(cudaMalloc(&t.loss, sizeof(float)));
  MLP_CK(cudaMalloc(&t.cnt, 2 * sizeof(unsigned)));
  return GPO_OK;
}

cudaError_t gemm(const bf16* A, long sam, long sak, const bf16* B, long sbk, long sbn, int M, int N,
                 int K, int epi, const float* bias, const bf16* act, float* cf, bf16* cb,
                 cudaStream_t s) {
  const int tiles = (M / 32) * (N / 32);
  gemm_bf16_kernel<<<(tiles + 3) / 4, 128, 0, s>>>(A, sam, sak, B, sbk, sbn, M, N, K, epi, bias,
                                                   act, cf, cb);
  return cudaGetLastError();
}

// Forward over rows (a multiple of 32) whose features and legal masks are in
// t.X / t.legal: H1, H2 (BF16) and logits Z (FP32).
cudaError_t forward(Net& t, int rows, cudaStream_t s) {
  const bf16* w = t.wb;
  cudaError_t e = gemm(t.X, kIn, 1, w + kW1, kH, 1, rows, kH, kIn, EPI_BIAS_RELU, t.w + kB1,
                       nullptr, nullptr, t.H1, s);
  if (e == cudaSuccess)
    e = gemm(t.H1, kH, 1, w + kW2, kH, 1, rows, kH, kH, EPI_BIAS_RELU, t.w + kB2, nullptr, nullptr,
             t.H2, s);
  if (e == cudaSuccess)
    e = gemm(t.H2, kH, 1, w + kW3, kOut, 1, rows, kOut, kH, EPI_BIAS, t.w + kB3, nullptr, t.Z,
             nullptr, s);
  return e;
}

// Backward from D3 (dlogits, BF16): gradients of every parameter in t.g.
cudaError_t backward(Net& t, int rows, cudaStream_t s) {
  const bf16* w = t.wb;
  cudaError_t e;
  // dW3 = H2^T D3 ; dB3 = colsum D3
  e = gemm(t.H2, 1, kH, t.D3, kOut, 1, kH, kOut, rows, EPI_NONE, nullptr, nullptr, t.g + kW3,
           nullptr, s);
  if (e != cudaSuccess) return e;
  colsum_kernel<<<1, 64, 0, s>>>(t.D3, rows, kOut, t.g + kB3);
  // D2 = (D3 W3^T) * relu'(H2)
  e = gemm(t.D3, kOut, 1, w + kW3, 1, kOut, rows, kH, kOut, EPI_RELU_MASK, nullptr, t.H2, nullptr,
           t.D2, s);
  if (e != cudaSuccess) return e;
  e = gemm(t.H1, 1, kH, t.D2, kH, 1, kH, kH, rows, EPI_NONE, nullptr, nullptr, t.g + kW2, nullptr,
           s);
  if (e != cudaSuccess) return e;
  colsum_kernel<<<1, 256, 0, s>>>(t.D2, rows, kH, t.g + kB2);
  // D1 = (D2 W2^T) * relu'(H1)
  e = gemm(t.D2, kH, 1, w + kW2, 1, kH, rows, kH, kH, EPI_RELU_MASK, nullptr, t.H1, nullptr, t.D1,
           s);
  if (e != cudaSuccess) return e;
  e = gemm(t.X, 1, kIn, t.D1, kH, 1, kIn, kH, rows, EPI_NONE, nullptr, nullptr, t.g + kW1, nullptr,
           s);
  if (e != cudaSuccess) return e;
  colsum_kernel<<<1, 256, 0, s>>>(t.D1, rows, kH, t.g + kB1);
  return cudaGetLastError();
}

int round32(int n) { return (n + 31) / 32 * 32; }

int upload_weights(Net& t, const float* w, cudaStream_t s) {
  MLP_CK(cudaMemcpyAsync(t.w, w, kParams * sizeof(float), cudaMemcpyHostToDevice, s));
  to_bf16_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(t.w, t.wb, kParams);
  MLP_CK(cudaGetLastError());
  return GPO_OK;
}

int features(Net& t, const uint64_t* P, const uint64_t* O, int n, int rows, cudaStream_t s) {
  MLP_CK(cudaMemcpyAsync(t.P, P, n * sizeof(u64), cudaMemcpyHostToDevice, s));
  MLP_CK(cudaMemcpyAsync(t.O, O, n * sizeof(u64), cudaMemcpyHostToDevice, s));
  features_kernel<<<rows, 64, 0, s>>>(t.P, t.O, n, rows, t.X, t.legal);
  MLP_CK(cudaGetLastError());
  return GPO_OK;
}


// Gathers rows idx[off .. off+rows) (zero rows past count) into X / legal,
// and their labels when y_src is given.
__global__ void gather_kernel(const u64* __restrict__ P, const u64* __restrict__ O,
                              const unsigned* __restrict__ idx, long off, long count, int rows,
                              bf16* __restrict__ X, u64* __restrict__ legal,
                              const signed char* __restrict__ y_src, signed char* __restrict__ y) {
  const int i = blockIdx.x;
  if (i >= rows) return;
  u64 p = 0, o = 0, m = 0;
  signed char lab = -1;
  if (off + i < count) {
    const unsigned j = idx ? idx[off + i] : static_cast<unsigned>(off + i);
    p = P[j];
    o = O[j];
    m = gpo_mobility(p, o);
    if (y_src) lab = y_src[j];
  }
  if (threadIdx.x == 0) {
    legal[i] = m;
    if (y) y[i] = lab;
  }
  for (int f = threadIdx.x; f < 192; f += blockDim.x) {
    const u64 w = f < 64 ? p : (f < 128 ? o : m);
    X[static_cast<long>(i) * 192 + f] = __float2bfloat16(static_cast<float>((w >> (f & 63)) & 1));
  }
}

// ---- learned order table: move lists for the top of the search ----
// The search asks for a node's move order when it creates the node, at
// random moments in 32 independent lanes per warp; a network evaluated then
// would run one row at a time.  Instead, before the search, every node with
// >= L empties in the top two plies below each deep root is enumerated (the
// frontier the search will meet first), the network scores the whole
// frontier in large batches on the tensor cores, and the resulting lists go
// into a table keyed exactly by position (the transposition table's
// bijective key, table.cuh).  Entry: 4 words {x, y, list, 0}; x = y = 0 is
// empty (no real position maps there).  Linear probing, at most
// kOrderProbe slots.

// Nodes with >= L empties from the root down two plies (a pass counts as a
// ply: the swapped position); emit = false only counts them.
__device__ __forceinline__ int frontier_walk(u64 P, u64 O, int L, const u64* rays, bool emit,
                                             u64* outP, u64* outO, long at, long cap) {
  int k = 0;
  auto put = [&](u64 a, u64 b) {
    if (emit && at + k < cap) {
      outP[at + k] = a;
      outO[at + k] = b;
    }
    ++k;
  };
  if (64 - popc(P | O) < L) return 0;
  put(P, O);
  u64 m1 = gpo_mobility(P, O);
  const bool pass1 = !m1;
  if (pass1) m1 = gpo_mobility(O, P) ? 1ULL << 63 : 0ULL;  // one "move": the pass
  while (m1) {
    const int s1 = ctz64(m1);
    m1 &= m1 - 1;
    u64 cP, cO;
    if (pass1) {
      cP = O;
      cO = P;
    } else {
      const u64 f = gpo_flip(P, O, s1, rays);
      cP = O ^ f;
      cO = P ^ f ^ (1ULL << s1);
    }
    if (64 - popc(cP | cO) < L) continue;
    put(cP, cO);
    u64 m2 = gpo_mobility(cP, cO);
    while (m2) {
      const int s2 = ctz64(m2);
      m2 &= m2 - 1;
      const u64 f = gpo_flip(cP, cO, s2, rays);
      const u64 gP = cO ^ f, gO = cP ^ f ^ (1ULL << s2);
      if (64 - popc(gP | gO) >= L) put(gP, gO);
    }
  }
  return k;
}

__global__ void frontier_kernel(const u64* __restrict__ P, const u64* __restrict__ O,
                                const unsigned* __restrict__ perm, long count, int L,
                                u64* __restrict__ outP, u64* __restrict__ outO,
                                unsigned long long* __restrict__ counter, long cap) {
  __shared__ __align__(16) u64 rays[256];
  gpo_build_rays(rays);
  __syncthreads();
  const long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const unsigned j = perm[i];
  const u64 p = P[j], o = O[j];
  const int k = frontier_walk(p, o, L, rays, false, nullptr, nullptr, 0, 0);
  if (!k) return;
  const long at = static_cast<long>(atomicAdd(counter, static_cast<unsigned long long>(k)));
  if (at + k <= cap) frontier_walk(p, o, L, rays, true, outP, outO, at, cap);
}

constexpr int kOrderProbe = 16;
constexpr int kInferRows = 1 << 18;

__global__ void order_insert_kernel(const u64* __restrict__ fP, const u64* __restrict__ fO,
                                    const u64* __restrict__ lists, long off, long count, int rows,
                                    u64* __restrict__ table, int bits) {
  const long r = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= rows || off + r >= count) return;
  const TTKey k = tt_key(fP[off + r], fO[off + r]);
  const size_t mask = (static_cast<size_t>(1) << bits) - 1;
  size_t h = static_cast<size_t>(k.y >> (64 - bits));
  for (int probe = 0; probe < kOrderProbe; ++probe, h = (h + 1) & mask) {
    u64 o0, o1;
    tt_cas128(table + 4 * h, 0, 0, k.x, k.y, o0, o1);
    if ((o0 | o1) == 0) {  // claimed
      table[4 * h + 2] = lists[r];
      return;
    }
    if (o0 == k.x && o1 == k.y) return;  // the same position, already there
  }
}

Net g_infer;        // network loaded for the solver
u64* g_lists_tmp = nullptr;
bool g_loaded = false;
int g_infer_device = -1;                 // device holding g_infer
cudaEvent_t g_infer_done = nullptr;      // recorded after the last inference batch
// Guards g_infer / g_loaded / g_infer_done.  The mutex is held only while a
// solve enqueues its inference work on the solve's (non-blocking) stream, so
// gpo_mlp_load first waits on g_infer_done: a reload never overwrites
// weights that enqueued inference kernels may still read.
std::mutex g_mlp_mutex;

bool loaded_here() {
  int dev = -1;
  return g_loaded && cudaGetDevice(&dev) == cudaSuccess && dev == g_infer_device;
}

}  // namespace

// True when a network is loaded on the current device (the network lives on
// the device that was current at gpo_mlp_load).
bool mlp_loaded() {
  std::lock_guard<std::mutex> lock(g_mlp_mutex);
  return loaded_here();
}

// Learned order table for the search: the frontier of the `count` roots
// d_idx[0..count) (nodes with >= L empties, top two plies) into
// frontP/frontO (capacity cap), scored by the network, inserted into the
// table of 2^table_bits entries (cleared here).  *frontier receives the
// number of frontier nodes (those past cap are left out: their nodes use
// the fastest-first order).
int mlp_order_frontier(const u64* d_player, const u64* d_opp, const unsigned* d_idx, long count,
                       int L, u64* frontP, u64* frontO, long cap, unsigned long long* counter,
                       u64* table, int table_bits, cudaStream_t s, unsigned* launched,
                       long* frontier) {
  *launched = 0;
  *frontier = 0;
  std::lock_guard<std::mutex> lock(g_mlp_mutex);
  if (!loaded_here()) return GPO_ERR_ARG;
  Net& t = g_infer;
  MLP_CK(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s));
  MLP_CK(cudaMemsetAsync(table, 0, (static_cast<size_t>(32)) << table_bits, s));
  frontier_kernel<<<static_cast<unsigned>((count + 127) / 128), 128, 0, s>>>(
      d_player, d_opp, d_idx, count, L, frontP, frontO, counter, cap);
  MLP_CK(cudaGetLastError());
  *launched += 1;
  unsigned long long nf = 0;
  MLP_CK(cudaMemcpyAsync(&nf, counter, sizeof(nf), cudaMemcpyDeviceToHost, s));
  MLP_CK(cudaStreamSynchronize(s));
  const long total = static_cast<long>(nf < static_cast<unsigned long long>(cap) ? nf : cap);
  for (long off = 0; off < total; off += t.rows) {
    *launched += 6;  // gather, three GEMMs, order, insert
    gather_kernel<<<t.rows, 64, 0, s>>>(frontP, frontO, nullptr, off, total, t.rows, t.X, t.legal,
                                         nullptr, nullptr);
    MLP_CK(cudaGetLastError());
    MLP_CK(forward(t, t.rows, s));
    order_kernel<<<(t.rows + 127) / 128, 128, 0, s>>>(t.Z, t.legal, t.rows, g_lists_tmp);
    order_insert_kernel<<<(t.rows + 127) / 128, 128, 0, s>>>(frontP, frontO, g_lists_tmp, off, total,
                                                              t.rows, table, table_bits);
    MLP_CK(cudaGetLastError());
  }
  MLP_CK(cudaEventRecord(g_infer_done, s));
  *frontier = total;
  return GPO_OK;
}

}  // namespace gpo

using namespace gpo;

extern "C" {

int gpo_mlp_param_count(void) { return kParams; }

// He-style initialisation from a splitmix64 stream (host side).
int gpo_mlp_init(uint64_t seed, float* w) {
  if (!w) return GPO_ERR_ARG;
  uint64_t x = seed;
  auto next = [&x]() {
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  };
  auto uniform = [&next]() { return static_cast<float>((next() >> 11) * (1.0 / 9007199254740992.0)); };
  auto fill = [&](int off, int fan_in, int count) {
    const float a = std::sqrt(6.0f / static_cast<float>(fan_in));
    for (int i = 0; i < count; ++i) w[off + i] = (2.f * uniform() - 1.f) * a;
  };
  fill(kW1, kIn, kIn * kH);
  fill(kW2, kH, kH * kH);
  fill(kW3, kH, kH * kOut);
  for (int i = 0; i < kH; ++i) w[kB1 + i] = 0.f, w[kB2 + i] = 0.f;
  for (int i = 0; i < kOut; ++i) w[kB3 + i] = 0.f;
  return GPO_OK;
}

int gpo_mlp_forward(const float* w, const uint64_t* player, const uint64_t* opp, int n,
                    float* logits) {
  if (!w || n < 0 || (n > 0 && (!player || !opp || !logits))) return GPO_ERR_ARG;
  if (n == 0) return GPO_OK;
  std::lock_guard<std::mutex> lock(g_mlp_mutex);
  const int rows = round32(n);
  Net t;
  int rc = net_alloc(t, rows, false);
  cudaStream_t s = nullptr;
  if (rc == GPO_OK) rc = upload_weights(t, w, s);
  if (rc == GPO_OK) rc = features(t, player, opp, n, rows, s);
  if (rc == GPO_OK && forward(t, rows, s) != cudaSuccess) rc = GPO_ERR_CUDA;
  if (rc == GPO_OK &&
      cudaMemcpy(logits, t.Z, static_cast<size_t>(n) * kOut * sizeof(float),
                 cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = GPO_ERR_CUDA;
  net_free(t);
  return rc;
}

// One forward + backward over n positions with labels: the gradient of the
// mean masked cross-entropy for every parameter (same layout as weights).
int gpo_mlp_gradients(const float* w, const uint64_t* player, const uint64_t* opp,
                      const int8_t* best, int n, float* grads, float* loss) {
  if (!w || n <= 0 || !player || !opp || !best || !grads) return GPO_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_mlp_mutex);
  const int rows = round32(n);
  Net t;
  int rc = net_alloc(t, rows, true);
  cudaStream_t s = nullptr;
  signed char* ysrc = nullptr;
  if (rc == GPO_OK) rc = upload_weights(t, w, s);
  if (rc == GPO_OK) rc = features(t, player, opp, n, rows, s);
  if (rc == GPO_OK && cudaMalloc(&ysrc, rows) != cudaSuccess) rc = GPO_ERR_NOMEM;
  if (rc == GPO_OK) {
    std::vector<signed char> yh(rows, -1);
    std::memcpy(yh.data(), best, n);
    if (cudaMemcpy(t.y, yh.data(), rows, cudaMemcpyHostToDevice) != cudaSuccess) rc = GPO_ERR_CUDA;
  }
  if (rc == GPO_OK) {
    cudaMemset(t.loss, 0, sizeof(float));
    cudaMemset(t.cnt, 0, 2 * sizeof(unsigned));
    if (forward(t, rows, s) != cudaSuccess) rc = GPO_ERR_CUDA;
  }
  if (rc == GPO_OK) {
    xent_kernel<<<(rows + 127) / 128, 128, 0, s>>>(t.Z, t.legal, t.y, rows, 1.f / n, t.D3, t.loss,
                                                   t.cnt, t.cnt + 1);
    if (backward(t, rows, s) != cudaSuccess) rc = GPO_ERR_CUDA;
  }
  if (rc == GPO_OK &&
      cudaMemcpy(grads, t.g, kParams * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = GPO_ERR_CUDA;
  if (rc == GPO_OK && loss) {
    float l = 0.f;
    cudaMemcpy(&l, t.loss, sizeof(float), cudaMemcpyDeviceToHost);
    *loss = l / n;
  }
  cudaFree(ysrc);
  net_free(t);
  return rc;
}

// Adam training on (player, opp, best) for `epochs` passes in batches of
// `batch` (a multiple of 32), in a seeded shuffled order.  `w` holds the
// initial weights on entry and the trained ones on return; history[2*e] /
// history[2*e+1] receive epoch e's mean loss and best-move accuracy.
int gpo_mlp_train(const uint64_t* player, const uint64_t* opp, const int8_t* best, int n,
                  int epochs, int batch, float lr, uint64_t seed, float* w, float* history) {
  if (!player || !opp || !best || !w || n <= 0 || epochs <= 0 || batch <= 0 || batch % 32)
    return GPO_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_mlp_mutex);
  Net t;
  int rc = net_alloc(t, batch, true);
  cudaStream_t s = nullptr;
  u64 *dP = nullptr, *dO = nullptr;
  signed char* dY = nullptr;
  unsigned* dIdx = nullptr;
  if (rc == GPO_OK) rc = upload_weights(t, w, s);
  if (rc == GPO_OK && (cudaMalloc(&dP, n * sizeof(u64)) != cudaSuccess ||
                       cudaMalloc(&dO, n * sizeof(u64)) != cudaSuccess ||
                       cudaMalloc(&dY, n) != cudaSuccess ||
                       cudaMalloc(&dIdx, n * sizeof(unsigned)) != cudaSuccess))
    rc = GPO_ERR_NOMEM;
  if (rc == GPO_OK) {
    cudaMemcpy(dP, player, n * sizeof(u64), cudaMemcpyHostToDevice);
    cudaMemcpy(dO, opp, n * sizeof(u64), cudaMemcpyHostToDevice);
    cudaMemcpy(dY, best, n, cudaMemcpyHostToDevice);
  }
  std::vector<unsigned> order(n);
  for (int i = 0; i < n; ++i) order[i] = static_cast<unsigned>(i);
  uint64_t x = seed;
  auto next = [&x]() {
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  };
  int step = 0;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs && rc == GPO_OK; ++ep) {
    for (int i = n - 1; i > 0; --i) {
      const int j = static_cast<int>(next() % static_cast<uint64_t>(i + 1));
      std::swap(order[i], order[j]);
    }
    cudaMemcpy(dIdx, order.data(), n * sizeof(unsigned), cudaMemcpyHostToDevice);
    cudaMemset(t.loss, 0, sizeof(float));
    cudaMemset(t.cnt, 0, 2 * sizeof(unsigned));
    for (long off = 0; off + batch <= n && rc == GPO_OK; off += batch) {
      gather_kernel<<<batch, 64, 0, s>>>(dP, dO, dIdx, off, n, batch, t.X, t.legal, dY, t.y);
      if (forward(t, batch, s) != cudaSuccess) rc = GPO_ERR_CUDA;
      xent_kernel<<<(batch + 127) / 128, 128, 0, s>>>(t.Z, t.legal, t.y, batch, 1.f / batch, t.D3,
                                                      t.loss, t.cnt, t.cnt + 1);
      if (rc == GPO_OK && backward(t, batch, s) != cudaSuccess) rc = GPO_ERR_CUDA;
      ++step;
      const float c1 = 1.f - std::pow(b1, static_cast<float>(step));
      const float c2 = 1.f - std::pow(b2, static_cast<float>(step));
      adam_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(t.w, t.g, t.m, t.v, t.wb, kParams, lr, b1,
                                                         b2, eps, c1, c2);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) rc = GPO_ERR_CUDA;
    if (history && rc == GPO_OK) {
      float l = 0.f;
      unsigned c[2] = {0, 0};
      cudaMemcpy(&l, t.loss, sizeof(float), cudaMemcpyDeviceToHost);
      cudaMemcpy(c, t.cnt, sizeof(c), cudaMemcpyDeviceToHost);
      history[2 * ep] = c[1] ? l / c[1] : 0.f;
      history[2 * ep + 1] = c[1] ? static_cast<float>(c[0]) / c[1] : 0.f;
    }
  }
  if (rc == GPO_OK &&
      cudaMemcpy(w, t.w, kParams * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = GPO_ERR_CUDA;
  cudaFree(dP);
  cudaFree(dO);
  cudaFree(dY);
  cudaFree(dIdx);
  net_free(t);
  return rc;
}

// Loads weights for the solver's learned ordering (use_learned) on the
// current device (a load on another device moves the network there); NULL
// unloads them.
int gpo_mlp_load(const float* w) {
  std::lock_guard<std::mutex> lock(g_mlp_mutex);
  // inference that a solve enqueued with the old weights finishes first
  if (g_infer_done && cudaEventSynchronize(g_infer_done) != cudaSuccess) return GPO_ERR_CUDA;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return GPO_ERR_CUDA;
  if (!w || (g_loaded && dev != g_infer_device)) {
    // unload, or move the network to the current device
    if (g_loaded && dev != g_infer_device && cudaSetDevice(g_infer_device) != cudaSuccess)
      return GPO_ERR_CUDA;
    net_free(g_infer);
    cudaFree(g_lists_tmp);
    if (g_infer_done) cudaEventDestroy(g_infer_done);
    g_lists_tmp = nullptr;
    g_infer_done = nullptr;
    g_loaded = false;
    g_infer_device = -1;
    if (cudaSetDevice(dev) != cudaSuccess) return GPO_ERR_CUDA;
    if (!w) return GPO_OK;
  }
  if (!g_loaded) {
    // rows per inference batch: the learned order table scores millions of
    // frontier positions per solve, in batches of this many
    int rc = net_alloc(g_infer, kInferRows, false);
    if (rc != GPO_OK) return rc;
    if (cudaMalloc(&g_lists_tmp, kInferRows * sizeof(u64)) != cudaSuccess) return GPO_ERR_NOMEM;
    if (!g_infer_done &&
        cudaEventCreateWithFlags(&g_infer_done, cudaEventDisableTiming) != cudaSuccess)
      return GPO_ERR_CUDA;
  }
  int rc = upload_weights(g_infer, w, nullptr);
  if (rc != GPO_OK) return rc;
  if (cudaDeviceSynchronize() != cudaSuccess) return GPO_ERR_CUDA;
  g_loaded = true;
  g_infer_device = dev;
  return GPO_OK;
}

}  // extern "C"

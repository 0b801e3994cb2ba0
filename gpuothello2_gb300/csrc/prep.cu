// Input checks, empties bucketing and the seeded position generator.
//
// Bucketing: a position's cost grows roughly geometrically with its empty
// count, so the batched kernel's queue holds the positions grouped by empty
// count, most empties first: lanes of one warp then search positions of
// similar size, and the cheapest positions are what is left at the tail of
// the launch.  Three short kernels: per-block histograms of the empty count
// (also validating each position), a one-block exclusive scan over the 65
// buckets in descending order, and a scatter that reserves one range per
// bucket per block and fills it.
#include "common.cuh"
#include "kernels.h"

namespace gpo {

constexpr int kBuckets = 65;

__global__ void bucket_count_kernel(const u64* __restrict__ player, const u64* __restrict__ opp,
                                    int n, int depth, unsigned* __restrict__ hist,
                                    DeviceStats* __restrict__ stats) {
  __shared__ unsigned h[kBuckets];
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) h[b] = 0;
  __syncthreads();
  unsigned err = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const u64 P = player[i], O = opp[i];
    const int e = 64 - popc(P | O);
    if (P & O) err |= kErrOverlap;
    if (e > depth) err |= kErrDepth;
    atomicAdd(&h[e], 1u);
  }
  if (err) atomicOr(&stats->status, err);
  __syncthreads();
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], h[b]);
}

// cursor[e] = number of positions with more than e empties.
__global__ void bucket_scan_kernel(const unsigned* __restrict__ hist, unsigned* __restrict__ cursor) {
  if (threadIdx.x == 0) {
    unsigned acc = 0;
    for (int e = kBuckets - 1; e >= 0; --e) {
      cursor[e] = acc;
      acc += hist[e];
    }
  }
}

__global__ void bucket_scatter_kernel(const u64* __restrict__ player, const u64* __restrict__ opp,
                                      int n, unsigned* __restrict__ cursor,
                                      unsigned* __restrict__ perm) {
  __shared__ unsigned h[kBuckets];
  __shared__ unsigned base[kBuckets];
  const int per_block = blockDim.x * 4;
  const int start = blockIdx.x * per_block;
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) h[b] = 0;
  __syncthreads();
  int e4[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i = start + k * blockDim.x + threadIdx.x;
    e4[k] = -1;
    if (i < n) {
      e4[k] = 64 - popc(player[i] | opp[i]);
      atomicAdd(&h[e4[k]], 1u);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) {
    base[b] = h[b] ? atomicAdd(&cursor[b], h[b]) : 0u;
    h[b] = 0;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i = start + k * blockDim.x + threadIdx.x;
    if (e4[k] >= 0) perm[base[e4[k]] + atomicAdd(&h[e4[k]], 1u)] = static_cast<unsigned>(i);
  }
}

// ---- seeded random-playout generator (one thread per position) ----
__device__ __forceinline__ u64 splitmix64(u64& x) {
  u64 z = (x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ u64 rotl64(u64 x, int k) { return (x << k) | (x >> (64 - k)); }

struct Xoshiro {
  u64 s0, s1, s2, s3;
  __device__ __forceinline__ u64 next() {
    const u64 result = rotl64(s1 * 5, 7) * 9;
    const u64 t = s1 << 17;
    s2 ^= s0;
    s3 ^= s1;
    s1 ^= s2;
    s0 ^= s3;
    s2 ^= t;
    s3 = rotl64(s3, 45);
    return result;
  }
  __device__ __forceinline__ u64 uniform(u64 k) { return __umul64hi(next(), k); }
};

__global__ void generate_kernel(u64 seed, u64 first, int n, int min_e, int max_e,
                                u64* __restrict__ out_p, u64* __restrict__ out_o) {
  __shared__ __align__(16) u64 rays[256];
  gpo_build_rays(rays);
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const u64 black0 = 0x0000000810000000ULL, white0 = 0x0000001008000000ULL;
  u64 x = (seed << 32) + first + static_cast<u64>(i);
  Xoshiro r;
  r.s0 = splitmix64(x);
  r.s1 = splitmix64(x);
  r.s2 = splitmix64(x);
  r.s3 = splitmix64(x);
  int target = min_e;
  if (max_e > min_e) target = min_e + static_cast<int>(r.uniform(static_cast<u64>(max_e - min_e + 1)));
  u64 P = black0, O = white0;
  // A game fills one square per move, so at most 60 moves per attempt; the
  // attempt cap only bounds the loop (an attempt that cannot reach the
  // target restarts from the same stream, as the oracle does).
  for (int steps = 0; steps < (1 << 20); ++steps) {
    if (64 - popc(P | O) == target) break;
    u64 moves = gpo_mobility(P, O);
    if (!moves) {
      if (gpo_mobility(O, P)) {
        const u64 t = P;
        P = O;
        O = t;
      } else {
        P = black0;
        O = white0;
      }
      continue;
    }
    u64 j = r.uniform(static_cast<u64>(popc(moves)));
    while (j--) moves &= moves - 1;
    const int sq = ctz64(moves);
    const u64 f = gpo_flip(P, O, sq, rays);
    const u64 nP = O ^ f, nO = P ^ f ^ (1ULL << sq);
    P = nP;
    O = nO;
  }
  out_p[i] = P;
  out_o[i] = O;
}

cudaError_t launch_bucket(const u64* player, const u64* opp, int n, int depth, unsigned* hist,
                          unsigned* cursor, unsigned* perm, DeviceStats* stats, int sms,
                          cudaStream_t s) {
  const int count_grid = sms > 0 ? sms * 4 : 256;
  bucket_count_kernel<<<count_grid, 256, 0, s>>>(player, opp, n, depth, hist, stats);
  bucket_scan_kernel<<<1, 32, 0, s>>>(hist, cursor);
  bucket_scatter_kernel<<<(n + 1023) / 1024, 256, 0, s>>>(player, opp, n, cursor, perm);
  return cudaGetLastError();
}

cudaError_t launch_generate(u64 seed, u64 first, int n, int min_e, int max_e, u64* out_p,
                            u64* out_o, cudaStream_t s) {
  generate_kernel<<<(n + 127) / 128, 128, 0, s>>>(seed, first, n, min_e, max_e, out_p, out_o);
  return cudaGetLastError();
}

}  // namespace gpo

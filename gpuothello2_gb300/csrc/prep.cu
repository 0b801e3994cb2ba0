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

// ---- second pass of hard positions ----
__global__ void collect_marked_kernel(const signed char* __restrict__ score, int n,
                                      unsigned* __restrict__ idx, unsigned* __restrict__ count) {
  // one block: keeps the marked indices in ascending order
  __shared__ unsigned base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  for (int start = 0; start < n; start += blockDim.x) {
    const int i = start + threadIdx.x;
    const bool m = i < n && score[i] == -128;
    const unsigned ballot = __ballot_sync(0xffffffffu, m);
    __shared__ unsigned warp_cnt[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_cnt[warp] = __popc(ballot);
    __syncthreads();
    unsigned off = base;
    for (int w = 0; w < warp; ++w) off += warp_cnt[w];
    if (m) idx[off + __popc(ballot & ((1u << lane) - 1u))] = static_cast<unsigned>(i);
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned total = 0;
      for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) total += warp_cnt[w];
      base += total;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = base;
}

__global__ void gather_kernel(const u64* __restrict__ P, const u64* __restrict__ O,
                              const unsigned* __restrict__ idx, int count, u64* __restrict__ outP,
                              u64* __restrict__ outO) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) {
    outP[i] = P[idx[i]];
    outO[i] = O[idx[i]];
  }
}

__global__ void scatter_scores_kernel(const signed char* __restrict__ sc,
                                      const signed char* __restrict__ best,
                                      const unsigned long long* __restrict__ nodes,
                                      const unsigned* __restrict__ idx, int count,
                                      signed char* __restrict__ score_out,
                                      signed char* __restrict__ best_out,
                                      unsigned long long* __restrict__ nodes_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) {
    score_out[idx[i]] = sc[i];
    if (best_out) best_out[idx[i]] = best[i];
    if (nodes_out) nodes_out[idx[i]] += nodes[i];
  }
}

cudaError_t launch_collect_marked(const signed char* score, int n, unsigned* idx, unsigned* count,
                                  cudaStream_t s) {
  collect_marked_kernel<<<1, 1024, 0, s>>>(score, n, idx, count);
  return cudaGetLastError();
}

cudaError_t launch_gather(const u64* P, const u64* O, const unsigned* idx, int count, u64* outP,
                          u64* outO, cudaStream_t s) {
  gather_kernel<<<(count + 255) / 256, 256, 0, s>>>(P, O, idx, count, outP, outO);
  return cudaGetLastError();
}

cudaError_t launch_scatter_scores(const signed char* sc, const signed char* best,
                                  const unsigned long long* nodes, const unsigned* idx, int count,
                                  signed char* score_out, signed char* best_out,
                                  unsigned long long* nodes_out, cudaStream_t s) {
  scatter_scores_kernel<<<(count + 255) / 256, 256, 0, s>>>(sc, best, nodes, idx, count, score_out,
                                                            best_out, nodes_out);
  return cudaGetLastError();
}

// ---- expansion of hard positions into their children ----
// For each marked position idx[i] of a level: its children (after each
// legal move, or the swapped position when it must pass) are appended to the
// next level, with the parent's index and the move (64 = pass).  When the
// level carries search windows (pa/pb), each child gets the negated,
// swapped window (-pb, -pa) in ca/cb.
__global__ void expand_kernel(const u64* __restrict__ P, const u64* __restrict__ O,
                              const unsigned* __restrict__ idx, int m, u64* __restrict__ cP,
                              u64* __restrict__ cO, unsigned* __restrict__ cparent,
                              unsigned char* __restrict__ cmove, unsigned* __restrict__ counter,
                              unsigned cap, const signed char* __restrict__ pa,
                              const signed char* __restrict__ pb, signed char* __restrict__ ca,
                              signed char* __restrict__ cb) {
  __shared__ __align__(16) u64 rays[256];
  gpo_build_rays(rays);
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const unsigned j = idx[i];
  const u64 p = P[j], o = O[j];
  u64 moves = gpo_mobility(p, o);
  const int cnt = moves ? popc(moves) : 1;
  const unsigned base = atomicAdd(counter, static_cast<unsigned>(cnt));
  if (base + cnt > cap) return;  // the host checks the counter against cap
  if (pa) {
    for (int k = 0; k < cnt; ++k) {
      ca[base + k] = static_cast<signed char>(-pb[j]);
      cb[base + k] = static_cast<signed char>(-pa[j]);
    }
  }
  if (!moves) {
    cP[base] = o;
    cO[base] = p;
    cparent[base] = j;
    cmove[base] = static_cast<unsigned char>(kMovePassDev);
    return;
  }
  for (int k = 0; moves; ++k) {
    const u64 bit = moves & (0ULL - moves);
    moves ^= bit;
    const int sq = ctz64(bit);
    const u64 f = gpo_flip(p, o, sq, rays);
    cP[base + k] = o ^ f;
    cO[base + k] = p ^ f ^ bit;
    cparent[base + k] = j;
    cmove[base + k] = static_cast<unsigned char>(sq);
  }
}

// acc[parent] = max over children of (-score) packed with the move;
// node counts of children are added to their parent's.
__global__ void combine_kernel(const signed char* __restrict__ cscore,
                               const unsigned* __restrict__ cparent,
                               const unsigned char* __restrict__ cmove,
                               const unsigned long long* __restrict__ cnodes, int count,
                               unsigned* __restrict__ acc, unsigned long long* __restrict__ nodes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int v = -static_cast<int>(cscore[i]);
  atomicMax(&acc[cparent[i]], (static_cast<unsigned>(v + 128) << 8) | cmove[i]);
  if (nodes && cnodes) atomicAdd(&nodes[cparent[i]], cnodes[i]);
}

__global__ void finalize_kernel(const unsigned* __restrict__ idx, int m,
                                const unsigned* __restrict__ acc, signed char* __restrict__ score,
                                signed char* __restrict__ best) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const unsigned a = acc[idx[i]];
  score[idx[i]] = static_cast<signed char>(static_cast<int>(a >> 8) - 128);
  if (best) best[idx[i]] = static_cast<signed char>(a & 255u);
}

// ---- principal-variation-first expansion (the expand_windows option) ----
// A marked position's children split in two: the first in fastest-first
// order (fewest replies for the opponent, lowest square on ties; the pass
// child when the position must pass) goes to set A at the parent's slot i,
// the others to set B.  A is searched with a full window; B with a null
// window around the value A gives the parent; only the B children that beat
// it are searched again (set C) -- the order alpha-beta itself would use.
__global__ void expand_first_kernel(const u64* __restrict__ P, const u64* __restrict__ O,
                                    const unsigned* __restrict__ idx, int m,
                                    u64* __restrict__ aP, u64* __restrict__ aO,
                                    unsigned* __restrict__ aparent,
                                    unsigned char* __restrict__ amove, u64* __restrict__ bP,
                                    u64* __restrict__ bO, unsigned* __restrict__ bparent,
                                    unsigned char* __restrict__ bmove,
                                    unsigned* __restrict__ counter, unsigned cap) {
  __shared__ __align__(16) u64 rays[256];
  gpo_build_rays(rays);
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const unsigned j = idx[i];
  const u64 p = P[j], o = O[j];
  const u64 moves = gpo_mobility(p, o);
  aparent[i] = j;
  if (!moves) {
    aP[i] = o;
    aO[i] = p;
    amove[i] = static_cast<unsigned char>(kMovePassDev);
    return;
  }
  int first = -1, first_key = 99;
  for (u64 t = moves; t; t &= t - 1) {
    const int sq = ctz64(t);
    const u64 bit = 1ULL << sq;
    const u64 f = gpo_flip(p, o, sq, rays);
    const int key = popc(gpo_mobility(o ^ f, p ^ f ^ bit));
    if (key < first_key) {
      first_key = key;
      first = sq;
    }
  }
  {
    const u64 bit = 1ULL << first;
    const u64 f = gpo_flip(p, o, first, rays);
    aP[i] = o ^ f;
    aO[i] = p ^ f ^ bit;
    amove[i] = static_cast<unsigned char>(first);
  }
  const int rest = popc(moves) - 1;
  if (rest == 0) return;
  const unsigned base = atomicAdd(counter, static_cast<unsigned>(rest));
  if (base + rest > cap) return;  // the host checks the counter against cap
  int k = 0;
  for (u64 t = moves & ~(1ULL << first); t; t &= t - 1, ++k) {
    const int sq = ctz64(t);
    const u64 bit = 1ULL << sq;
    const u64 f = gpo_flip(p, o, sq, rays);
    bP[base + k] = o ^ f;
    bO[base + k] = p ^ f ^ bit;
    bparent[base + k] = j;
    bmove[base + k] = static_cast<unsigned char>(sq);
  }
}

// bound[parent] = the parent's value through its first child (exact).
__global__ void pvs_bound_kernel(const signed char* __restrict__ ascore,
                                 const unsigned* __restrict__ aparent, int m,
                                 signed char* __restrict__ bound) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) bound[aparent[i]] = static_cast<signed char>(-ascore[i]);
}

// The B children's windows: the null window (bound, bound + 1) of the
// parent, negated and swapped.
__global__ void pvs_window_kernel(const unsigned* __restrict__ bparent, int nb,
                                  const signed char* __restrict__ bound,
                                  signed char* __restrict__ ba, signed char* __restrict__ bb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int v = bound[bparent[i]];
  ba[i] = static_cast<signed char>(-v - 1);
  bb[i] = static_cast<signed char>(-v);
}

// B children that beat their parent's bound: gathered into set C with the
// window (-64, -bound), the parent's (bound, 64).
__global__ void pvs_research_kernel(const u64* __restrict__ bP, const u64* __restrict__ bO,
                                    const unsigned* __restrict__ bparent,
                                    const unsigned char* __restrict__ bmove,
                                    const signed char* __restrict__ bscore, int nb,
                                    const signed char* __restrict__ bound,
                                    u64* __restrict__ cP, u64* __restrict__ cO,
                                    unsigned* __restrict__ cparent,
                                    unsigned char* __restrict__ cmove, signed char* __restrict__ ca,
                                    signed char* __restrict__ cb, unsigned* __restrict__ counter) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const unsigned j = bparent[i];
  if (-static_cast<int>(bscore[i]) <= bound[j]) return;
  const unsigned k = atomicAdd(counter, 1u);  // k < nb: one slot per B child at most
  cP[k] = bP[i];
  cO[k] = bO[i];
  cparent[k] = j;
  cmove[k] = bmove[i];
  ca[k] = -64;
  cb[k] = static_cast<signed char>(-bound[j]);
}

// ---- recursive principal-variation-first expansion (expand_windows = 2) ----
// Windows of a parent (pa/pb, null = -64/64) as seen from its children.
__device__ __forceinline__ int window_lo(const signed char* pa, unsigned j) {
  return pa ? pa[j] : -64;
}
__device__ __forceinline__ int window_hi(const signed char* pb, unsigned j) {
  return pb ? pb[j] : 64;
}

// ca/cb[i] = the window of child i: its parent's window negated and swapped.
__global__ void child_window_kernel(const unsigned* __restrict__ cparent, int count,
                                    const signed char* __restrict__ pa,
                                    const signed char* __restrict__ pb, signed char* __restrict__ ca,
                                    signed char* __restrict__ cb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const unsigned j = cparent[i];
  ca[i] = static_cast<signed char>(-window_hi(pb, j));
  cb[i] = static_cast<signed char>(-window_lo(pa, j));
}

// The siblings of first children: skipped when the first child already cut
// the parent off (bound >= beta); the others get the null window above
// a' = max(alpha, bound), and flag[k] = 1 when the parent's window is wider
// than that null window (a sibling that beats a' must then be searched
// again for its value).  skip[k] = 1 when the sibling's result must stay out
// of the parent's max: its parent is re-searched and a' = bound, so the
// sibling is worth at most the first child's value unless its re-search
// says otherwise (a bound tying the first child must not supply the move).
// When a' = alpha > bound the parent fails low and every sibling's upper
// bound has to count.
__global__ void pvs_siblings_kernel(const u64* __restrict__ bP, const u64* __restrict__ bO,
                                    const unsigned* __restrict__ bparent,
                                    const unsigned char* __restrict__ bmove, int nb,
                                    const signed char* __restrict__ pa,
                                    const signed char* __restrict__ pb,
                                    const signed char* __restrict__ bound, u64* __restrict__ oP,
                                    u64* __restrict__ oO, unsigned* __restrict__ opar,
                                    unsigned char* __restrict__ omove, signed char* __restrict__ oa,
                                    signed char* __restrict__ ob, unsigned char* __restrict__ oflag,
                                    unsigned char* __restrict__ oskip,
                                    unsigned* __restrict__ counter) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const unsigned j = bparent[i];
  const int lo = window_lo(pa, j), hi = window_hi(pb, j), b = bound[j];
  if (b >= hi) return;
  const int a2 = b > lo ? b : lo;
  const unsigned k = atomicAdd(counter, 1u);  // k < nb
  oP[k] = bP[i];
  oO[k] = bO[i];
  opar[k] = j;
  omove[k] = bmove[i];
  oa[k] = static_cast<signed char>(-a2 - 1);
  ob[k] = static_cast<signed char>(-a2);
  oflag[k] = hi > a2 + 1 ? 1 : 0;
  oskip[k] = hi > a2 + 1 && b >= lo ? 1 : 0;
}

// Flagged siblings that beat a': searched again with the window (a', beta)
// of the parent, i.e. (-beta, -a') for the child.
__global__ void pvs_research2_kernel(const u64* __restrict__ sP, const u64* __restrict__ sO,
                                     const unsigned* __restrict__ spar,
                                     const unsigned char* __restrict__ smove,
                                     const signed char* __restrict__ sscore,
                                     const unsigned char* __restrict__ sflag, int ns,
                                     const signed char* __restrict__ pa,
                                     const signed char* __restrict__ pb,
                                     const signed char* __restrict__ bound, u64* __restrict__ cP,
                                     u64* __restrict__ cO, unsigned* __restrict__ cpar,
                                     unsigned char* __restrict__ cmove, signed char* __restrict__ ca,
                                     signed char* __restrict__ cb, unsigned* __restrict__ counter) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns || !sflag[i]) return;
  const unsigned j = spar[i];
  const int lo = window_lo(pa, j), hi = window_hi(pb, j), b = bound[j];
  const int a2 = b > lo ? b : lo;
  if (-static_cast<int>(sscore[i]) <= a2) return;
  const unsigned k = atomicAdd(counter, 1u);  // k < ns
  cP[k] = sP[i];
  cO[k] = sO[i];
  cpar[k] = j;
  cmove[k] = smove[i];
  ca[k] = static_cast<signed char>(-hi);
  cb[k] = static_cast<signed char>(-a2);
}

// combine_kernel for siblings: node counts always, values only for the
// unflagged ones (a flagged sibling's value comes from its re-search, or is
// a bound no better than the first child's).
__global__ void combine_masked_kernel(const signed char* __restrict__ cscore,
                                      const unsigned* __restrict__ cparent,
                                      const unsigned char* __restrict__ cmove,
                                      const unsigned long long* __restrict__ cnodes,
                                      const unsigned char* __restrict__ skip, int count,
                                      unsigned* __restrict__ acc,
                                      unsigned long long* __restrict__ nodes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  if (!skip[i]) {
    const int v = -static_cast<int>(cscore[i]);
    atomicMax(&acc[cparent[i]], (static_cast<unsigned>(v + 128) << 8) | cmove[i]);
  }
  if (nodes && cnodes) atomicAdd(&nodes[cparent[i]], cnodes[i]);
}

cudaError_t launch_child_window(const unsigned* cparent, int count, const signed char* pa,
                                const signed char* pb, signed char* ca, signed char* cb,
                                cudaStream_t s) {
  child_window_kernel<<<(count + 255) / 256, 256, 0, s>>>(cparent, count, pa, pb, ca, cb);
  return cudaGetLastError();
}

cudaError_t launch_pvs_siblings(const u64* bP, const u64* bO, const unsigned* bparent,
                                const unsigned char* bmove, int nb, const signed char* pa,
                                const signed char* pb, const signed char* bound, u64* oP, u64* oO,
                                unsigned* opar, unsigned char* omove, signed char* oa,
                                signed char* ob, unsigned char* oflag, unsigned char* oskip,
                                unsigned* counter, cudaStream_t s) {
  pvs_siblings_kernel<<<(nb + 255) / 256, 256, 0, s>>>(bP, bO, bparent, bmove, nb, pa, pb, bound,
                                                       oP, oO, opar, omove, oa, ob, oflag, oskip,
                                                       counter);
  return cudaGetLastError();
}

cudaError_t launch_pvs_research2(const u64* sP, const u64* sO, const unsigned* spar,
                                 const unsigned char* smove, const signed char* sscore,
                                 const unsigned char* sflag, int ns, const signed char* pa,
                                 const signed char* pb, const signed char* bound, u64* cP, u64* cO,
                                 unsigned* cpar, unsigned char* cmove, signed char* ca,
                                 signed char* cb, unsigned* counter, cudaStream_t s) {
  pvs_research2_kernel<<<(ns + 255) / 256, 256, 0, s>>>(sP, sO, spar, smove, sscore, sflag, ns,
                                                        pa, pb, bound, cP, cO, cpar, cmove, ca,
                                                        cb, counter);
  return cudaGetLastError();
}

cudaError_t launch_combine_masked(const signed char* cscore, const unsigned* cparent,
                                  const unsigned char* cmove, const unsigned long long* cnodes,
                                  const unsigned char* skip, int count, unsigned* acc,
                                  unsigned long long* nodes, cudaStream_t s) {
  combine_masked_kernel<<<(count + 255) / 256, 256, 0, s>>>(cscore, cparent, cmove, cnodes, skip,
                                                            count, acc, nodes);
  return cudaGetLastError();
}

cudaError_t launch_expand_first(const u64* P, const u64* O, const unsigned* idx, int m, u64* aP,
                                u64* aO, unsigned* aparent, unsigned char* amove, u64* bP, u64* bO,
                                unsigned* bparent, unsigned char* bmove, unsigned* counter,
                                unsigned cap, cudaStream_t s) {
  expand_first_kernel<<<(m + 127) / 128, 128, 0, s>>>(P, O, idx, m, aP, aO, aparent, amove, bP, bO,
                                                       bparent, bmove, counter, cap);
  return cudaGetLastError();
}

cudaError_t launch_pvs_bound(const signed char* ascore, const unsigned* aparent, int m,
                             signed char* bound, cudaStream_t s) {
  pvs_bound_kernel<<<(m + 255) / 256, 256, 0, s>>>(ascore, aparent, m, bound);
  return cudaGetLastError();
}

cudaError_t launch_pvs_window(const unsigned* bparent, int nb, const signed char* bound,
                              signed char* ba, signed char* bb, cudaStream_t s) {
  pvs_window_kernel<<<(nb + 255) / 256, 256, 0, s>>>(bparent, nb, bound, ba, bb);
  return cudaGetLastError();
}

cudaError_t launch_pvs_research(const u64* bP, const u64* bO, const unsigned* bparent,
                                const unsigned char* bmove, const signed char* bscore, int nb,
                                const signed char* bound, u64* cP, u64* cO, unsigned* cparent,
                                unsigned char* cmove, signed char* ca, signed char* cb,
                                unsigned* counter, cudaStream_t s) {
  pvs_research_kernel<<<(nb + 255) / 256, 256, 0, s>>>(bP, bO, bparent, bmove, bscore, nb, bound,
                                                       cP, cO, cparent, cmove, ca, cb, counter);
  return cudaGetLastError();
}

cudaError_t launch_expand(const u64* P, const u64* O, const unsigned* idx, int m, u64* cP, u64* cO,
                          unsigned* cparent, unsigned char* cmove, unsigned* counter, unsigned cap,
                          const signed char* pa, const signed char* pb, signed char* ca,
                          signed char* cb, cudaStream_t s) {
  expand_kernel<<<(m + 127) / 128, 128, 0, s>>>(P, O, idx, m, cP, cO, cparent, cmove, counter,
                                                 cap, pa, pb, ca, cb);
  return cudaGetLastError();
}

cudaError_t launch_combine(const signed char* cscore, const unsigned* cparent,
                           const unsigned char* cmove, const unsigned long long* cnodes, int count,
                           unsigned* acc, unsigned long long* nodes, cudaStream_t s) {
  combine_kernel<<<(count + 255) / 256, 256, 0, s>>>(cscore, cparent, cmove, cnodes, count, acc,
                                                     nodes);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const unsigned* idx, int m, const unsigned* acc, signed char* score,
                            signed char* best, cudaStream_t s) {
  finalize_kernel<<<(m + 255) / 256, 256, 0, s>>>(idx, m, acc, score, best);
  return cudaGetLastError();
}

}  // namespace gpo

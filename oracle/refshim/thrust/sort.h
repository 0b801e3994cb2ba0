/*
 * Host stand-in for the one Thrust call the reference search makes:
 * thrust::sort_by_key(thrust::seq, keys, keys + n, values) (solver.cu:92),
 * which orders an upper node's legal moves by ascending opponent mobility.
 *
 * Thrust (bundled with CUDA 13.0) implements sort_by_key for the sequential
 * policy as a stable sort, so equal keys keep their generation order
 * (corners first, then lowest square, node.cuh:21-28).  This restatement is
 * a stable insertion sort on at most 46 pairs, which gives the same order.
 * Move order does not change scores, only node counts.
 */
#pragma once
#include "execution_policy.h"

namespace thrust {
template <class K, class V>
void sort_by_key(const detail_seq_t&, K* first, K* last, V* values) {
  const long n = last - first;
  for (long i = 1; i < n; ++i) {
    K k = first[i];
    V v = values[i];
    long j = i - 1;
    while (j >= 0 && k < first[j]) {
      first[j + 1] = first[j];
      values[j + 1] = values[j];
      --j;
    }
    first[j + 1] = k;
    values[j + 1] = v;
  }
}
}  // namespace thrust

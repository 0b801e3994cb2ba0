/* Host stand-in for thrust::seq (see sort.h in this directory). */
#pragma once

namespace thrust {
struct detail_seq_t {};
static const detail_seq_t seq{};
}  // namespace thrust

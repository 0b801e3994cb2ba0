// The whole solve pipeline of the library -- the C-ABI layer (capi.cu), the
// bucketing and generator kernels (prep.cu), the plain and batched search
// kernels and the allocation-free entry point -- compiled as
// host C++ and run on CPU threads under the SIMT emulation
// (tests/simt/simt_prelude.h, tests/simt/cuda_runtime.h).  Test
// infrastructure only: the product never links this file, and the library
// it makes (oracle/lib/libpipeline_emu.so) is loaded only by
// tests/test_pipeline_emu.py, which calls the same C ABI the product
// exports and checks it against the golden scores and the oracle without a
// GPU.
//
// The emulation build copies batched.cu, prep.cu and plain.cu with their
// `k<<<grid, block, smem, stream>>>(args)` launches rewritten to
// simt_launch(k, simt_cfg(grid, block, smem, stream), args) (see
// gpuothello2_gb300/build.py); noalloc.cu and capi.cu compile unchanged.  The learned orderer (mlp.cu, tensor-core code) is left out:
// the solver sees no network loaded.

// batched.cu's dynamic shared memory is `extern __shared__`: keep
// __shared__ empty for it ...
#include "batched_emu.cu"

// ... and make the other kernels' static __shared__ arrays function
// statics: blocks of an ordinary launch run one after another.
#undef __shared__
#define __shared__ static
#include "prep_emu.cu"
#include "plain_emu.cu"
#include "../gpuothello2_gb300/csrc/noalloc.cu"
#include "../gpuothello2_gb300/csrc/capi.cu"

thread_local simt_uint3 threadIdx, blockIdx;
simt_uint3 blockDim, gridDim;
thread_local SimtWarp* simt_warp = nullptr;
SimtBarrier* simt_block = nullptr;
std::mutex simt_cas128_mutex;

namespace gpo {

// dynamic shared memory of a block of the batched kernel (blocks of a launch
// run one after another): the ray table, the split-node state and up to 30
// frame slots for 256 threads
constexpr size_t kEmuSmemWords = (kTableBytes + 256 * (kSplitBytes + 30 * kFrameBytes)) / 8 + 8;
alignas(16) u64 smem_raw[kEmuSmemWords];

// the learned orderer is not part of this build
bool mlp_loaded() { return false; }
int mlp_order_frontier(const u64*, const u64*, const unsigned*, long, int, u64*, u64*, long,
                       unsigned long long*, u64*, int, cudaStream_t, unsigned* launched,
                       long* frontier) {
  *launched = 0;
  *frontier = 0;
  return GPO_ERR_ARG;
}

}  // namespace gpo

// The whole solve pipeline of the library -- the C-ABI layer (capi.cu), the
// preparation, expansion and combination kernels (prep.cu), the plain and
// batched search kernels and the allocation-free entry point -- compiled as
// host C++ and run on CPU threads under the SIMT emulation
// (tests/simt/simt_prelude.h, tests/simt/cuda_runtime.h).  Test
// infrastructure only: the product never links this file, and the library
// it makes (oracle/lib/libpipeline_emu.so) is loaded only by
// tests/test_pipeline_emu.py, which calls the same C ABI the product
// exports and checks it against the golden scores and the oracle without a
// GPU.
//
// The emulation build copies prep.cu and plain.cu with their
// `k<<<grid, block, smem, stream>>>(args)` launches rewritten to
// simt_launch(k, simt_cfg(grid, block, smem, stream), args) (see
// gpuothello2_gb300/build.py); batched.cu, noalloc.cu and capi.cu compile
// unchanged.  The learned orderer (mlp.cu, tensor-core code) is left out:
// the solver sees no network loaded.

// batched.cu's dynamic shared memory is `extern __shared__`: keep
// __shared__ empty for it ...
#include "../gpuothello2_gb300/csrc/batched.cu"

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

// dynamic shared memory of the one emulated block of the batched kernel
constexpr size_t kEmuSmemWords = (kRayBytes + 256 * 31 * kFrameBytes) / 8 + 8;
alignas(16) u64 smem_raw[kEmuSmemWords];

// the learned orderer is not part of this build
bool mlp_loaded() { return false; }
int mlp_order_roots(const u64*, const u64*, const unsigned*, long, u64*, cudaStream_t,
                    unsigned* launched) {
  *launched = 0;
  return GPO_ERR_ARG;
}

namespace {

// The cooperative launch of batched_kernel: every block at once (their
// lanes may wait on one another), each with its own threads.
cudaError_t emu_cooperative(const void* f, dim3 grid, dim3 block, void** args) {
  if (f != reinterpret_cast<const void*>(batched_kernel) || grid.x != 1) return 1;
  const size_t smem = kRayBytes + static_cast<size_t>(block.x) *
                                      (static_cast<const BatchedArgs*>(args[0])->smem_top >= 2
                                           ? static_cast<const BatchedArgs*>(args[0])->smem_top - 1
                                           : 0) *
                                      kFrameBytes;
  if (smem > sizeof(smem_raw)) return cudaErrorInvalidConfiguration;
  const BatchedArgs a = *static_cast<const BatchedArgs*>(args[0]);
  simt_run_block(0, 1, block.x, [&] { batched_kernel(a); });
  return cudaSuccess;
}

struct HookInstaller {
  HookInstaller() { simt_coop_hook() = emu_cooperative; }
} g_install_hook;

}  // namespace
}  // namespace gpo

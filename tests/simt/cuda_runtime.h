// Stand-in for the CUDA runtime header when a kernel source is compiled as
// host C++ by the SIMT emulation (test infrastructure; see simt_prelude.h).
// Declares only the types and calls the solver's launcher code names; the
// calls report "not supported" -- the emulation launches kernels itself.
#pragma once
#include <cstddef>

typedef int cudaError_t;
typedef void* cudaStream_t;
static const cudaError_t cudaSuccess = 0;
static const cudaError_t cudaErrorNotSupported = 801;
static const cudaError_t cudaErrorInvalidConfiguration = 9;
enum cudaFuncAttribute { cudaFuncAttributeMaxDynamicSharedMemorySize = 8 };
enum cudaDeviceAttr { cudaDevAttrMaxSharedMemoryPerMultiprocessor = 81 };

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

template <class F>
inline cudaError_t cudaFuncSetAttribute(F, cudaFuncAttribute, int) {
  return cudaErrorNotSupported;
}
template <class F>
inline cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessor(int*, F, int, size_t) {
  return cudaErrorNotSupported;
}
inline cudaError_t cudaGetDevice(int*) { return cudaErrorNotSupported; }
inline cudaError_t cudaDeviceGetAttribute(int*, cudaDeviceAttr, int) {
  return cudaErrorNotSupported;
}
inline cudaError_t cudaLaunchCooperativeKernel(const void*, dim3, dim3, void**, size_t,
                                               cudaStream_t) {
  return cudaErrorNotSupported;
}
inline cudaError_t cudaGetLastError() { return cudaSuccess; }

// Stand-in for the CUDA runtime header when the solver's sources are
// compiled as host C++ by the SIMT emulation (test infrastructure; see
// simt_prelude.h).  Device memory is host memory, every stream is the
// calling thread (work runs when it is enqueued), events read the steady
// clock, and the emulated device has one SM.  Kernel launches written
// `k<<<grid, block, smem, stream>>>(args)` are rewritten to simt_launch()
// when the emulation build copies a source.
#pragma once
#include <chrono>
#include <cstddef>
#include <cstdlib>
#include <cstring>

typedef int cudaError_t;
static const cudaError_t cudaSuccess = 0;
static const cudaError_t cudaErrorInvalidConfiguration = 9;
static const cudaError_t cudaErrorMemoryAllocation = 2;

struct SimtStream {
  int unused;
};
typedef SimtStream* cudaStream_t;
static const unsigned cudaStreamNonBlocking = 1;

struct SimtEvent {
  std::chrono::steady_clock::time_point t;
};
typedef SimtEvent* cudaEvent_t;

enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3
};
enum cudaFuncAttribute { cudaFuncAttributeMaxDynamicSharedMemorySize = 8 };
enum cudaDeviceAttr {
  cudaDevAttrMultiProcessorCount = 16,
  cudaDevAttrMaxSharedMemoryPerMultiprocessor = 81
};

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

struct cudaDeviceProp {
  char name[256];
  int multiProcessorCount;
  size_t totalGlobalMem;
};

// ---- memory: host memory, filled with a pattern so that a read of memory
// the code never wrote shows up as a wrong result ----
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t n) {
  const size_t bytes = ((n ? n : 1) + 255) / 256 * 256;
  void* m = std::aligned_alloc(256, bytes);
  if (!m) return cudaErrorMemoryAllocation;
  std::memset(m, 0xCD, bytes);
  *p = static_cast<T*>(m);
  return cudaSuccess;
}
inline cudaError_t cudaFree(void* p) {
  std::free(p);
  return cudaSuccess;
}
inline cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind,
                                   cudaStream_t = nullptr) {
  if (n) std::memmove(d, s, n);
  return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind k) {
  return cudaMemcpyAsync(d, s, n, k);
}
inline cudaError_t cudaMemsetAsync(void* p, int v, size_t n, cudaStream_t = nullptr) {
  if (n) std::memset(p, v, n);
  return cudaSuccess;
}
template <class T>
inline cudaError_t cudaGetSymbolAddress(void** p, T& symbol) {
  *p = static_cast<void*>(&symbol);
  return cudaSuccess;
}

// ---- streams and events ----
inline cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned) {
  *s = new SimtStream();
  return cudaSuccess;
}
inline cudaError_t cudaStreamDestroy(cudaStream_t s) {
  delete s;
  return cudaSuccess;
}
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaEventCreate(cudaEvent_t* e) {
  *e = new SimtEvent();
  return cudaSuccess;
}
inline cudaError_t cudaEventDestroy(cudaEvent_t e) {
  delete e;
  return cudaSuccess;
}
inline cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t = nullptr) {
  e->t = std::chrono::steady_clock::now();
  return cudaSuccess;
}
inline cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) {
  *ms = std::chrono::duration<float, std::milli>(b->t - a->t).count();
  return cudaSuccess;
}

// ---- device: one SM with a GB300's shared memory ----
inline cudaError_t cudaGetDevice(int* d) {
  *d = 0;
  return cudaSuccess;
}
inline cudaError_t cudaSetDevice(int d) { return d == 0 ? cudaSuccess : 1; }
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int) {
  std::memset(p, 0, sizeof(*p));
  std::strcpy(p->name, "SIMT emulation");
  p->multiProcessorCount = 1;
  return cudaSuccess;
}
inline cudaError_t cudaDeviceGetAttribute(int* v, cudaDeviceAttr a, int) {
  *v = a == cudaDevAttrMultiProcessorCount ? 1 : 233472;
  return cudaSuccess;
}
template <class F>
inline cudaError_t cudaFuncSetAttribute(F, cudaFuncAttribute, int) {
  return cudaSuccess;
}
template <class F>
inline cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessor(int* n, F, int, size_t) {
  *n = 1;
  return cudaSuccess;
}
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline const char* cudaGetErrorName(cudaError_t) { return "simtError"; }
inline const char* cudaGetErrorString(cudaError_t) { return "error in the SIMT emulation"; }

// ---- CUDA graphs: not emulated (capture reports "not supported") ----
struct SimtGraph {
  int unused;
};
typedef SimtGraph* cudaGraph_t;
typedef SimtGraph* cudaGraphExec_t;
enum cudaStreamCaptureMode { cudaStreamCaptureModeThreadLocal = 1 };
static const cudaError_t cudaErrorNotSupported = 801;
inline cudaError_t cudaStreamBeginCapture(cudaStream_t, cudaStreamCaptureMode) {
  return cudaErrorNotSupported;
}
inline cudaError_t cudaStreamEndCapture(cudaStream_t, cudaGraph_t* g) {
  *g = nullptr;
  return cudaErrorNotSupported;
}
inline cudaError_t cudaGraphInstantiate(cudaGraphExec_t*, cudaGraph_t, unsigned long long) {
  return cudaErrorNotSupported;
}
inline cudaError_t cudaGraphLaunch(cudaGraphExec_t, cudaStream_t) { return cudaErrorNotSupported; }
inline cudaError_t cudaGraphDestroy(cudaGraph_t) { return cudaSuccess; }
inline cudaError_t cudaGraphExecDestroy(cudaGraphExec_t) { return cudaSuccess; }
inline cudaError_t cudaMallocHost(void* p, size_t n) {
  *static_cast<void**>(p) = std::malloc(n ? n : 1);
  return cudaSuccess;
}
inline cudaError_t cudaFreeHost(void* p) {
  std::free(p);
  return cudaSuccess;
}

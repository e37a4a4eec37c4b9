// A fixed-size block of device memory for entry points that must not allocate.
//
// Some callers cannot let a library call allocate device memory: a host code that has handed
// the whole device to its own pool allocator (PETSc or a caching allocator owns every byte, so a
// cudaMalloc inside the call fails or evicts), or a time-stepping loop that must not meet the
// device-wide synchronisation a cudaMalloc / cudaFree brings. For those callers the scratch that
// an entry point would otherwise allocate lives here, in one file-scope __device__ array whose
// size is fixed when the library is built. The array is per device and per process, and it is
// shared: two calls that use it at the same time (from two host threads, or on two streams
// without ordering between them) overwrite each other's intermediate results.
#include <cuda_runtime.h>

#include <mutex>

#include "cm_noalloc.h"

static __device__ __align__(256) unsigned char cm_static_scratch[cm::kStaticScratchBytes];

namespace cm {

cudaError_t static_scratch(void **ptr, size_t *bytes) {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static void *addr[kMaxDevices] = {};
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    // first use on this device (the current one): loads this module there and looks the array up
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, cm_static_scratch);
    if (e != cudaSuccess) return e;
    addr[dev] = p;
  }
  *ptr = addr[dev];
  *bytes = kStaticScratchBytes;
  return cudaSuccess;
}

}  // namespace cm

// Fixed-size device scratch for the entry points that allocate nothing (cm_noalloc.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace cm {

// 8 MiB per device. Nothing in it has to start at zero: every user writes all of the scratch
// it later reads within the same call.
constexpr size_t kStaticScratchBytes = size_t(8) << 20;

// Address and size of the scratch on the current device. The first call on a device looks the
// address up (cudaGetSymbolAddress, with that device current) and caches it; later calls only
// read the cache.
cudaError_t static_scratch(void **ptr, size_t *bytes);

}  // namespace cm

// memory.cuh -- the library's device and pinned-host memory cache.
//
// cudaMalloc/cudaFree and cudaMallocHost/cudaFreeHost are slow and cudaFree
// synchronizes the device, so every allocation of the runtime (batch arrays,
// propagator scratch, Anderson state, warm-start buffers) goes through this
// cache: a released block is kept for its device and handed out again to a
// request of at most its size (and at least 2/3 of it).  A failed cudaMalloc
// releases the cached blocks of the device and retries once.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace scft {

cudaError_t mem_alloc(void **p, size_t bytes);
void mem_free(void *p);
cudaError_t host_alloc(void **p, size_t bytes);
void host_free(void *p);
// Release every cached (unused) device block of the current device and every
// cached pinned host block; returns the bytes released.
size_t mem_trim();

}  // namespace scft

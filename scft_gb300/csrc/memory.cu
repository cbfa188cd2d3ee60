// memory.cu -- device and pinned-host memory cache of the library (see memory.cuh).
#include <atomic>
#include <map>
#include <mutex>
#include <unordered_map>
#include <utility>

#include "memory.cuh"
#include "scft.h"

namespace scft {
namespace {

// Requests are rounded up: to a power of two up to 1 MiB, to a multiple of
// 2 MiB above, so that blocks of a repeated workload match exactly.
size_t round_size(size_t b) {
  if (b == 0) b = 1;
  if (b <= (1u << 20)) {
    size_t r = 256;
    while (r < b) r <<= 1;
    return r;
  }
  const size_t g = (size_t)2 << 20;
  return (b + g - 1) / g * g;
}

struct Pool {
  std::mutex mu;
  std::multimap<std::pair<int, size_t>, void *> cached;     // (device or -1 for host, size) -> block
  std::unordered_map<void *, std::pair<int, size_t>> live;  // block -> (device, size)
};

std::atomic<long long> g_requests{0}, g_cuda_allocs{0};

Pool &pool() {
  static Pool *p = new Pool();  // never destroyed: blocks may be released during process exit
  return *p;
}

// A cached block of `dev` with size in [need, need * 3 / 2], removed from the cache.
void *take(Pool &P, int dev, size_t need, size_t *got) {
  auto it = P.cached.lower_bound({dev, need});
  if (it == P.cached.end() || it->first.first != dev || it->first.second > need + need / 2) return nullptr;
  void *p = it->second;
  *got = it->first.second;
  P.cached.erase(it);
  return p;
}

size_t release_cached(Pool &P, int dev) {
  size_t bytes = 0;
  for (auto it = P.cached.begin(); it != P.cached.end();) {
    if (it->first.first == dev) {
      if (dev < 0) cudaFreeHost(it->second);
      else cudaFree(it->second);
      bytes += it->first.second;
      it = P.cached.erase(it);
    } else {
      ++it;
    }
  }
  return bytes;
}

cudaError_t acquire(void **p, size_t bytes, bool host) {
  *p = nullptr;
  int dev = -1;
  if (!host) {
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
  }
  const size_t need = round_size(bytes);
  g_requests++;
  Pool &P = pool();
  std::lock_guard<std::mutex> g(P.mu);
  size_t got = 0;
  if (void *q = take(P, dev, need, &got)) {
    P.live[q] = {dev, got};
    *p = q;
    return cudaSuccess;
  }
  g_cuda_allocs++;
  cudaError_t e = host ? cudaMallocHost(p, need) : cudaMalloc(p, need);
  if (e != cudaSuccess) {
    cudaGetLastError();
    release_cached(P, dev);
    g_cuda_allocs++;
    e = host ? cudaMallocHost(p, need) : cudaMalloc(p, need);
    if (e != cudaSuccess) {
      cudaGetLastError();
      *p = nullptr;
      return e;
    }
  }
  P.live[*p] = {dev, need};
  return cudaSuccess;
}

void release(void *p) {
  if (!p) return;
  // as cudaFree would: no kernel or copy may still use the block when another
  // request can receive it
  cudaDeviceSynchronize();
  Pool &P = pool();
  std::lock_guard<std::mutex> g(P.mu);
  auto it = P.live.find(p);
  if (it == P.live.end()) return;  // not from the cache
  P.cached.insert({it->second, p});
  P.live.erase(it);
}

}  // namespace

cudaError_t mem_alloc(void **p, size_t bytes) { return acquire(p, bytes, false); }
void mem_free(void *p) { release(p); }
cudaError_t host_alloc(void **p, size_t bytes) { return acquire(p, bytes, true); }
void host_free(void *p) { release(p); }

size_t mem_trim() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  Pool &P = pool();
  std::lock_guard<std::mutex> g(P.mu);
  return release_cached(P, dev) + release_cached(P, -1);
}

}  // namespace scft

extern "C" long long scft_mem_trim(void) { return (long long)scft::mem_trim(); }

extern "C" void scft_mem_counters(long long *requests, long long *cuda_allocs) {
  if (requests) *requests = scft::g_requests.load();
  if (cuda_allocs) *cuda_allocs = scft::g_cuda_allocs.load();
}

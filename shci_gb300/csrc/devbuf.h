// Device buffers and CUDA error plumbing for the SHCI library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>

namespace shci {

struct CudaError : std::runtime_error {
  cudaError_t code;
  CudaError(cudaError_t c, const std::string& where)
      : std::runtime_error(where + ": " + cudaGetErrorString(c)), code(c) {}
};
struct OomError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct ArgError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct OverflowError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define SHCI_CUDA(call)                                                        \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) throw ::shci::CudaError(e_, #call);                 \
  } while (0)

#define SHCI_LAUNCH_CHECK() SHCI_CUDA(cudaGetLastError())

// Device bytes held by one context against an optional budget, and the context's cache of
// released blocks.  A build or a PT2 pass allocates and frees scratch of the same sizes again
// and again (gigabytes at n = 40, where cudaMalloc / cudaFree of a large block costs about a
// millisecond and the free synchronises the device); a released block is kept and handed to
// the next request it fits (up to twice the size asked for).  All work of a context runs on
// its one stream, so a block reused after a release is ordered after the work that used it.
// A request that does not fit the device or the budget first returns the cache to the driver.
// The cache holds at most a quarter of the device's memory, so the driver always keeps room
// for what it allocates by itself (local memory of launches, library workspaces).
struct MemTracker {
  size_t budget = 0;  // 0 = unlimited
  size_t used = 0;    // held: live blocks and cached ones
  size_t peak = 0;
  size_t peak_live = 0;  // the most held by live blocks
  size_t cached = 0;     // held in the cache
  size_t cache_cap = 0;  // 0: not set yet (a quarter of the device's memory)
  std::multimap<size_t, void*> cache;  // released blocks by size in bytes

  MemTracker() = default;
  MemTracker(const MemTracker&) = delete;
  MemTracker& operator=(const MemTracker&) = delete;
  ~MemTracker() { flush(); }

  // A cached block of at least `bytes` (at most twice that); *got = its size.
  void* take(size_t bytes, size_t* got) {
    auto it = cache.lower_bound(bytes);
    if (it == cache.end() || it->first > 2 * bytes) return nullptr;
    void* p = it->second;
    *got = it->first;
    cached -= it->first;
    cache.erase(it);
    return p;
  }
  void give(void* p, size_t bytes) {
    if (cache_cap == 0) {
      size_t f = 0, t = 0;
      cache_cap = cudaMemGetInfo(&f, &t) == cudaSuccess ? t / 4 : 1;
    }
    if (cached + bytes > cache_cap) {
      cudaFree(p);
      used -= bytes;
      return;
    }
    cache.emplace(bytes, p);
    cached += bytes;
  }
  void note_live() {
    if (live() > peak_live) peak_live = live();
  }
  // Returns every cached block to the driver.
  void flush() {
    for (auto& kv : cache) cudaFree(kv.second);
    used -= cached;
    cached = 0;
    cache.clear();
  }
  // Bytes held by live blocks.
  size_t live() const { return used - cached; }
};

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  size_t cap = 0;
  MemTracker* mt = nullptr;

  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }

  void release() {
    if (p) {
      if (mt) mt->give(p, cap * sizeof(T));  // kept for the context's next request
      else cudaFree(p);
    }
    p = nullptr;
    n = cap = 0;
  }
  // Grows (never shrinks) capacity; contents are NOT preserved.
  void reserve(size_t k, double slack = 1.0) {
    if (k <= cap) return;
    release();
    size_t c = static_cast<size_t>(k * slack);
    if (c < k) c = k;
    if (c == 0) c = 1;
    const size_t bytes = c * sizeof(T);
    if (mt) {
      size_t got = 0;
      if (void* b = mt->take(bytes, &got)) {
        p = static_cast<T*>(b);
        cap = got / sizeof(T);
        mt->note_live();
        return;
      }
      if (mt->budget && mt->used + bytes > mt->budget) mt->flush();
      if (mt->budget && mt->used + bytes > mt->budget)
        throw OomError("device budget exceeded (" + std::to_string(mt->used + bytes) + " > " +
                       std::to_string(mt->budget) + " bytes)");
    }
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess && mt && mt->cached) {  // the cache first, then once more
      cudaGetLastError();
      mt->flush();
      e = cudaMalloc(&p, bytes);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      throw OomError("cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    cap = c;
    if (mt) {
      mt->used += bytes;
      if (mt->used > mt->peak) mt->peak = mt->used;
      mt->note_live();
    }
  }
  void resize(size_t k, double slack = 1.0) {
    reserve(k, slack);
    n = k;
  }
  // Grows capacity keeping the first n elements.
  void grow_keep(size_t k, cudaStream_t s, double slack = 1.5) {
    if (k <= cap) {
      n = k;
      return;
    }
    DevBuf<T> nb;
    nb.mt = mt;
    nb.reserve(k, slack);
    if (n) SHCI_CUDA(cudaMemcpyAsync(nb.p, p, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    std::swap(p, nb.p);
    std::swap(cap, nb.cap);
    nb.n = 0;
    n = k;
  }
  size_t bytes() const { return n * sizeof(T); }
  // Exchanges the buffers (and their tracker) of two DevBufs.
  void swap(DevBuf& o) {
    std::swap(p, o.p);
    std::swap(n, o.n);
    std::swap(cap, o.cap);
    std::swap(mt, o.mt);
  }
};

inline unsigned grid_for(size_t n, unsigned block, unsigned max_blocks = 152u * 64u) {
  size_t g = (n + block - 1) / block;
  if (g == 0) g = 1;
  if (g > max_blocks) g = max_blocks;
  return static_cast<unsigned>(g);
}

}  // namespace shci

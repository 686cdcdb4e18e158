// Device buffers and CUDA error plumbing for the SHCI library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
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

// Tracks device bytes held by one context against an optional budget.
struct MemTracker {
  size_t budget = 0;  // 0 = unlimited
  size_t used = 0;
  size_t peak = 0;
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
      cudaFree(p);
      if (mt) mt->used -= cap * sizeof(T);
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
    if (mt && mt->budget && mt->used + bytes > mt->budget)
      throw OomError("device budget exceeded (" + std::to_string(mt->used + bytes) + " > " +
                     std::to_string(mt->budget) + " bytes)");
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      throw OomError("cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    cap = c;
    if (mt) {
      mt->used += bytes;
      if (mt->used > mt->peak) mt->peak = mt->used;
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

// Device scan and stable LSD radix sort (hand-written; no library sort).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <utility>

#include "devbuf.h"

namespace shci {

// Scratch owned by the caller and reused across calls.
struct SortScratch {
  DevBuf<uint32_t> hist;     // [256 * n_tiles]
  DevBuf<uint32_t> part32;   // scan partials
  DevBuf<uint64_t> part64;
  DevBuf<uint64_t> kalt;     // ping-pong keys
  DevBuf<uint32_t> kalt32;
  DevBuf<uint32_t> valt32;   // ping-pong values
  DevBuf<uint64_t> valt64;
  void set_tracker(MemTracker* m) {
    hist.mt = part32.mt = kalt.mt = valt32.mt = valt64.mt = m;
    part64.mt = kalt32.mt = m;
  }
};

// out[i] = sum_{k<i} in[i]; returns the total (synchronises the stream).  in may equal out.
uint64_t exclusive_scan_u64(const uint64_t* in, uint64_t* out, size_t n, cudaStream_t s,
                            SortScratch& sc);
uint32_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s,
                            SortScratch& sc);
// Same without returning the total (no synchronisation); total written to *total_dev if set.
void exclusive_scan_u64_async(const uint64_t* in, uint64_t* out, size_t n, cudaStream_t s,
                              SortScratch& sc, uint64_t* total_dev);

// Stable sort of the first n (keys, vals) by key bits [begin_bit, end_bit).  When the
// result ends up in the scratch ping-pong buffers, their storage is swapped into `keys` /
// `vals`, so the caller's buffers always hold the sorted data on return.
void radix_sort_pairs(DevBuf<uint64_t>& keys, DevBuf<uint32_t>& vals, size_t n, int begin_bit,
                      int end_bit, cudaStream_t s, SortScratch& sc);
void radix_sort_pairs64(DevBuf<uint64_t>& keys, DevBuf<uint64_t>& vals, size_t n,
                        int begin_bit, int end_bit, cudaStream_t s, SortScratch& sc);
void radix_sort_pairs32(DevBuf<uint32_t>& keys, DevBuf<uint32_t>& vals, size_t n,
                        int begin_bit, int end_bit, cudaStream_t s, SortScratch& sc);

template <class T>
inline void swap_storage(DevBuf<T>& a, DevBuf<T>& b) {
  std::swap(a.p, b.p);
  std::swap(a.cap, b.cap);
  std::swap(a.n, b.n);
}

// vals[i] = i
void iota_u32(uint32_t* v, size_t n, cudaStream_t s);
// out[i] = src[idx[i]]
void gather_u64(const uint64_t* src, const uint32_t* idx, uint64_t* out, size_t n,
                cudaStream_t s);

}  // namespace shci

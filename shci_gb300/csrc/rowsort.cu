// Column order of the element store's rows (a post-pass of the Hamiltonian build).
//
// H*v (spmv.cu) streams a row's (col, val) pairs 32 at a time, one per lane, and each pair
// costs a scattered read of x[j] and a scattered atomic on y[j].  Those scattered accesses
// bound the kernel, and a warp instruction costs one L1 wavefront per distinct line it
// touches, so columns that fall in the same 32-byte sector or 128-byte line should sit in
// the same 32-element chunk of the row.  The build emits a row in the order its traversal
// finds the columns (unrelated to j), so this pass sorts every row by column, in tiles of
// 2,048 elements: on the n = 40 10a10b workload that cuts the distinct sectors per element
// from 0.99 to about 0.85 and the distinct lines from 0.98 to about 0.69.  Only the order
// inside a row changes: connection lists and values are the same (the reference's
// SparseMatrix rows carry no order beyond the diagonal first, src/solver/sparse_matrix.h).
//
// A CTA takes one row at a time (work counter; the next row is taken early and its first
// tile prefetched into L2 while the current one is sorted) and sorts its elements in tiles
// of kTile, fully by column, with few shared-memory accesses per element (random shared
// accesses bound this pass).  Each thread holds kPer elements in registers.  A 65,536-bin bitmap
// over the tile's column range [jmin, jmax] (bin width 2^s, the smallest that covers the
// range) marks the occupied bins; prefix popcounts give each occupied bin a dense id; one
// shared atomic per element counts its bin and returns its arrival index; the counts are
// scanned into bin starts.  Columns are unique within a row, so an element alone in its bin
// has its final slot (the bin start); the elements of a bin holding several (nearby
// columns, at most 2^s) are ranked by the popcount of a mask of the bin's columns below
// their own (bins of up to 128 columns) or by counting the smaller columns of the bin.  Each element
// is stored once at its final slot and the tile goes back to global memory coalesced.  The
// outcome does not depend on the order of the atomics: every tile ends up in strictly
// increasing column order.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "ctx.h"
#include "kernels.h"

namespace shci {

namespace {

constexpr int kTile = 2048;          // elements per sorted tile
constexpr int kSortWarps = 16;
constexpr int kSortThreads = kSortWarps * 32;
constexpr int kBinWords = 2048;      // 65,536-bin bitmap
constexpr int kPer = kTile / kSortThreads;
static_assert(kBinWords == kTile && kPer * kSortThreads == kTile, "one scan layout for both");

struct SortSmem {
  // aux[0, kBinWords): occupied bins; aux[kBinWords, 2 kBinWords): occupied bins before each
  // bitmap word.  Once every element has its dense bin id, aux holds the column masks of the
  // bins with several elements (or, for bins wider than 128 columns, their columns).
  uint32_t aux[2 * kBinWords];
  uint32_t cnt[kTile];      // per dense bin: count, then start
  uint32_t ocol[kTile];     // the tile in column order
  uint64_t oval[kTile];     // FP64 value, or FP32 value (low word) + FP32 residual (high word)
  uint32_t wsum[kSortWarps], wlo[kSortWarps], whi[kSortWarps];
  uint32_t row, next;
};

enum ScanMode { kScanPack, kScanPopc };

// Block-wide exclusive scan into dst[0, m), m <= kTile (kPer consecutive entries per thread;
// threads past m contribute nothing).  kScanPack: in place (src == dst), keeping each count
// in the low 16 bits (dst[i] = start << 16 | count).  kScanPopc: of the popcounts of src.
template <ScanMode MODE>
__device__ void block_scan(SortSmem& S, const uint32_t* src, uint32_t* dst, int m) {
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int base = threadIdx.x * kPer;
  uint32_t v[kPer], tot = 0;
  if (base < m) {
#pragma unroll
    for (int k = 0; k < kPer; k++) {
      v[k] = base + k < m ? src[base + k] : 0u;
      if (MODE == kScanPopc) v[k] = __popc(v[k]);
      tot += v[k];
    }
  }
  uint32_t inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, inc, o);
    if (lane >= (unsigned)o) inc += t;
  }
  if (lane == 31) S.wsum[warp] = inc;
  __syncthreads();
  // exclusive prefix of the warp totals, by a shuffle scan in every warp
  const uint32_t w0 = lane < static_cast<unsigned>(kSortWarps) ? S.wsum[lane] : 0u;
  uint32_t ws = w0;
#pragma unroll
  for (int o = 1; o < kSortWarps; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, ws, o);
    if (lane >= (unsigned)o) ws += t;
  }
  const uint32_t before = __shfl_sync(kFull, ws - w0, warp);
  if (base < m) {
    uint32_t run = inc - tot + before;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
      if (base + k < m) dst[base + k] = MODE == kScanPack ? (run << 16) | v[k] : run;
      run += v[k];
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

template <bool MIXED>
__global__ void __launch_bounds__(kSortThreads, 2)
    k_sort_rows(const uint64_t* __restrict__ row_ptr, const uint32_t* __restrict__ row_len,
                uint32_t n, uint32_t* col, double* v64, float* v32, float* r32, unsigned* work,
                int mask_max_s) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SortSmem& S = *reinterpret_cast<SortSmem*>(smem_raw);
  const unsigned lane = threadIdx.x & 31;
  if (threadIdx.x == 0) S.row = atomicAdd(work, 1u);
  __syncthreads();
  uint32_t i = S.row;
  while (i < n) {
    // the next row is taken now so that its first tile can be prefetched into L2
    if (threadIdx.x == 0) S.next = atomicAdd(work, 1u);
    __syncthreads();
    const uint32_t nxt = S.next;
    const uint32_t len = row_len[i];
    // rows of one chunk keep their order (it does not matter to H*v)
    for (uint32_t t0 = 0; len > 32 && t0 < len; t0 += kTile) {
      const int L = static_cast<int>(min(static_cast<uint32_t>(kTile), len - t0));
      if (L <= 32) break;
      const uint64_t g = row_ptr[i] + t0;
      for (int t = threadIdx.x; t < L; t += kSortThreads) S.cnt[t] = 0u;
      // all of a thread's loads are issued before any is used
      uint32_t rj[kPer];
      uint64_t rv[kPer];
#pragma unroll
      for (int k = 0; k < kPer; k++) {
        const int p = threadIdx.x + k * kSortThreads;
        if (p < L) {
          rj[k] = col[g + p];
          if (MIXED)
            rv[k] = static_cast<uint64_t>(__float_as_uint(v32[g + p])) |
                    (static_cast<uint64_t>(__float_as_uint(r32[g + p])) << 32);
          else
            rv[k] = static_cast<uint64_t>(__double_as_longlong(v64[g + p]));
        }
      }
      uint64_t nptr = 0;
      uint32_t nlen = 0;
      if (t0 == 0 && nxt < n) {
        nptr = row_ptr[nxt];
        nlen = row_len[nxt];
      }
      uint32_t lo = 0xffffffffu, hi = 0u;
#pragma unroll
      for (int k = 0; k < kPer; k++)
        if (threadIdx.x + k * kSortThreads < L) {
          lo = min(lo, rj[k]);
          hi = max(hi, rj[k]);
        }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(kFull, lo, o));
        hi = max(hi, __shfl_xor_sync(kFull, hi, o));
      }
      if (lane == 0) {
        S.wlo[threadIdx.x >> 5] = lo;
        S.whi[threadIdx.x >> 5] = hi;
      }
      __syncthreads();  // counts cleared, warp ranges written
      lo = lane < static_cast<unsigned>(kSortWarps) ? S.wlo[lane] : 0xffffffffu;
      hi = lane < static_cast<unsigned>(kSortWarps) ? S.whi[lane] : 0u;
      // butterfly over all 32 lanes, so that every lane ends with the block range
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(kFull, lo, o));
        hi = max(hi, __shfl_xor_sync(kFull, hi, o));
      }
      // bin b = (j - jmin) >> s < 65,536; the bitmap covers the bins up to the last one
      const uint32_t jmin = lo;
      const uint32_t wide = (hi - jmin) >> 16;
      const int s = wide ? 32 - __clz(wide) : 0;
      const int W = static_cast<int>(((hi - jmin) >> s) >> 5) + 1;
      for (int t = threadIdx.x; t < W; t += kSortThreads) S.aux[t] = 0u;
      __syncthreads();
#pragma unroll
      for (int k = 0; k < kPer; k++)
        if (threadIdx.x + k * kSortThreads < L) {
          const uint32_t b = (rj[k] - jmin) >> s;
          atomicOr(&S.aux[b >> 5], 1u << (b & 31));
        }
      if (nlen > 32) {
        // first tile of the next row -> L2 (16 elements per thread, within the row)
        const uint32_t e = threadIdx.x * 16u;
        if (e < min(nlen, static_cast<uint32_t>(kTile))) {
          prefetch_l2(col + nptr + e);
          if (MIXED) {
            prefetch_l2(v32 + nptr + e);
            prefetch_l2(r32 + nptr + e);
          } else {
            prefetch_l2(v64 + nptr + e);
          }
        }
      }
      __syncthreads();
      block_scan<kScanPopc>(S, S.aux, S.aux + kBinWords, W);
      const uint32_t nb = S.aux[kBinWords + W - 1] + __popc(S.aux[W - 1]);  // occupied bins
      // dense bin id and arrival index of each element
      uint32_t rd[kPer], ra[kPer];
#pragma unroll
      for (int k = 0; k < kPer; k++)
        if (threadIdx.x + k * kSortThreads < L) {
          const uint32_t b = (rj[k] - jmin) >> s, w = b >> 5;
          rd[k] = S.aux[kBinWords + w] + __popc(S.aux[w] & ((1u << (b & 31)) - 1u));
          ra[k] = atomicAdd(&S.cnt[rd[k]], 1u);
        }
      __syncthreads();
      block_scan<kScanPack>(S, S.cnt, S.cnt, static_cast<int>(nb));  // bin start << 16 | size
      // An element alone in its bin goes to the bin start now.  A bin with several elements
      // spans at most 2^s columns: for s <= 7 its elements set their bits in a 128-bit mask
      // (4 words of aux at 4 * (start / 2), distinct for bins of two or more) and rank by
      // popcount; wider bins list their columns in aux and rank by counting.
      const bool masks = s <= mask_max_s;
      uint32_t multi = 0;  // bit k: element k shares its bin
#pragma unroll
      for (int k = 0; k < kPer; k++)
        if (threadIdx.x + k * kSortThreads < L) {
          const uint32_t e = S.cnt[rd[k]];
          const uint32_t st = e >> 16, m = e & 0xffffu;
          if (m == 1) {
            S.ocol[st] = rj[k];
            S.oval[st] = rv[k];
          } else {
            const uint32_t slot = st + ra[k];
            if (!masks) {
              S.aux[slot] = rj[k];
            } else if (ra[k] == 0) {
              uint32_t* mk = S.aux + 4 * (st >> 1);
              mk[0] = mk[1] = mk[2] = mk[3] = 0u;
            }
            multi |= 1u << k;
            rd[k] = st;
            ra[k] = m | (slot << 16);
          }
        }
      if (nb < static_cast<uint32_t>(L)) {  // some bin holds several elements
        __syncthreads();
        if (masks) {
#pragma unroll
          for (int k = 0; k < kPer; k++)
            if ((multi >> k) & 1u) {
              const uint32_t off = (rj[k] - jmin) & ((1u << s) - 1u);
              atomicOr(&S.aux[4 * (rd[k] >> 1) + (off >> 5)], 1u << (off & 31));
            }
          __syncthreads();
        }
#pragma unroll
        for (int k = 0; k < kPer; k++)
          if ((multi >> k) & 1u) {
            const uint32_t st = rd[k];
            uint32_t rank = 0;
            if (masks) {
              const uint32_t off = (rj[k] - jmin) & ((1u << s) - 1u);
              const uint32_t* mk = S.aux + 4 * (st >> 1);
              for (uint32_t w = 0; w < (off >> 5); w++) rank += __popc(mk[w]);
              rank += __popc(mk[off >> 5] & ((1u << (off & 31)) - 1u));
            } else {
              const uint32_t m = ra[k] & 0xffffu, slot = ra[k] >> 16;
              // smaller columns of the bin (ties, absent for unique columns, by slot)
              for (uint32_t q = st; q < st + m; q++) {
                const uint32_t jq = S.aux[q];
                rank += (jq < rj[k]) | ((jq == rj[k]) & (q < slot));
              }
            }
            S.ocol[st + rank] = rj[k];
            S.oval[st + rank] = rv[k];
          }
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < kPer; k++) {
        const int p = threadIdx.x + k * kSortThreads;
        if (p < L) {
          col[g + p] = S.ocol[p];
          const uint64_t v = S.oval[p];
          if (MIXED) {
            v32[g + p] = __uint_as_float(static_cast<uint32_t>(v));
            r32[g + p] = __uint_as_float(static_cast<uint32_t>(v >> 32));
          } else {
            v64[g + p] = __longlong_as_double(static_cast<long long>(v));
          }
        }
      }
      __syncthreads();
    }
    __syncthreads();  // S.next read by every thread before it is replaced
    i = nxt;
  }
}

}  // namespace

// SHCI_ROW_SORT=0 turns the pass off; SHCI_ROW_SORT=loop ranks every shared bin by counting
// (the path of bins wider than 128 columns, which only tiles spanning more than 2^23 dets
// need), so that tests can exercise it on small systems.
bool row_sort_enabled() {
  const char* e = std::getenv("SHCI_ROW_SORT");
  return !(e && std::strcmp(e, "0") == 0);
}

void sort_rows(shci_ctx* c) {
  auto& H = c->H;
  const uint32_t n = static_cast<uint32_t>(H.n);
  if (n == 0 || H.nnz_current == 0) return;
  cudaStream_t s = c->stream;
  int dev_sms = 0, per_sm = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device));
  const size_t smem = sizeof(SortSmem);
  const bool mixed = H.precision != SHCI_PREC_FP64;
  if (mixed) {
    SHCI_CUDA(cudaFuncSetAttribute(k_sort_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
    SHCI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sort_rows<true>,
                                                            kSortThreads, smem));
  } else {
    SHCI_CUDA(cudaFuncSetAttribute(k_sort_rows<false>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
    SHCI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sort_rows<false>,
                                                            kSortThreads, smem));
  }
  const unsigned grid = static_cast<unsigned>(dev_sms) * static_cast<unsigned>(std::max(1, per_sm));
  c->err_word.resize(8);
  unsigned* work = c->err_word.p;
  SHCI_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned), s));
  const char* e = std::getenv("SHCI_ROW_SORT");
  const int mask_max_s = e && std::strcmp(e, "loop") == 0 ? -1 : 7;  // 128-bit column masks
  ProfScope ps(c->prof, s, "hbuild_rowsort");
  if (mixed)
    k_sort_rows<true><<<grid, kSortThreads, smem, s>>>(H.row_ptr.p, H.row_cnt.p, n, H.col.p,
                                                       nullptr, H.val32.p, H.res32.p, work,
                                                       mask_max_s);
  else
    k_sort_rows<false><<<grid, kSortThreads, smem, s>>>(H.row_ptr.p, H.row_cnt.p, n, H.col.p,
                                                        H.val64.p, nullptr, nullptr, work,
                                                        mask_max_s);
  SHCI_LAUNCH_CHECK();
  c->launches += 1;
}

}  // namespace shci

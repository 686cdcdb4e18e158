// Device-wide exclusive scan and stable LSD radix sort.
//
// Radix sort: 8-bit digits, one pass per digit over [begin_bit, end_bit).  Each pass is
//   (1) per-tile digit histograms (shared atomics),
//   (2) an exclusive scan of the digit-major [256 x tiles] histogram -> scatter bases,
//   (3) a stable scatter of each 4096-item tile: every warp holds 512 consecutive items in
//       registers, counts their digits, and after one scan over (digit, warp) places them
//       chunk by chunk (ranks of equal digits from ballots) into a digit-sorted copy of the
//       tile in shared memory, written out run by run so global writes are coalesced.
// Passes whose digit is constant over all keys are skipped (a pre-pass ORs key differences).
// Keys are 32 or 64 bit, values 32 or 64 bit.
#include "sort.cuh"

namespace shci {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ __forceinline__ T warp_inclusive(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive prefix and
// writes the block total to *total.
template <class T>
__device__ __forceinline__ T block_exclusive(T v, T* total) {
  __shared__ T s_w[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const T inc = warp_inclusive(v);
  if (lane == 31) s_w[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = lane < kScanThreads / 32 ? s_w[lane] : T(0);
    w = warp_inclusive(w);
    if (lane < kScanThreads / 32) s_w[lane] = w;
  }
  __syncthreads();
  const T before = warp ? s_w[warp - 1] : T(0);
  *total = s_w[kScanThreads / 32 - 1];
  __syncthreads();
  return before + inc - v;
}

template <class T>
__global__ void k_tile_sums(const T* in, size_t n, T* sums) {
  const size_t base = (size_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  T acc = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    if (base + k < n) acc += in[base + k];
  T tot;
  block_exclusive(acc, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <class T>
__global__ void k_tile_scan(const T* in, T* out, size_t n, const T* offsets, T* total_dev) {
  const size_t base = (size_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  T items[kScanItems];
  T acc = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    items[k] = base + k < n ? in[base + k] : T(0);
    acc += items[k];
  }
  T tot;
  T pre = block_exclusive(acc, &tot);
  if (offsets) pre += offsets[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) {
      out[base + k] = pre;
      if (total_dev && base + k == n - 1) *total_dev = pre + items[k];
    }
    pre += items[k];
  }
}

template <class T>
void scan_rec(const T* in, T* out, size_t n, cudaStream_t s, T* part, T* total_dev) {
  const size_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb <= 1) {
    k_tile_scan<T><<<1, kScanThreads, 0, s>>>(in, out, n, nullptr, total_dev);
    SHCI_LAUNCH_CHECK();
    return;
  }
  k_tile_sums<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, part);
  SHCI_LAUNCH_CHECK();
  scan_rec<T>(part, part, nb, s, part + nb, nullptr);
  k_tile_scan<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, part, total_dev);
  SHCI_LAUNCH_CHECK();
}

size_t scan_part_size(size_t n) {
  size_t tot = 2, m = n;
  while (m > (size_t)kScanTile) {
    m = (m + kScanTile - 1) / kScanTile;
    tot += m;
  }
  return tot + 1;
}

// ------------------------------------------------------------------------- radix sort
constexpr int kSortThreads = 256;
constexpr int kSortRounds = 16;
constexpr int kSortTile = kSortThreads * kSortRounds;

template <class K>
__global__ void k_radix_hist(const K* keys, size_t n, int shift, uint32_t* hist,
                             unsigned n_tiles) {
  __shared__ uint32_t s_h[256];
  s_h[threadIdx.x] = 0;
  const size_t t0 = (size_t)blockIdx.x * kSortTile;
  // every load of the thread is issued before the first count
  unsigned d[kSortRounds];
#pragma unroll
  for (int r = 0; r < kSortRounds; r++) {
    const size_t idx = t0 + (size_t)r * kSortThreads + threadIdx.x;
    d[r] = idx < n ? (unsigned)((keys[idx] >> shift) & 255u) : 256u;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kSortRounds; r++)
    if (d[r] < 256u) atomicAdd(&s_h[d[r]], 1u);
  __syncthreads();
  hist[(size_t)threadIdx.x * n_tiles + blockIdx.x] = s_h[threadIdx.x];
}

// Lanes of the warp holding the same 8-bit digit as this lane (valid lanes only): one ballot
// per digit bit, which GB300 issues at about twice the rate of __match_any_sync.
__device__ __forceinline__ unsigned radix_peers(unsigned d, bool valid) {
  unsigned m = __ballot_sync(0xffffffffu, valid);
#pragma unroll
  for (int b = 0; b < 8; b++) {
    const bool bit = (d >> b) & 1u;
    const unsigned bb = __ballot_sync(0xffffffffu, valid && bit);
    m &= bit ? bb : ~bb;
  }
  return m;
}

// Stable scatter of one tile.  Warp w owns the tile's items [512 w, 512 w + 512) and holds
// them in registers (16 chunks of 32 consecutive items).  Each warp counts its digits into
// its own shared counters; one scan over (digit, warp) turns the counts into offsets, so
// warp w's items of digit d follow those of lower warps; the warp then places its chunks in
// order, ranking equal digits of a chunk with ballots, into a digit-sorted copy of the tile
// in shared memory, which goes to global memory run by run (coalesced) at the digit's
// global offset.  offs is the exclusively scanned digit-major histogram with the total
// appended, so the tile's count of digit d is offs[d * n_tiles + tile + 1] - offs[d *
// n_tiles + tile].
// Three CTAs per SM (an 80-register cap) for items of up to 12 bytes: 4.5 against 5.5 ms for
// a pass over 851M u32 pairs; 16-byte items keep two (the cap made them slower).
template <class K, class V>
__global__ void __launch_bounds__(kSortThreads, sizeof(K) + sizeof(V) > 12 ? 2 : 3)
    k_radix_scatter(const K* __restrict__ kin, const V* __restrict__ vin, K* __restrict__ kout,
                    V* __restrict__ vout, size_t n, int shift, const uint32_t* __restrict__ offs,
                    unsigned n_tiles) {
  constexpr int kW = kSortThreads / 32;
  constexpr int kC = kSortTile / kSortThreads;  // chunks of 32 items per warp
  extern __shared__ __align__(16) unsigned char s_raw[];
  K* s_k = reinterpret_cast<K*>(s_raw);
  V* s_v = reinterpret_cast<V*>(s_raw + sizeof(K) * kSortTile);
  __shared__ uint32_t s_wc[kW][256];
  __shared__ uint32_t s_gbase[256], s_lstart[256], s_ws[kW];
  const unsigned tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const unsigned lt = (1u << lane) - 1u;
  const size_t t0 = (size_t)blockIdx.x * kSortTile;
  const size_t hi = (size_t)tid * n_tiles + blockIdx.x;
  const uint32_t g0 = offs[hi];
  const uint32_t tcnt = offs[hi + 1] - g0;
  s_gbase[tid] = g0;
#pragma unroll
  for (int w = 0; w < kW; w++) s_wc[w][tid] = 0;
  K kk[kC];
  V vv[kC];
  const size_t wb = t0 + (size_t)warp * 32 * kC + lane;
#pragma unroll
  for (int c = 0; c < kC; c++) {
    const size_t idx = wb + (size_t)c * 32;
    kk[c] = idx < n ? kin[idx] : K(0);
    vv[c] = idx < n ? vin[idx] : V(0);
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < kC; c++)
    if (wb + (size_t)c * 32 < n) atomicAdd(&s_wc[warp][(unsigned)((kk[c] >> shift) & 255u)], 1u);
  __syncthreads();
  {
    // digit d = tid: its start in the tile (exclusive scan of the tile's counts), then the
    // start of each warp's items of d
    uint32_t inc = tcnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= (unsigned)o) inc += t;
    }
    if (lane == 31) s_ws[warp] = inc;
    __syncthreads();
    uint32_t run = inc - tcnt;
    for (unsigned w = 0; w < warp; w++) run += s_ws[w];
    s_lstart[tid] = run;
#pragma unroll
    for (int w = 0; w < kW; w++) {
      const uint32_t c = s_wc[w][tid];
      s_wc[w][tid] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < kC; c++) {
    const bool valid = wb + (size_t)c * 32 < n;
    const unsigned d = valid ? (unsigned)((kk[c] >> shift) & 255u) : 0u;
    const unsigned pm = radix_peers(d, valid);
    uint32_t off = 0;
    if (valid) off = s_wc[warp][d];
    __syncwarp();
    if (valid) {
      const uint32_t pos = off + __popc(pm & lt);
      s_k[pos] = kk[c];
      s_v[pos] = vv[c];
      if ((pm & lt) == 0) s_wc[warp][d] = off + __popc(pm);
    }
    __syncwarp();
  }
  __syncthreads();
  const unsigned tile_n = static_cast<unsigned>(n - t0 < (size_t)kSortTile ? n - t0 : kSortTile);
  for (unsigned p = tid; p < tile_n; p += kSortThreads) {
    const K k = s_k[p];
    const unsigned d = (unsigned)((k >> shift) & 255u);
    const size_t g = (size_t)s_gbase[d] + (p - s_lstart[d]);
    kout[g] = k;
    vout[g] = s_v[p];
  }
}

// Bits set in the OR of (k xor k0) over all keys: digits where every key agrees are skipped.
template <class K>
__global__ void k_key_spread(const K* keys, size_t n, unsigned long long* spread) {
  const K k0 = keys[0];
  uint64_t acc = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    acc |= keys[i] ^ k0;
  for (int o = 16; o; o >>= 1) acc |= __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicOr(spread, (unsigned long long)acc);
}

template <class K, class V>
void radix_sort_impl(DevBuf<K>& keys, DevBuf<V>& vals, size_t n, int begin_bit, int end_bit,
                     cudaStream_t s, SortScratch& sc, DevBuf<K>& kalt, DevBuf<V>& valt) {
  if (n <= 1 || begin_bit >= end_bit) return;
  if (n >= 0xffffffffull) throw ArgError("radix sort: 2^32 or more items");
  end_bit = end_bit > (int)(8 * sizeof(K)) ? (int)(8 * sizeof(K)) : end_bit;
  // Which digits vary at all?
  sc.part64.reserve(scan_part_size(1));
  unsigned long long* spread = reinterpret_cast<unsigned long long*>(sc.part64.p);
  SHCI_CUDA(cudaMemsetAsync(spread, 0, sizeof(unsigned long long), s));
  k_key_spread<K><<<grid_for(n, 256, 152 * 8), 256, 0, s>>>(keys.p, n, spread);
  SHCI_LAUNCH_CHECK();
  unsigned long long sp = 0;
  SHCI_CUDA(cudaMemcpyAsync(&sp, spread, sizeof(sp), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));

  const unsigned n_tiles = static_cast<unsigned>((n + kSortTile - 1) / kSortTile);
  const size_t n_hist = (size_t)256 * n_tiles;
  kalt.reserve(n, 1.25);
  valt.reserve(n, 1.25);
  sc.hist.reserve(n_hist + 1, 1.25);
  sc.part32.reserve(scan_part_size(n_hist), 1.25);
  const int smem = static_cast<int>((sizeof(K) + sizeof(V)) * kSortTile);
  SHCI_CUDA(cudaFuncSetAttribute(k_radix_scatter<K, V>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  K* kin = keys.p;
  V* vin = vals.p;
  K* kout = kalt.p;
  V* vout = valt.p;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    const uint64_t mask = (shift + 8 >= 64 ? ~0ull : ((1ull << (shift + 8)) - 1ull)) &
                          ~((1ull << shift) - 1ull);
    if ((sp & mask) == 0) continue;
    k_radix_hist<K><<<n_tiles, kSortThreads, 0, s>>>(kin, n, shift, sc.hist.p, n_tiles);
    SHCI_LAUNCH_CHECK();
    scan_rec<uint32_t>(sc.hist.p, sc.hist.p, n_hist, s, sc.part32.p, sc.hist.p + n_hist);
    k_radix_scatter<K, V><<<n_tiles, kSortThreads, smem, s>>>(kin, vin, kout, vout, n, shift,
                                                               sc.hist.p, n_tiles);
    SHCI_LAUNCH_CHECK();
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (kin != keys.p) {
    // the result lives in the ping-pong buffers: hand their storage to the caller
    const size_t kn = keys.n, vn = vals.n;
    swap_storage(keys, kalt);
    swap_storage(vals, valt);
    keys.n = kn;
    vals.n = vn;
  }
}

__global__ void k_iota(uint32_t* v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    v[i] = static_cast<uint32_t>(i);
}

__global__ void k_gather_u64(const uint64_t* src, const uint32_t* idx, uint64_t* out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = src[idx[i]];
}

}  // namespace

uint64_t exclusive_scan_u64(const uint64_t* in, uint64_t* out, size_t n, cudaStream_t s,
                            SortScratch& sc) {
  if (n == 0) return 0;
  sc.part64.reserve(scan_part_size(n) + 1, 1.25);
  uint64_t* total_dev = sc.part64.p + scan_part_size(n);
  scan_rec<uint64_t>(in, out, n, s, sc.part64.p, total_dev);
  uint64_t tot = 0;
  SHCI_CUDA(cudaMemcpyAsync(&tot, total_dev, sizeof(tot), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  return tot;
}

void exclusive_scan_u64_async(const uint64_t* in, uint64_t* out, size_t n, cudaStream_t s,
                              SortScratch& sc, uint64_t* total_dev) {
  if (n == 0) return;
  sc.part64.reserve(scan_part_size(n) + 1, 1.25);
  scan_rec<uint64_t>(in, out, n, s, sc.part64.p, total_dev);
}

uint32_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s,
                            SortScratch& sc) {
  if (n == 0) return 0;
  sc.part32.reserve(scan_part_size(n) + 1, 1.25);
  uint32_t* total_dev = sc.part32.p + scan_part_size(n);
  scan_rec<uint32_t>(in, out, n, s, sc.part32.p, total_dev);
  uint32_t tot = 0;
  SHCI_CUDA(cudaMemcpyAsync(&tot, total_dev, sizeof(tot), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  return tot;
}

void radix_sort_pairs(DevBuf<uint64_t>& keys, DevBuf<uint32_t>& vals, size_t n, int begin_bit,
                      int end_bit, cudaStream_t s, SortScratch& sc) {
  radix_sort_impl<uint64_t, uint32_t>(keys, vals, n, begin_bit, end_bit, s, sc, sc.kalt,
                                      sc.valt32);
}

void radix_sort_pairs64(DevBuf<uint64_t>& keys, DevBuf<uint64_t>& vals, size_t n,
                        int begin_bit, int end_bit, cudaStream_t s, SortScratch& sc) {
  radix_sort_impl<uint64_t, uint64_t>(keys, vals, n, begin_bit, end_bit, s, sc, sc.kalt,
                                      sc.valt64);
}

void radix_sort_pairs32(DevBuf<uint32_t>& keys, DevBuf<uint32_t>& vals, size_t n,
                        int begin_bit, int end_bit, cudaStream_t s, SortScratch& sc) {
  radix_sort_impl<uint32_t, uint32_t>(keys, vals, n, begin_bit, end_bit, s, sc, sc.kalt32,
                                      sc.valt32);
}

void iota_u32(uint32_t* v, size_t n, cudaStream_t s) {
  k_iota<<<grid_for(n, 256), 256, 0, s>>>(v, n);
  SHCI_LAUNCH_CHECK();
}

void gather_u64(const uint64_t* src, const uint32_t* idx, uint64_t* out, size_t n,
                cudaStream_t s) {
  k_gather_u64<<<grid_for(n, 256), 256, 0, s>>>(src, idx, out, n);
  SHCI_LAUNCH_CHECK();
}

}  // namespace shci

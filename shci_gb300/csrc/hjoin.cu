// Hamiltonian build by a two-hole core join.
//
// Two determinants with the same electron counts are connected by at most a double
// excitation exactly when they share an (n_e - 2)-electron "core": the det with some pair of
// its electrons removed.  Every det contributes K = C(n_e, 2) entries, one per electron pair
// (alpha-alpha, beta-beta or alpha-beta), keyed by a hash of its core.  After a stable sort by
// key, each bucket of equal keys holds, in det-id order, dets that share a core (plus, rarely,
// dets whose different cores hash alike).  Row i then examines, for each of its K entries,
// only the members after its own entry in that bucket: exactly the dets j > i sharing that
// core.  This finds the same element set as the group scan of the reference's
// Hamiltonian<S>::update_matrix (src/solver/hamiltonian.h:415-598: same-alpha, same-beta and
// alpha-single x beta-single partners) while examining about 1.4 candidates per stored
// element instead of tens.
//
// A pair (i, j) shares one core if it is a double excitation and n_e - 1 cores if it is a
// single; it is taken only from its canonical core: the two electrons of i absent from j
// (double), or the electron of i absent from j plus the lowest electron the two share, alpha
// orbitals before beta ones (single).  The test uses the actual spin strings, so a hash
// collision can only add candidates that fail it; the one collision that could repeat a
// column (two cores of j in one bucket, adjacent by construction) is skipped explicitly.
//
// Used when n_e >= 2, n * K < 2^32 and the index fits in memory; otherwise the scan path
// (hbuild.cu) builds the matrix.
#include <algorithm>
#include <cstdlib>
#include <vector>

#include "ctx.h"
#include "heatbath.cuh"
#include "hrow.cuh"
#include "kernels.h"

namespace shci {

namespace {

constexpr int kJoinWarps = 8;

__device__ __forceinline__ uint64_t core_hash(uint64_t cu, uint64_t cd) {
  uint64_t h = cu * 0x9E3779B97F4A7C15ull ^ (cd + 0x632BE59BD9B4E019ull) * 0xC2B2AE3D27D4EB4Full;
  h ^= h >> 29;
  h *= 0xBF58476D1CE4E5B9ull;
  h ^= h >> 32;
  return h;
}

// Removed-electron masks (alpha, beta) of pair entry k of det (u, d).
__device__ __forceinline__ void pair_masks(uint32_t pr, uint64_t u, uint64_t d, int n_up,
                                           uint64_t* ru, uint64_t* rd) {
  const int r1 = static_cast<int>(pr & 0xffffu), r2 = static_cast<int>(pr >> 16);
  uint64_t a = 0, b = 0;
  if (r1 < n_up) a |= 1ull << nth_bit(u, r1);
  else b |= 1ull << nth_bit(d, r1 - n_up);
  if (r2 < n_up) a |= 1ull << nth_bit(u, r2);
  else b |= 1ull << nth_bit(d, r2 - n_up);
  *ru = a;
  *rd = b;
}

// Entries in det order: key = top `bits` bits of the core hash, value = entry index.
template <class KT>
__global__ void k_core_keys(const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn,
                            uint32_t n, const uint32_t* __restrict__ pairs, uint32_t K, int n_up,
                            int n_dn, int bits, KT* keys, uint32_t* vals, unsigned* err) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = warp0; i < n; i += n_warps) {
    const uint64_t u = up[i], d = dn[i];
    if (popc64(u) != n_up || popc64(d) != n_dn) {
      if (lane == 0) atomicOr(err, (unsigned)kDevCheck);
      continue;
    }
    for (uint32_t k = lane; k < K; k += 32) {
      uint64_t ru, rd;
      pair_masks(pairs[k], u, d, n_up, &ru, &rd);
      const size_t t = (size_t)i * K + k;
      keys[t] = static_cast<KT>(core_hash(u & ~ru, d & ~rd) >> (64 - bits));
      vals[t] = static_cast<uint32_t>(t);
    }
  }
}

// After the sort, buckets in three parallel steps: flag bucket starts, scan the flags
// (bucket index of every position), record each bucket's start; then every position p of
// bucket b writes span[entry] = p | end(b) << 32 and jdet[p] = det id (over the entry index).
template <class KT>
__device__ __forceinline__ uint32_t bucket_head(const KT* keys, size_t p) {
  return (p == 0 || keys[p] != keys[p - 1]) ? 1u : 0u;
}

template <class KT>
__global__ void k_bucket_flags(const KT* __restrict__ keys, size_t m, uint32_t* flags) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < m;
       p += (size_t)gridDim.x * blockDim.x)
    flags[p] = bucket_head(keys, p);
}

template <class KT>
__global__ void k_bucket_starts(const KT* __restrict__ keys, const uint32_t* __restrict__ scan,
                                size_t m, uint32_t n_buckets, uint32_t* bstart) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < m;
       p += (size_t)gridDim.x * blockDim.x)
    if (bucket_head(keys, p)) bstart[scan[p]] = static_cast<uint32_t>(p);
  if (blockIdx.x == 0 && threadIdx.x == 0) bstart[n_buckets] = static_cast<uint32_t>(m);
}

template <class KT>
__global__ void k_bucket_spans(const KT* __restrict__ keys, const uint32_t* __restrict__ scan,
                               const uint32_t* __restrict__ bstart, uint32_t* vals, size_t m,
                               uint32_t K, uint64_t* span) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < m;
       p += (size_t)gridDim.x * blockDim.x) {
    const uint32_t b = scan[p] + bucket_head(keys, p) - 1u;
    const uint32_t v = vals[p];
    span[v] = static_cast<uint64_t>(p) | (static_cast<uint64_t>(bstart[b + 1]) << 32);
    vals[p] = v / K;
  }
}

}  // namespace

namespace {

struct JoinView {
  uint32_t K;
  int n_up;
  const uint32_t* pairs;
  const uint64_t* span;
  const uint32_t* jdet;
  uint32_t n_prev;  // incremental update: rows < n_prev take only members >= n_prev
};

// Members of entry sp = (position p | bucket end << 32) of row i: positions (p', end) with
// p' = p, or, for a row built before (i < n_prev), the last position whose det precedes
// n_prev (a bucket lists its dets in increasing id order, so the members >= n_prev follow).
__device__ __forceinline__ uint32_t member_start(const uint32_t* __restrict__ jdet, uint64_t sp,
                                                 uint32_t i, uint32_t n_prev) {
  uint32_t p = static_cast<uint32_t>(sp);
  if (i < n_prev) {
    uint32_t lo = p + 1u, hi = static_cast<uint32_t>(sp >> 32);
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (jdet[mid] < n_prev) lo = mid + 1u;
      else hi = mid;
    }
    p = lo - 1u;
  }
  return p;
}

// Row kernel of the join (MODE as in RowSink).  A warp per row: lanes take the row's entries
// 32 at a time, the members after each entry are flattened over the lanes, and every member
// that passes the canonical-core test goes to the row's queues.
// Five CTAs per SM (48 registers, a few spilled): 144 ms for the n = 40 fill against 151 ms
// at the register-limited four (64 registers) and 156 ms at six (40 registers).
template <int MODE>
__global__ void __launch_bounds__(kJoinWarps * 32, 5)
    k_hjoin(DevIntegrals I, const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn,
            uint32_t n, JoinView jv, uint32_t* row_cnt, const uint64_t* row_ptr, uint32_t* col,
            double* v64, float* v32, float* r32, unsigned* work, float* absacc) {
  __shared__ RowQueues qs[kJoinWarps];
  RowQueues& q = qs[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31;
  const uint32_t K = jv.K;
  while (true) {
    uint32_t i = 0;
    if (lane == 0) i = atomicAdd(work, 1u);
    i = __shfl_sync(kFull, i, 0);
    if (i >= n) break;
    const uint64_t ui = up[i], di = dn[i];
    RowSink<MODE> sink(q, I, ui, di, MODE ? row_ptr[i] : 0, col, v64, v32, r32);
    if (absacc) sink.track_abs(absacc, i);
    uint64_t n_cand = 0;
    for (uint32_t k0 = 0; k0 < K; k0 += 32) {
      const uint32_t k = k0 + lane;
      uint32_t p = 0, len = 0;
      uint64_t ru = 0, rd = 0;
      if (k < K) {
        const uint64_t sp = jv.span[(size_t)i * K + k];
        p = member_start(jv.jdet, sp, i, jv.n_prev);
        len = static_cast<uint32_t>(sp >> 32) - p - 1u;
        pair_masks(jv.pairs[k], ui, di, jv.n_up, &ru, &rd);
      }
      const uint32_t inc = warp_inclusive_u32(len);
      const uint32_t total = __shfl_sync(kFull, inc, 31);
      n_cand += total;
      for (uint32_t t0 = 0; t0 < total; t0 += 32) {
        const uint32_t t = t0 + lane;
        const uint32_t o = owner_lane(inc, t);
        const uint32_t o_inc = __shfl_sync(kFull, inc, o);
        const uint32_t o_len = __shfl_sync(kFull, len, o);
        const uint32_t o_p = __shfl_sync(kFull, p, o);
        const uint64_t o_ru = __shfl_sync(kFull, ru, o);
        const uint64_t o_rd = __shfl_sync(kFull, rd, o);
        bool cand = false, single = false;
        uint32_t j = 0;
        uint64_t uj = 0, dj = 0;
        if (t < total) {
          const uint32_t pos = o_p + 1u + (t - (o_inc - o_len));
          j = jv.jdet[pos];
          // a second entry of j in this bucket (its two cores hashed alike) sits right after
          // the first; take j once
          const bool repeat = pos > o_p + 1u && jv.jdet[pos - 1u] == j;
          if (!repeat) {
            uj = up[j];
            dj = dn[j];
            const uint64_t xu = ui ^ uj, xd = di ^ dj;
            const int x2 = popc64(xu) + popc64(xd);
            const uint64_t iu = ui & xu, id = di & xd;  // electrons of i absent from j
            if (x2 == 4) {
              cand = o_ru == iu && o_rd == id;
            } else if (x2 == 2) {
              const uint64_t cu = ui & uj, cd = di & dj;
              const uint64_t lu = cu & (~cu + 1ull);
              const uint64_t ld = cu ? 0ull : (cd & (~cd + 1ull));
              cand = o_ru == (iu | lu) && o_rd == (id | ld);
              single = true;
            }
          }
        }
        sink.push(cand, single, j, uj, dj);
      }
    }
    const uint32_t cnt = sink.finish();
    if (lane == 0) {
      if (row_cnt) row_cnt[i] = cnt;
      atomicAdd(reinterpret_cast<unsigned long long*>(work + 2), (unsigned long long)n_cand);
    }
  }
}

// Row capacity of a single-pass build: the candidates of row i (members after each of its
// entries), an upper bound on the elements it keeps.
__global__ void k_join_caps(const uint64_t* __restrict__ span, const uint32_t* __restrict__ jdet,
                            uint32_t n, uint32_t K, uint32_t n_prev, uint64_t* caps) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    uint64_t c = 0;
    for (uint32_t k = lane; k < K; k += 32) {
      const uint64_t sp = span[(size_t)i * K + k];
      c += static_cast<uint32_t>(sp >> 32) - member_start(jdet, sp, i, n_prev) - 1u;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
    if (lane == 0) caps[i] = c;
  }
}

void release_sort_pingpong(shci_ctx* c) {
  c->sort.kalt.release();
  c->sort.kalt32.release();
  c->sort.valt32.release();
  c->sort.valt64.release();
}

void sort_keys(DevBuf<uint32_t>& k, DevBuf<uint32_t>& v, size_t m, int bits, shci_ctx* c) {
  radix_sort_pairs32(k, v, m, 0, bits, c->stream, c->sort);
}
void sort_keys(DevBuf<uint64_t>& k, DevBuf<uint32_t>& v, size_t m, int bits, shci_ctx* c) {
  radix_sort_pairs(k, v, m, 0, bits, c->stream, c->sort);
}

// Entries -> sorted buckets -> spans; keys of type KT hold `bits` hash bits.
template <class KT>
void join_index(shci_ctx* c, DevBuf<KT>& keys, int bits, size_t n, int n_up, int n_dn) {
  auto& J = c->join;
  cudaStream_t s = c->stream;
  const size_t m = J.m;
  keys.resize(m);
  J.jdet.resize(m);
  c->err_word.resize(8);
  {
    ProfScope ps(c->prof, s, "join_keys");
    SHCI_CUDA(cudaMemsetAsync(c->err_word.p, 0, 4, s));
    k_core_keys<KT><<<grid_for(n * 32, 256), 256, 0, s>>>(
        c->d_up.p, c->d_dn.p, static_cast<uint32_t>(n), J.pairs.p, J.K, n_up, n_dn, bits,
        keys.p, J.jdet.p, c->err_word.p);
    SHCI_LAUNCH_CHECK();
  }
  unsigned err = 0;
  SHCI_CUDA(cudaMemcpyAsync(&err, c->err_word.p, 4, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  if (err) throw ArgError("dets do not all have the electron counts of the first det");
  {
    ProfScope ps(c->prof, s, "join_sort");
    sort_keys(keys, J.jdet, m, bits, c);
  }
  // the sort's ping-pong storage is not needed again for this build
  release_sort_pingpong(c);
  J.span.resize(m);
  J.scan.resize(m + 1);
  {
    ProfScope ps(c->prof, s, "join_buckets");
    k_bucket_flags<KT><<<grid_for(m, 256), 256, 0, s>>>(keys.p, m, J.scan.p);
    SHCI_LAUNCH_CHECK();
    const uint32_t nb = exclusive_scan_u32(J.scan.p, J.scan.p, m, s, c->sort);
    J.bstart.resize((size_t)nb + 1);
    k_bucket_starts<KT><<<grid_for(m, 256), 256, 0, s>>>(keys.p, J.scan.p, m, nb, J.bstart.p);
    SHCI_LAUNCH_CHECK();
    k_bucket_spans<KT><<<grid_for(m, 256), 256, 0, s>>>(keys.p, J.scan.p, J.bstart.p, J.jdet.p,
                                                          m, J.K, J.span.p);
    SHCI_LAUNCH_CHECK();
  }
  SHCI_CUDA(cudaStreamSynchronize(s));
  keys.release();
  J.scan.release();
  J.bstart.release();
  J.key_bytes = sizeof(KT);
  J.bits = bits;
  c->launches += 12;
}

}  // namespace

bool join_prepare(shci_ctx* c) {
  auto& J = c->join;
  const size_t n = c->up.size();
  cudaStream_t s = c->stream;
  if (n == 0) return false;
  const int n_up = __builtin_popcountll(c->up[0]), n_dn = __builtin_popcountll(c->dn[0]);
  const int ne = n_up + n_dn;
  if (ne < 2 || ne > 128) return false;
  const uint64_t K = static_cast<uint64_t>(ne) * (ne - 1) / 2;
  const uint64_t m = n * K;
  if (m >= 0xffffffffull) return false;
  // memory: keys + sort ping-pong (16 B), entry values + ping-pong (8 B), then span (8 B)
  size_t free_b = 0, total_b = 0;
  SHCI_CUDA(cudaMemGetInfo(&free_b, &total_b));
  size_t avail = free_b + c->mem.cached;  // cached blocks return to the driver on demand
  const size_t live = c->mem.live();
  if (c->mem.budget) avail = std::min(avail, c->mem.budget > live ? c->mem.budget - live : 0);
  if (static_cast<double>(m) * 26.0 > 0.85 * static_cast<double>(avail)) return false;
  J.K = static_cast<uint32_t>(K);
  J.n_up = n_up;
  J.n_dn = n_dn;
  J.m = m;
  try {
    std::vector<uint32_t> pr;
    pr.reserve(K);
    for (int r1 = 0; r1 < ne; r1++)
      for (int r2 = r1 + 1; r2 < ne; r2++) pr.push_back(static_cast<uint32_t>(r1 | (r2 << 16)));
    J.pairs.resize(K);
    SHCI_CUDA(cudaMemcpyAsync(J.pairs.p, pr.data(), K * 4, cudaMemcpyHostToDevice, s));
    // hash bits: 32 while the entries are few enough that merged buckets stay rare.
    // SHCI_JOIN_BITS (4..40) narrows it, so tests can force colliding buckets.
    int bits = m <= (1ull << 30) ? 32 : 40;
    if (const char* e = std::getenv("SHCI_JOIN_BITS")) bits = std::min(40, std::max(4, std::atoi(e)));
    if (bits <= 32) join_index(c, J.keys32, bits, n, n_up, n_dn);
    else join_index(c, J.keys, bits, n, n_up, n_dn);
  } catch (const OomError&) {
    join_release(c);
    release_sort_pingpong(c);
    return false;
  }
  return true;
}

void join_rows(shci_ctx* c, int mode, uint32_t* row_cnt, const uint64_t* row_ptr,
               uint32_t* col, double* v64, float* v32, float* r32, unsigned* work,
               unsigned grid, float* absacc, uint32_t n_prev) {
  const auto& J = c->join;
  const uint32_t n = static_cast<uint32_t>(c->up.size());
  JoinView v{J.K, J.n_up, J.pairs.p, J.span.p, J.jdet.p, n_prev};
  cudaStream_t s = c->stream;
  if (mode == 0)
    k_hjoin<0><<<grid, kJoinWarps * 32, 0, s>>>(c->dI, c->d_up.p, c->d_dn.p, n, v, row_cnt,
                                                 nullptr, nullptr, nullptr, nullptr, nullptr,
                                                 work, absacc);
  else if (mode == 1)
    k_hjoin<1><<<grid, kJoinWarps * 32, 0, s>>>(c->dI, c->d_up.p, c->d_dn.p, n, v, row_cnt,
                                                 row_ptr, col, v64, nullptr, nullptr, work,
                                                 absacc);
  else
    k_hjoin<2><<<grid, kJoinWarps * 32, 0, s>>>(c->dI, c->d_up.p, c->d_dn.p, n, v, row_cnt,
                                                 row_ptr, col, nullptr, v32, r32, work,
                                                 absacc);
  SHCI_LAUNCH_CHECK();
  c->launches += 1;
}

uint64_t join_row_caps(shci_ctx* c, uint64_t* row_start, uint32_t n_prev) {
  const auto& J = c->join;
  const uint32_t n = static_cast<uint32_t>(c->up.size());
  cudaStream_t s = c->stream;
  k_join_caps<<<grid_for((size_t)n * 32, 256), 256, 0, s>>>(J.span.p, J.jdet.p, n, J.K, n_prev,
                                                           row_start);
  SHCI_LAUNCH_CHECK();
  const uint64_t tot = exclusive_scan_u64(row_start, row_start, n, s, c->sort);
  SHCI_CUDA(cudaMemcpyAsync(row_start + n, &tot, 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 1;
  return tot;
}

void join_release(shci_ctx* c) {
  auto& J = c->join;
  J.keys.release();
  J.keys32.release();
  J.scan.release();
  J.bstart.release();
  J.jdet.release();
  J.span.release();
  J.m = 0;
}

}  // namespace shci

// Determinant index (K1/K2) and Hamiltonian build (K3).
//
// Replaces Hamiltonian<S>::update_abdet / update_abm1 / update_absingles / update_matrix
// (src/solver/hamiltonian.h:157-598).  The reference keeps hash maps from alpha / beta
// strings to det lists and intersects alpha-single lists with beta-single lists per row.
// Here the det list is radix-sorted on the device into:
//   alpha groups ordered by beta string (am_*): dets sharing an alpha string;
//   alpha groups and beta groups ordered by det id (ad_*, bd_*);
// and each unique alpha (beta) string gets the list of unique alphas (betas) one single
// excitation away, found by binary search of its n_e * (n - n_e) single excitations in the
// sorted unique strings (this replaces the alpha-minus-one hash map).  A warp builds a row:
//   (a) same beta string, any alpha  (hamiltonian.h:430-442): scan the beta group from the
//       first det id > i (the group is in det-id order, so the lower triangle is skipped);
//   (b) same alpha string, any beta  (:456-468): the same over the alpha group;
//   (c) alpha single x beta single   (:482-532): for each alpha single a' of the row, either
//       scan a''s group keeping members whose beta differs by one electron, or - when the
//       group is larger than a few times the row's beta-single list - binary-search each
//       beta single of the row in a''s group (ordered by beta string), whichever is cheaper;
// keeping j > i (strict upper triangle) and |H_ij| >= 1e-12 (:440).  The result is the
// element set the reference builds (its incremental update only changes the order in which
// rows are filled).  A count pass sizes each row, a scan gives row offsets, and a fill pass
// writes columns / values in the same deterministic traversal order.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "ctx.h"
#include "heatbath.cuh"
#include "hrow.cuh"
#include "kernels.h"

namespace shci {

namespace {

constexpr int kWarps = 8;  // warps per block in the row kernels

__global__ void k_group_flags(const uint64_t* sorted, size_t n, uint32_t* flags) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    flags[k] = (k == 0 || sorted[k] != sorted[k - 1]) ? 1u : 0u;
}

// After the exclusive scan of the flags: g = scan[k] + flag[k] - 1 is the group of k.
__global__ void k_group_fill(const uint64_t* sorted, const uint32_t* perm, const uint32_t* flags,
                             const uint32_t* scan, const uint64_t* other, size_t n,
                             uint32_t* start, uint64_t* uniq, uint32_t* det_gid,
                             uint64_t* other_sorted) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const uint32_t g = scan[k] + flags[k] - 1u;
    const uint32_t d = perm[k];
    if (flags[k]) {
      start[g] = static_cast<uint32_t>(k);
      uniq[g] = sorted[k];
    }
    det_gid[d] = g;
    if (other_sorted) other_sorted[k] = other[d];
  }
}

__global__ void k_widen_ids(const uint32_t* in, uint64_t* out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

__device__ __forceinline__ bool bsearch_u64(const uint64_t* a, uint32_t n, uint64_t key,
                                            uint32_t* pos) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const uint64_t v = a[mid];
    if (v < key) lo = mid + 1;
    else hi = mid;
  }
  *pos = lo;
  return lo < n && a[lo] == key;
}

// Singles of unique strings: for each sorted unique string u[g], the ids of the unique strings
// one single excitation away (and, if str_out, their strings).
template <bool FILL>
__global__ void k_singles(const uint64_t* u, uint32_t n_u, int n_orbs, uint32_t* cnt,
                          const uint32_t* off, uint32_t* list, uint64_t* str_out) {
  const uint64_t full = n_orbs == 64 ? ~0ull : ((1ull << n_orbs) - 1ull);
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < n_u; g += gridDim.x * blockDim.x) {
    const uint64_t a = u[g];
    uint32_t c = 0;
    const uint32_t base = FILL ? off[g] : 0;
    for (uint64_t mo = a; mo; mo &= mo - 1) {
      const uint64_t ob = mo & (~mo + 1);
      for (uint64_t mv = full & ~a; mv; mv &= mv - 1) {
        const uint64_t vb = mv & (~mv + 1);
        uint32_t pos;
        if (bsearch_u64(u, n_u, a ^ ob ^ vb, &pos)) {
          if (FILL) {
            list[base + c] = pos;
            if (str_out) str_out[base + c] = a ^ ob ^ vb;
          }
          c++;
        }
      }
    }
    if (!FILL) cnt[g] = c;
  }
}

struct IndexView {
  const uint32_t *det_aid, *det_bid, *a_start, *b_start;
  const uint32_t *am_idx, *ad_idx, *bd_idx;
  const uint64_t *am_dn, *ad_dn, *bd_up;
  const uint64_t* ua;
  const uint32_t *as_off, *as_list, *bs_off;
  const uint64_t* bs_str;
};

// first k in [lo, hi) with idx[k] > i (idx ascending)
__device__ __forceinline__ uint32_t first_after(const uint32_t* idx, uint32_t lo, uint32_t hi,
                                                uint32_t i) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (idx[mid] <= i) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// first k in [lo, hi) with a[k] >= key (a ascending)
__device__ __forceinline__ uint32_t lower_bound_u64(const uint64_t* a, uint32_t lo, uint32_t hi,
                                                    uint64_t key) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Diagonal elements, a thread per det (chem_system.cc:426-432 via h_diag).
__global__ void k_hdiag(DevIntegrals I, const uint64_t* __restrict__ up,
                        const uint64_t* __restrict__ dn, uint32_t n, double* diag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    diag[i] = h_diag(I, up[i], dn[i]);
}

// Scan traversal.  MODE 0: count, MODE 1: fill FP64, MODE 2: fill mixed (RowSink).
template <int MODE>
__global__ void __launch_bounds__(kWarps * 32)
    k_hbuild(DevIntegrals I, const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn,
             uint32_t n, IndexView ix, uint32_t* row_cnt, const uint64_t* row_ptr,
             uint32_t* col, double* v64, float* v32, float* r32, unsigned* work,
             float* absacc) {
  __shared__ RowQueues qs[kWarps];
  RowQueues& q = qs[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31;
  while (true) {
    uint32_t i = 0;
    if (lane == 0) i = atomicAdd(work, 1u);
    i = __shfl_sync(kFull, i, 0);
    if (i >= n) break;
    const uint64_t ui = up[i], di = dn[i];
    const uint32_t a = ix.det_aid[i], b = ix.det_bid[i];
    RowSink<MODE> sink(q, I, ui, di, MODE ? row_ptr[i] : 0, col, v64, v32, r32);
    if (MODE == 0 && absacc) sink.track_abs(absacc, i);
    uint64_t n_scan_a = 0, n_scan_b = 0, n_mixed = 0;
    auto push = [&](bool cand, bool single, uint32_t j, uint64_t uj, uint64_t dj) {
      sink.push(cand, single, j, uj, dj);
    };
    // (a) same beta string: beta group in det-id order, from the first j > i
    {
      const uint32_t e = ix.b_start[b + 1];
      const uint32_t s = first_after(ix.bd_idx, ix.b_start[b], e, i);
      n_scan_a = e - s;
      for (uint32_t k0 = s; k0 < e; k0 += 32) {
        const uint32_t k = k0 + lane;
        bool cand = false;
        uint32_t j = 0;
        uint64_t uj = 0;
        int x = 0;
        if (k < e) {
          j = ix.bd_idx[k];
          uj = ix.bd_up[k];
          x = popc64(uj ^ ui);
          cand = x <= 4;
        }
        push(cand, x == 2, j, uj, di);
      }
    }
    // (b) same alpha string: alpha group in det-id order, from the first j > i
    {
      const uint32_t e = ix.a_start[a + 1];
      const uint32_t s = first_after(ix.ad_idx, ix.a_start[a], e, i);
      n_scan_b = e - s;
      for (uint32_t k0 = s; k0 < e; k0 += 32) {
        const uint32_t k = k0 + lane;
        bool cand = false;
        uint32_t j = 0;
        uint64_t dj = 0;
        int x = 0;
        if (k < e) {
          j = ix.ad_idx[k];
          dj = ix.ad_dn[k];
          x = popc64(dj ^ di);
          cand = x <= 4;
        }
        push(cand, x == 2, j, ui, dj);
      }
    }
    // (c) alpha single x beta single
    {
      const uint32_t s0 = ix.as_off[a], s1 = ix.as_off[a + 1];
      const uint32_t b0 = ix.bs_off[b], nbs = ix.bs_off[b + 1] - b0;
      const uint32_t thr = 4u * nbs + 32u;  // probe groups larger than this
      for (uint32_t c0 = s0; c0 < s1; c0 += 32) {
        const uint32_t c = c0 + lane;
        uint32_t g = 0, gs = 0, gn = 0;
        if (c < s1) {
          g = ix.as_list[c];
          gs = ix.a_start[g];
          gn = ix.a_start[g + 1] - gs;
        }
        const bool probe = gn > thr;
        const uint32_t sn = probe ? 0u : gn;
        // scan mode: flatten (alpha single, group member) pairs over lanes
        uint32_t inc = sn;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(kFull, inc, o);
          if (lane >= (unsigned)o) inc += t;
        }
        const uint32_t total = __shfl_sync(kFull, inc, 31);
        n_mixed += total;
        for (uint32_t t0 = 0; t0 < total; t0 += 32) {
          const uint32_t t = t0 + lane;
          bool cand = false;
          uint32_t j = 0;
          uint64_t uj = 0, dj = 0;
          // owner lane = number of lanes whose inclusive prefix is <= t (prefixes are
          // non-decreasing); a fixed 5-step search so every lane runs the same shuffles
          uint32_t lo = 0;
#pragma unroll
          for (uint32_t step = 16; step; step >>= 1) {
            const uint32_t v = __shfl_sync(kFull, inc, lo + step - 1);
            if (v <= t) lo += step;
          }
          const uint32_t o_inc = __shfl_sync(kFull, inc, lo);
          const uint32_t o_n = __shfl_sync(kFull, sn, lo);
          const uint32_t o_gs = __shfl_sync(kFull, gs, lo);
          const uint32_t o_g = __shfl_sync(kFull, g, lo);
          if (t < total) {
            const uint32_t k = o_gs + (t - (o_inc - o_n));
            j = ix.am_idx[k];
            if (j > i) {
              dj = ix.am_dn[k];
              if (popc64(dj ^ di) == 2) {
                uj = ix.ua[o_g];
                cand = true;
              }
            }
          }
          push(cand, false, j, uj, dj);
        }
        // probe mode: binary-search each beta single of the row in the big groups
        unsigned pmask = __ballot_sync(kFull, probe);
        while (pmask) {
          const int l = __ffs(pmask) - 1;
          pmask &= pmask - 1;
          const uint32_t p_gs = __shfl_sync(kFull, gs, l);
          const uint32_t p_gn = __shfl_sync(kFull, gn, l);
          const uint32_t p_g = __shfl_sync(kFull, g, l);
          const uint64_t ua2 = ix.ua[p_g];
          n_mixed += nbs;
          for (uint32_t k0 = 0; k0 < nbs; k0 += 32) {
            const uint32_t k = k0 + lane;
            bool cand = false;
            uint32_t j = 0;
            uint64_t bstr = 0;
            if (k < nbs) {
              bstr = ix.bs_str[b0 + k];
              const uint32_t pos = lower_bound_u64(ix.am_dn, p_gs, p_gs + p_gn, bstr);
              if (pos < p_gs + p_gn && ix.am_dn[pos] == bstr) {
                j = ix.am_idx[pos];
                cand = j > i;
              }
            }
            push(cand, false, j, ua2, bstr);
          }
        }
      }
    }
    const uint32_t cnt = sink.finish();
    if (MODE == 0 && lane == 0) {
      row_cnt[i] = cnt;
      // candidates examined by this row, per part
      unsigned long long* cc = reinterpret_cast<unsigned long long*>(work + 2);
      atomicAdd(cc + 0, (unsigned long long)n_scan_a);
      atomicAdd(cc + 1, (unsigned long long)n_scan_b);
      atomicAdd(cc + 2, (unsigned long long)n_mixed);
    }
    __syncwarp();
  }
}

}  // namespace

// Sorts det ids by group id (stable: det-id order within each group) and gathers `other`.
static void group_by_det_id(shci_ctx* c, const uint32_t* gid, size_t n_groups,
                            const uint64_t* other, DevBuf<uint32_t>& idx_out,
                            DevBuf<uint64_t>& other_out) {
  const size_t n = c->up.size();
  cudaStream_t s = c->stream;
  int bits = 1;
  while ((1ull << bits) < n_groups + 1) bits++;
  k_widen_ids<<<grid_for(n, 256), 256, 0, s>>>(gid, c->k0.p, n);
  SHCI_LAUNCH_CHECK();
  iota_u32(c->u0.p, n, s);
  radix_sort_pairs(c->k0, c->u0, n, 0, bits, s, c->sort);
  SHCI_CUDA(cudaMemcpyAsync(idx_out.p, c->u0.p, n * 4, cudaMemcpyDeviceToDevice, s));
  gather_u64(other, c->u0.p, other_out.p, n, s);
  c->launches += 3;
}

static void build_singles(shci_ctx* c, const DevBuf<uint64_t>& u, size_t n_u, DevBuf<uint32_t>& off,
                          DevBuf<uint32_t>& list, DevBuf<uint64_t>* str) {
  cudaStream_t s = c->stream;
  const int nb = c->I.n;
  const uint32_t nu = static_cast<uint32_t>(n_u);
  off.resize(nu + 1, 1.25);
  c->u1.reserve(nu + 1, 1.25);
  k_singles<false><<<grid_for(nu, 128), 128, 0, s>>>(u.p, nu, nb, c->u1.p, nullptr, nullptr,
                                                     nullptr);
  SHCI_LAUNCH_CHECK();
  const uint32_t tot = exclusive_scan_u32(c->u1.p, off.p, nu, s, c->sort);
  SHCI_CUDA(cudaMemcpyAsync(off.p + nu, &tot, 4, cudaMemcpyHostToDevice, s));
  list.resize(tot ? tot : 1, 1.25);
  if (str) str->resize(tot ? tot : 1, 1.25);
  k_singles<true><<<grid_for(nu, 128), 128, 0, s>>>(u.p, nu, nb, nullptr, off.p, list.p,
                                                    str ? str->p : nullptr);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 3;
}

void build_index(shci_ctx* c) {
  auto& ix = c->idx;
  const size_t n = c->up.size();
  cudaStream_t s = c->stream;
  ProfScope ps(c->prof, s, "det_index");
  const int nb = c->I.n;
  ix.n = n;
  c->k0.resize(n, 1.25);
  c->k1.resize(n, 1.25);
  c->u0.resize(n, 1.25);
  c->u1.resize(n, 1.25);
  c->u2.resize(n, 1.25);
  ix.det_aid.resize(n, 1.25);
  ix.det_bid.resize(n, 1.25);
  ix.am_idx.resize(n, 1.25);
  ix.am_dn.resize(n, 1.25);
  ix.ad_idx.resize(n, 1.25);
  ix.ad_dn.resize(n, 1.25);
  ix.bd_idx.resize(n, 1.25);
  ix.bd_up.resize(n, 1.25);
  for (int major = 0; major < 2; major++) {
    // major 0: by (up, dn) - sort by dn, then stably by up; major 1: by (dn, up).
    const uint64_t* first = major == 0 ? c->d_dn.p : c->d_up.p;
    const uint64_t* second = major == 0 ? c->d_up.p : c->d_dn.p;
    SHCI_CUDA(cudaMemcpyAsync(c->k0.p, first, n * 8, cudaMemcpyDeviceToDevice, s));
    iota_u32(c->u0.p, n, s);
    radix_sort_pairs(c->k0, c->u0, n, 0, nb, s, c->sort);
    gather_u64(second, c->u0.p, c->k1.p, n, s);
    radix_sort_pairs(c->k1, c->u0, n, 0, nb, s, c->sort);
    k_group_flags<<<grid_for(n, 256), 256, 0, s>>>(c->k1.p, n, c->u1.p);
    SHCI_LAUNCH_CHECK();
    const uint32_t ng = exclusive_scan_u32(c->u1.p, c->u2.p, n, s, c->sort);
    auto& start = major == 0 ? ix.a_start : ix.b_start;
    auto& uniq = major == 0 ? ix.ua : ix.ub;
    auto& gid = major == 0 ? ix.det_aid : ix.det_bid;
    start.resize(ng + 1, 1.25);
    uniq.resize(ng, 1.25);
    if (major == 0)
      SHCI_CUDA(cudaMemcpyAsync(ix.am_idx.p, c->u0.p, n * 4, cudaMemcpyDeviceToDevice, s));
    k_group_fill<<<grid_for(n, 256), 256, 0, s>>>(c->k1.p, c->u0.p, c->u1.p, c->u2.p, first, n,
                                                  start.p, uniq.p, gid.p,
                                                  major == 0 ? ix.am_dn.p : nullptr);
    SHCI_LAUNCH_CHECK();
    const uint32_t nn = static_cast<uint32_t>(n);
    SHCI_CUDA(cudaMemcpyAsync(start.p + ng, &nn, 4, cudaMemcpyHostToDevice, s));
    if (major == 0) ix.n_alpha = ng;
    else ix.n_beta = ng;
    SHCI_CUDA(cudaStreamSynchronize(s));
    c->launches += 10;
  }
  // groups in det-id order (the sort is stable and starts from det-id order)
  group_by_det_id(c, ix.det_aid.p, ix.n_alpha, c->d_dn.p, ix.ad_idx, ix.ad_dn);
  group_by_det_id(c, ix.det_bid.p, ix.n_beta, c->d_up.p, ix.bd_idx, ix.bd_up);
  // single-excitation lists of the unique strings
  build_singles(c, ix.ua, ix.n_alpha, ix.as_off, ix.as_list, nullptr);
  build_singles(c, ix.ub, ix.n_beta, ix.bs_off, ix.bs_list, &ix.bs_str);
}

// Allocates the element store for `cap` elements in the build's precision.
static void alloc_store(shci_ctx* c, int precision, size_t cap) {
  auto& H = c->H;
  if (cap == 0) cap = 1;
  H.col.resize(cap, 1.1);
  if (precision == SHCI_PREC_FP64) {
    H.val32.release();
    H.res32.release();
    H.val64.resize(cap, 1.1);
  } else {
    H.val64.release();
    H.val32.resize(cap, 1.1);
    H.res32.resize(cap, 1.1);
  }
}

// Bytes free for the element store: device free memory within the context's budget.
static size_t store_room(shci_ctx* c) {
  size_t free_b = 0, total_b = 0;
  SHCI_CUDA(cudaMemGetInfo(&free_b, &total_b));
  // the store's current allocation is reused or freed before the new one is made
  const auto& H = c->H;
  size_t held = H.col.cap * 4 + H.val64.cap * 8 + H.val32.cap * 4 + H.res32.cap * 4;
  size_t room = free_b + c->mem.cached + held;  // cached blocks return to the driver on demand
  const size_t live = c->mem.live();
  if (c->mem.budget)
    room = std::min(room, c->mem.budget > live - held ? c->mem.budget - (live - held)
                                                      : (size_t)0);
  return room;
}

// Builds H for the current dets.  Paths:
//   join, one pass  - rows sized by their join candidate counts (an upper bound), filled in a
//                     single pass that also records each row's kept length (rows not packed);
//   join, two pass  - count, scan, fill (packed rows), when the bound does not fit in memory;
//   scan            - group index + scan traversal, count and fill (packed rows).
// SHCI_HBUILD=scan forces the scan path, SHCI_HBUILD=join2 the two-pass join.
namespace {

// Bound of sum_j |H_ij| over every excitation of det i (both triangles of its row): the singles
// queue values of its electrons' orbitals (each S_pr bounds |H| of p -> r for any det) plus
// the doubles queue values of its electron pairs (the exact |H| of each pq -> rs), summed per
// orbital / pair ahead (s_tot, d_tot); a warp per det, lanes over its electrons.  The mixed
// H*v only needs a valid bound for its fixed-point scale, and one per det, independent of the
// det list, saves the fill an FP32 atomic per stored element.
__global__ void k_hb_row_bound(const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn,
                               uint32_t begin, uint32_t end, int n, int n_up, int n_elecs,
                               const double* __restrict__ stot, const double* __restrict__ dtot,
                               float* __restrict__ rowabs) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = begin + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < end;
       i += warps) {
    const uint64_t u = up[i], d = dn[i];
    double acc = 0.0;
    for (int a = static_cast<int>(lane); a < n_elecs; a += 32) {
      const int p = elec_orb(u, d, a, n_up, n);
      acc += stot[p < n ? p : p - n];
      for (int b = a + 1; b < n_elecs; b++) {
        const int q = elec_orb(u, d, b, n_up, n);
        int p2 = p, q2 = q;
        if (p >= n && q >= n) {
          p2 -= n;
          q2 -= n;
        } else if (p < n && q >= n && p > q - n) {
          p2 = q - n;
          q2 = p + n;
        }
        acc += dtot[c2(p2, q2)];
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if (lane == 0) rowabs[i] = __double2float_ru(acc);
  }
}

}  // namespace

size_t build_hamiltonian(shci_ctx* c, int precision) {
  if (c->time_sym) return build_time_sym(c, precision);
  auto& H = c->H;
  auto& ix = c->idx;
  const size_t n = c->up.size();
  cudaStream_t s = c->stream;
  if (n >= 0xffffffffull) throw ArgError("more than 2^32-1 dets");
  const char* force = std::getenv("SHCI_HBUILD");
  const bool scan_only = force && std::strcmp(force, "scan") == 0;
  const bool two_pass = force && std::strcmp(force, "join2") == 0;
  // Incremental update (Hamiltonian<S>::update with n_dets_prev, hamiltonian.h:89-93,
  // 421-428): when the stored matrix is that of the first H.n dets of the list and dets were
  // only appended, the new segment holds the new rows and the old rows' new columns.
  // SHCI_HBUILD_INCREMENTAL=0 forces full rebuilds.
  const char* inc_env = std::getenv("SHCI_HBUILD_INCREMENTAL");
  const bool inc_ok = !(inc_env && std::strcmp(inc_env, "0") == 0);
  size_t n_prev = 0;
  if (inc_ok && H.prefix_ok && H.join && H.n > 0 && H.n < n && H.precision == precision &&
      H.older.size() + 1 < kMaxSegments &&
      (precision == SHCI_PREC_FP64 || H.rowabs.n == H.n))
    n_prev = H.n;
  H.prefix_ok = false;
  H.valid = false;
  H.build_id++;
  H.bound_valid = false;
  H.join = !scan_only && join_prepare(c);
  if (!H.join) n_prev = 0;  // the group scan builds whole matrices only
  if (n_prev) {
    // keep the current store as an older segment
    auto seg = std::make_unique<HSeg>();
    seg->row_ptr.mt = seg->col.mt = &c->mem;
    seg->row_cnt.mt = &c->mem;
    seg->val64.mt = seg->val32.mt = seg->res32.mt = &c->mem;
    seg->n = H.n;
    seg->nnz = H.nnz_current;
    seg->packed = H.packed;
    seg->row_ptr.swap(H.row_ptr);
    seg->row_cnt.swap(H.row_cnt);
    seg->col.swap(H.col);
    seg->val64.swap(H.val64);
    seg->val32.swap(H.val32);
    seg->res32.swap(H.res32);
    H.older.push_back(std::move(seg));
  } else {
    H.older.clear();
  }
  H.n_prev = n_prev;
  H.n = n;
  H.precision = precision;
  if (!H.join) build_index(c);
  H.row_ptr.resize(n + 1, 1.25);
  H.row_cnt.resize(n + 1, 1.25);
  H.diag.resize(n, 1.25);
  // err_word layout: [0] row work counter, [1] unused, [2..7] three u64 candidate counters
  c->err_word.resize(8);
  IndexView v{ix.det_aid.p, ix.det_bid.p, ix.a_start.p, ix.b_start.p, ix.am_idx.p,
              ix.ad_idx.p,  ix.bd_idx.p,  ix.am_dn.p,   ix.ad_dn.p,   ix.bd_up.p,
              ix.ua.p,      ix.as_off.p,  ix.as_list.p, ix.bs_off.p,  ix.bs_str.p};
  int dev_sms = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device));
  const unsigned grid = static_cast<unsigned>(dev_sms) * 8u;
  unsigned* work = c->err_word.p;
  SHCI_CUDA(cudaMemsetAsync(work, 0, 8 * sizeof(unsigned), s));
  // A mixed build needs a bound of sum_j |H_ij| per det (the H*v fixed-point scale): the
  // heat-bath bound of each det when the queues exist (new dets only on an incremental update
  // over such bounds), else the stored elements' |H| summed by the fill (an incremental one
  // adding to the sums of the older segments).
  float* absacc = nullptr;
  bool hb_bound = false;
  if (precision == SHCI_PREC_MIXED) {
    if (n_prev) H.rowabs.grow_keep(n, s, 1.1);
    else H.rowabs.resize(n, 1.1);
    if (c->Q.built) {
      const uint32_t begin = (n_prev && H.rowabs_hb) ? static_cast<uint32_t>(n_prev) : 0u;
      const int n_elecs = static_cast<int>(c->I.n_up + c->I.n_dn);
      k_hb_row_bound<<<grid_for((size_t)(n - begin) * 32, 256), 256, 0, s>>>(
          c->d_up.p, c->d_dn.p, begin, static_cast<uint32_t>(n), static_cast<int>(c->I.n),
          static_cast<int>(c->I.n_up), n_elecs, c->Q.s_tot.p, c->Q.d_tot.p, H.rowabs.p);
      SHCI_LAUNCH_CHECK();
      c->launches += 1;
      H.rowabs_hb = true;
      hb_bound = true;
    } else {
      // (older rows keep their sums, or their heat-bath bounds, which bound any new columns too)
      if (n_prev)
        SHCI_CUDA(cudaMemsetAsync(H.rowabs.p + n_prev, 0, (n - n_prev) * sizeof(float), s));
      else
        SHCI_CUDA(cudaMemsetAsync(H.rowabs.p, 0, n * sizeof(float), s));
      absacc = H.rowabs.p;
      H.rowabs_hb = false;
    }
  } else {
    H.rowabs.release();
    H.rowabs_hb = false;
  }
  k_hdiag<<<grid_for(n, 256), 256, 0, s>>>(c->dI, c->d_up.p, c->d_dn.p, (uint32_t)n, H.diag.p);
  SHCI_LAUNCH_CHECK();
  const int fill_mode = precision == SHCI_PREC_FP64 ? 1 : 2;
  uint64_t nnz = 0;
  bool one_pass = false;
  if (H.join && !two_pass) {
    const uint64_t cap = join_row_caps(c, H.row_ptr.p, static_cast<uint32_t>(n_prev));
    one_pass = static_cast<double>(cap) * 12.0 * 1.1 < 0.9 * static_cast<double>(store_room(c));
    if (one_pass) {
      alloc_store(c, precision, cap);
      {
        ProfScope ps(c->prof, s, "hbuild_fill");
        join_rows(c, fill_mode, H.row_cnt.p, H.row_ptr.p, H.col.p, H.val64.p, H.val32.p,
                  H.res32.p, work, grid, absacc, static_cast<uint32_t>(n_prev));
      }
      c->k0.resize(n, 1.25);
      widen_u32_u64(H.row_cnt.p, c->k0.p, n, s);
      nnz = exclusive_scan_u64(c->k0.p, c->k0.p, n, s, c->sort);
      H.packed = false;
    }
  }
  if (!one_pass) {
    {
      ProfScope ps(c->prof, s, "hbuild_count");
      if (H.join) {
        join_rows(c, 0, H.row_cnt.p, nullptr, nullptr, nullptr, nullptr, nullptr, work, grid,
                  absacc, static_cast<uint32_t>(n_prev));
      } else {
        k_hbuild<0><<<grid, kWarps * 32, 0, s>>>(c->dI, c->d_up.p, c->d_dn.p, (uint32_t)n, v,
                                                 H.row_cnt.p, nullptr, nullptr, nullptr,
                                                 nullptr, nullptr, work, absacc);
        SHCI_LAUNCH_CHECK();
      }
    }
    // row_ptr = exclusive scan of counts (counts widened to 64 bit)
    widen_u32_u64(H.row_cnt.p, H.row_ptr.p, n, s);
    nnz = exclusive_scan_u64(H.row_ptr.p, H.row_ptr.p, n, s, c->sort);
    SHCI_CUDA(cudaMemcpyAsync(H.row_ptr.p + n, &nnz, 8, cudaMemcpyHostToDevice, s));
  }
  unsigned long long cand[3] = {0, 0, 0};
  SHCI_CUDA(cudaMemcpyAsync(cand, work + 2, 24, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  if (absacc || hb_bound) finish_mixed_bound(c);
  H.nnz_current = nnz;
  H.nnz = nnz;
  for (const auto& sg : H.older) H.nnz += sg->nnz;
  H.candidates = cand[0] + cand[1] + cand[2];
  for (int k = 0; k < 3; k++) H.cand_parts[k] = cand[k];
  if (H.join) {
    H.cand_parts[0] = c->join.m;
    H.cand_parts[1] = H.cand_parts[2] = 0;
  }
  if (!one_pass) {
    alloc_store(c, precision, nnz);
    SHCI_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned), s));
    {
      ProfScope ps(c->prof, s, "hbuild_fill");
      if (H.join) {
        join_rows(c, fill_mode, nullptr, H.row_ptr.p, H.col.p, H.val64.p, H.val32.p, H.res32.p,
                  work, grid, nullptr, static_cast<uint32_t>(n_prev));
      } else if (precision == SHCI_PREC_FP64) {
        k_hbuild<1><<<grid, kWarps * 32, 0, s>>>(c->dI, c->d_up.p, c->d_dn.p, (uint32_t)n, v,
                                                 nullptr, H.row_ptr.p, H.col.p, H.val64.p,
                                                 nullptr, nullptr, work, nullptr);
      } else {
        k_hbuild<2><<<grid, kWarps * 32, 0, s>>>(c->dI, c->d_up.p, c->d_dn.p, (uint32_t)n, v,
                                                 nullptr, H.row_ptr.p, H.col.p, nullptr,
                                                 H.val32.p, H.res32.p, work, nullptr);
      }
      SHCI_LAUNCH_CHECK();
    }
    H.packed = true;
  }
  SHCI_CUDA(cudaStreamSynchronize(s));
  if (H.join) join_release(c);
  if (row_sort_enabled()) sort_rows(c);
  c->prof.flush();
  H.valid = true;
  H.prefix_ok = true;
  H.build_id++;
  c->launches += 5;
  return nnz;
}

}  // namespace shci

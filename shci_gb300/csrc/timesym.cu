// Time-reversal-symmetric Hamiltonian (config "time_sym"): the packed matrix that
// Hamiltonian<S>::update_matrix builds with time_sym (src/solver/hamiltonian.h:415-598), with
// elements get_hamiltonian_elem_time_sym (src/base_system.h:86-101).
//
// The det list holds one det of each time-reversal pair, the one with up <= dn; an open det a
// (up != dn) stands for (|a> + |a~>) / sqrt(2), a~ = (dn, up).  Two packed dets a, b are
// connected when b is within a double excitation of a or of a~; the reference finds those
// pairs with extra passes over the reversed strings (:448-459, 473-484, 535-590).  Here the
// ordinary build (two-hole core join) runs once over the unpacked list U = the packed dets
// followed by the reverses of the open ones, which yields every connected pair (u, v) of U;
// each maps to the packed pair (P(u), P(v)) (pairs (a, a~) feed the diagonal instead), a radix
// sort makes the packed pairs unique, and every pair is evaluated with the reference's formula
//   closed a: H_ab (b closed) or sqrt(2) H_ab (b open)
//   open a:   sqrt(2) H_ab (b closed) or H_ab + H_a~b (b open)
// and kept when |value| >= 1e-12.  The diagonal is H_aa + H_a~a for open a.  The pairs come out
// sorted, so each row is in increasing column order.  (The unpacked build keeps elements of
// |H| >= 1e-12, so a packed pair whose every unpacked element is below that threshold while
// their combination is not would be missed; no such pair has been seen.)
#include <algorithm>
#include <stdexcept>
#include <vector>

#include "ctx.h"
#include "heatbath.cuh"
#include "kernels.h"
#include "sort.cuh"

namespace shci {

namespace {

__device__ __forceinline__ double ts_elem(const DevIntegrals& I, uint64_t ua, uint64_t da,
                                          uint64_t ub, uint64_t db) {
  double h = h_offdiag(I, ua, da, ub, db);
  if (ua == da) {
    if (ub != db) h *= kSqrt2;
  } else if (ub == db) {
    h *= kSqrt2;
  } else {
    h += h_offdiag(I, da, ua, ub, db);
  }
  return h;
}

// Packed pair key (min << 32 | max) of every stored element of the unpacked store; kInvalid
// for an element between a det and its own reverse.  keys was filled with kInvalid (gaps).
__global__ void k_ts_pairs(const uint64_t* __restrict__ row_ptr, const uint32_t* __restrict__ row_cnt,
                           const uint32_t* __restrict__ col, const uint32_t* __restrict__ pidx,
                           uint32_t m, uint64_t* __restrict__ keys) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t u = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < m; u += warps) {
    const uint64_t rs = row_ptr[u], re = rs + row_cnt[u];
    const uint64_t pu = pidx[u];
    for (uint64_t k = rs + lane; k < re; k += 32) {
      const uint64_t pv = pidx[col[k]];
      keys[k] = pu == pv ? kInvalid : (pu < pv ? (pu << 32 | pv) : (pv << 32 | pu));
    }
  }
}

__global__ void k_ts_eval(const uint64_t* __restrict__ keys, size_t K, DevIntegrals I,
                          const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn,
                          double* __restrict__ val, uint32_t* __restrict__ keep,
                          uint32_t* __restrict__ row_cnt) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < K;
       k += (size_t)gridDim.x * blockDim.x) {
    const uint32_t a = static_cast<uint32_t>(keys[k] >> 32), b = static_cast<uint32_t>(keys[k]);
    const double h = ts_elem(I, up[a], dn[a], up[b], dn[b]);
    const bool kp = keep_elem(h);
    val[k] = h;
    keep[k] = kp ? 1u : 0u;
    if (kp) atomicAdd(&row_cnt[a], 1u);
  }
}

__global__ void k_ts_place(const uint64_t* __restrict__ keys, const double* __restrict__ val,
                           const uint32_t* __restrict__ keep, const uint32_t* __restrict__ pos,
                           size_t K, int mixed, uint32_t* __restrict__ col,
                           double* __restrict__ v64, float* __restrict__ v32,
                           float* __restrict__ r32) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < K;
       k += (size_t)gridDim.x * blockDim.x) {
    if (!keep[k]) continue;
    const uint32_t p = pos[k];
    col[p] = static_cast<uint32_t>(keys[k]);
    const double h = val[k];
    if (mixed) {
      const float hi = static_cast<float>(h);
      v32[p] = hi;
      r32[p] = static_cast<float>(h - static_cast<double>(hi));
    } else {
      v64[p] = h;
    }
  }
}

// H_aa + H_a~a for open a (get_hamiltonian_elem_time_sym(a, a, 0))
__global__ void k_ts_diag(DevIntegrals I, const uint64_t* __restrict__ up,
                          const uint64_t* __restrict__ dn, uint32_t n, double* __restrict__ d) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t u = up[i], w = dn[i];
    double h = h_diag(I, u, w);
    if (u != w) h += h_offdiag(I, w, u, u, w);
    d[i] = h;
  }
}

}  // namespace

size_t build_time_sym(shci_ctx* c, int precision) {
  auto& H = c->H;
  cudaStream_t s = c->stream;
  const size_t n = c->up.size();
  // the unpacked list and the packed index of each of its dets
  std::vector<uint64_t> uu(c->up), ud(c->dn);
  std::vector<uint32_t> pidx(n);
  for (size_t i = 0; i < n; i++) pidx[i] = static_cast<uint32_t>(i);
  for (size_t i = 0; i < n; i++)
    if (c->up[i] != c->dn[i]) {
      uu.push_back(c->dn[i]);
      ud.push_back(c->up[i]);
      pidx.push_back(static_cast<uint32_t>(i));
    }
  const size_t m = uu.size();
  if (m >= 0xffffffffull) throw ArgError("more than 2^32-1 unpacked dets");
  // the ordinary build over U, with U as the context's det list
  DevBuf<uint64_t> d_uu, d_ud;
  d_uu.mt = d_ud.mt = &c->mem;
  d_uu.resize(m);
  d_ud.resize(m);
  SHCI_CUDA(cudaMemcpyAsync(d_uu.p, uu.data(), m * 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(d_ud.p, ud.data(), m * 8, cudaMemcpyHostToDevice, s));
  std::swap(c->up, uu);
  std::swap(c->dn, ud);
  c->d_up.swap(d_uu);
  c->d_dn.swap(d_ud);
  auto restore = [&]() {
    std::swap(c->up, uu);
    std::swap(c->dn, ud);
    c->d_up.swap(d_uu);
    c->d_dn.swap(d_ud);
  };
  DevBuf<uint64_t> keys, zero;
  keys.mt = zero.mt = &c->mem;
  size_t K = 0;
  try {
    c->time_sym = false;
    H.prefix_ok = false;
    build_hamiltonian(c, SHCI_PREC_FP64);
    c->time_sym = true;
    // packed pairs of every unpacked element
    DevBuf<uint32_t> d_pidx;
    d_pidx.mt = &c->mem;
    d_pidx.resize(m);
    SHCI_CUDA(cudaMemcpyAsync(d_pidx.p, pidx.data(), m * 4, cudaMemcpyHostToDevice, s));
    const size_t len = std::max<size_t>(H.col.n, 1);
    DevBuf<uint64_t> raw;
    raw.mt = &c->mem;
    raw.resize(len);
    SHCI_CUDA(cudaMemsetAsync(raw.p, 0xff, len * 8, s));
    k_ts_pairs<<<grid_for((size_t)m * 32, 256), 256, 0, s>>>(H.row_ptr.p, H.row_cnt.p, H.col.p,
                                                             d_pidx.p, (uint32_t)m, raw.p);
    SHCI_LAUNCH_CHECK();
    SHCI_CUDA(cudaStreamSynchronize(s));
    // drop the unpacked store before sorting the pairs
    H.col.release();
    H.val64.release();
    H.val32.release();
    H.res32.release();
    DevBuf<uint64_t> rz;
    rz.mt = &c->mem;
    rz.resize(len);
    SHCI_CUDA(cudaMemsetAsync(rz.p, 0, len * 8, s));
    compact_valid(c, raw.p, rz.p, nullptr, 0, len, keys, zero, nullptr, &K);
    raw.release();
    rz.release();
    K = sort_unique_pairs(c, keys, zero, K, nullptr, 1, 64);
    c->launches += 1;
  } catch (...) {
    c->time_sym = true;
    restore();
    H.valid = false;
    throw;
  }
  restore();
  // evaluate, keep, place
  H.older.clear();
  H.n = n;
  H.n_prev = 0;
  H.precision = precision;
  H.join = false;
  H.packed = true;
  H.bound_valid = false;
  H.rowabs.release();
  H.rowabs_hb = false;
  H.row_ptr.resize(n + 1, 1.25);
  H.row_cnt.resize(n + 1, 1.25);
  H.diag.resize(n, 1.25);
  SHCI_CUDA(cudaMemsetAsync(H.row_cnt.p, 0, (n + 1) * 4, s));
  DevBuf<double> val;
  DevBuf<uint32_t> keep, pos;
  val.mt = &c->mem;
  keep.mt = pos.mt = &c->mem;
  val.resize(std::max<size_t>(K, 1));
  keep.resize(std::max<size_t>(K, 1));
  pos.resize(std::max<size_t>(K, 1));
  if (K) {
    k_ts_eval<<<grid_for(K, 256), 256, 0, s>>>(keys.p, K, c->dI, c->d_up.p, c->d_dn.p, val.p,
                                               keep.p, H.row_cnt.p);
    SHCI_LAUNCH_CHECK();
  }
  const uint32_t nnz = K ? exclusive_scan_u32(keep.p, pos.p, K, s, c->sort) : 0u;
  widen_u32_u64(H.row_cnt.p, H.row_ptr.p, n, s);
  const uint64_t total = exclusive_scan_u64(H.row_ptr.p, H.row_ptr.p, n, s, c->sort);
  SHCI_CUDA(cudaMemcpyAsync(H.row_ptr.p + n, &total, 8, cudaMemcpyHostToDevice, s));
  const bool mixed = precision == SHCI_PREC_MIXED;
  H.col.mt = H.val64.mt = H.val32.mt = H.res32.mt = &c->mem;
  H.col.resize(std::max<uint64_t>(nnz, 1));
  if (mixed) {
    H.val32.resize(std::max<uint64_t>(nnz, 1));
    H.res32.resize(std::max<uint64_t>(nnz, 1));
  } else {
    H.val64.resize(std::max<uint64_t>(nnz, 1));
  }
  if (K) {
    k_ts_place<<<grid_for(K, 256), 256, 0, s>>>(keys.p, val.p, keep.p, pos.p, K, mixed ? 1 : 0,
                                                H.col.p, H.val64.p, H.val32.p, H.res32.p);
    SHCI_LAUNCH_CHECK();
  }
  k_ts_diag<<<grid_for(n, 256), 256, 0, s>>>(c->dI, c->d_up.p, c->d_dn.p, (uint32_t)n, H.diag.p);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));
  if (total != nnz)
    throw std::runtime_error("time-symmetric build: row counts disagree with the kept pairs");
  H.nnz = H.nnz_current = nnz;
  H.candidates = K;
  H.cand_parts[0] = K;
  H.cand_parts[1] = H.cand_parts[2] = 0;
  H.valid = true;
  H.prefix_ok = false;  // every update rebuilds (the unpacked list is not append-only)
  H.build_id++;
  c->launches += 5;
  return nnz;
}

}  // namespace shci

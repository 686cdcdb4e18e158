// Heat-bath selection (K6): one step of Solver<S>::run_variation's "get next det list".
//
// Reference: src/solver/solver.h:435-495 driving ChemSystem::find_connected_dets
// (src/chem/chem_system.cc:289-402).  For each pass j = 0..4 over var dets i = j (mod 5):
//   eps_min = eps_var / |c_i| (0 for i = 0 with var_sd), skipped when eps_min >=
//   eps_tried_prev[i]; singles from singles_queue[p] with S >= eps_min whose |H_ai| >= eps_min,
//   doubles from hci_queue[pq] with eps_min <= H < eps_tried_prev[i]; dets already in the
//   variational set are dropped; eps_tried_prev[i] = 1.000000001 * eps_min.
// The reference walks each sorted queue until the first entry below eps_min.  Here the
// queues are sorted the same way in HBM and a binary search gives the exact entry range of
// every (det, queue) slot, so the number of candidates each det emits is known before any
// is generated:
//   k_sel_count: a warp per source det -> candidate count (also updates eps_tried_prev),
//   scan        : output segment per det,
//   k_sel_emit  : a warp per source det flattens its (slot, entry) ranges over lanes, builds
//                 each candidate det, tests membership by binary search in the sorted
//                 variational set and (singles) the |H_ai| >= eps_min rule,
//   compaction + two-stage radix sort + unique -> this pass's new dets in ascending Det order.
// New dets of a pass join the variational set before the next pass, as in the reference.
// With second rejection (off by default) the emission also drops window entries whose
// |H|^2 / (one-body energy difference to HF) is below factor * eps_min^2 and records, per
// source, the largest |H| it dropped; eps_tried_prev then becomes 1.000000001 * max(that,
// eps_min) (solver.h:461-465, chem_system.cc:300-308, 318-324, 364-370, 401).
#include <algorithm>
#include <cmath>

#include "ctx.h"
#include "heatbath.cuh"
#include "kernels.h"

namespace shci {

namespace {

// Counts candidates per source det (sources k = 0.. of this pass).  Also records whether
// the det is processed and updates eps_tried_prev (solver.h:448, 468).
__global__ void __launch_bounds__(kSelWarps * 32)
    k_sel_count(SelParams P, uint32_t k_begin, uint32_t k_end, uint64_t* cnt_out,
                double* eps_min_out) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t wpg = gridDim.x * kSelWarps;
  for (uint32_t k = k_begin + blockIdx.x * kSelWarps + (threadIdx.x >> 5); k < k_end; k += wpg) {
    const uint32_t i = P.pass + 5u * k;
    const double eps_min = src_eps_min(P, i);
    const double eps_max = P.eps_tried[i];
    uint64_t tot = 0;
    if (eps_min < eps_max) {
      const uint64_t up = P.up[i], dn = P.dn[i];
      const int n_slots = P.n_elecs + P.n_pairs;
      for (int s0 = 0; s0 < n_slots; s0 += 32) {
        uint32_t lo = 0, c = 0;
        if (s0 + (int)lane < n_slots) slot_range(P, up, dn, s0 + lane, eps_min, eps_max, &lo, &c);
        uint64_t cc = c;
#pragma unroll
        for (int o = 16; o; o >>= 1) cc += __shfl_xor_sync(kFull, cc, o);
        tot += cc;
      }
    }
    if (lane == 0) {
      cnt_out[k - k_begin] = tot;
      eps_min_out[k - k_begin] = eps_min;
    }
  }
}

// rej_max (second rejection only): the largest rejected |H| of each source, else null.  As
// find_connected_dets returns it: max(largest rejected, eps_min), except that a det whose
// eps_min is above every double's |H|, or a system without double excitations, returns
// eps_min before the doubles (chem_system.cc:339-340, 345), dropping what its singles
// rejected.
__global__ void k_sel_mark(SelParams P, uint32_t k_begin, uint32_t k_end,
                           const double* eps_min_in, const double* rej_max) {
  for (uint32_t k = k_begin + blockIdx.x * blockDim.x + threadIdx.x; k < k_end;
       k += gridDim.x * blockDim.x) {
    const uint32_t i = P.pass + 5u * k;
    const double eps_min = eps_min_in[k - k_begin];
    if (eps_min < P.eps_tried[i]) {
      const bool rej = rej_max && !P.no_doubles && !(eps_min > P.max_hci);
      P.eps_tried[i] = 1.000000001 * (rej ? fmax(rej_max[k - k_begin], eps_min) : eps_min);
    }
  }
}

// One-body energy difference of det (up, dn) from HF, accumulated in the reference's order
// (chem_system.cc:300-308): -e_hf_1b, then h_pp over the alpha electrons, then the beta ones.
__device__ __forceinline__ double diff_from_hf(const SelParams& P, uint64_t up, uint64_t dn) {
  const int n = P.n_orbs;
  double d = -P.e_hf_1b;
  for (uint64_t m = up; m; m &= m - 1) d += P.I.h1[ctz64(m) * (n + 1)];
  for (uint64_t m = dn; m; m &= m - 1) d += P.I.h1[ctz64(m) * (n + 1)];
  return d;
}

// Second-rejection test of entry e of slot `slot` (chem_system.cc:318-324, 364-370): true
// when the entry is dropped; *h is its |H| (the queue's S or H).
__device__ __forceinline__ bool second_rejected(const SelParams& P, uint64_t up, uint64_t dn,
                                                int slot, uint32_t e, double diff,
                                                double eps_min, double* h) {
  const int n = P.n_orbs;
  const double* d1 = P.I.h1;
  double den;
  if (slot < P.n_elecs) {
    const int p = slot < P.n_up ? nth_bit(up, slot) : nth_bit(dn, slot - P.n_up);
    const int r = static_cast<int>(P.s_r[e]);
    *h = P.s_S[e];
    den = diff - d1[p * (n + 1)] + d1[r * (n + 1)];
  } else {
    const uint32_t pr = P.pair_tab[slot - P.n_elecs];
    const int p = elec_orb(up, dn, pr & 0xffff, P.n_up, n);
    const int q = elec_orb(up, dn, pr >> 16, P.n_up, n);
    const uint32_t rs = P.d_rs[e];
    int r = static_cast<int>(rs & 0xffff) % n, s = static_cast<int>(rs >> 16) % n;
    if (p < n && q >= n && p > q - n) {  // the reference swaps r and s here (:357-361)
      const int t = r;
      r = s;
      s = t;
    }
    *h = P.d_H[e];
    den = diff - d1[(p % n) * (n + 1)] - d1[(q % n) * (n + 1)] + d1[r * (n + 1)] +
          d1[s * (n + 1)];
  }
  const double hv = *h;
  return den > 0. && __ddiv_rn(__dmul_rn(hv, hv), den) <
                         __dmul_rn(__dmul_rn(P.rej_factor, eps_min), eps_min);
}

__global__ void __launch_bounds__(kSelWarps * 32)
    k_sel_emit(SelParams P, uint32_t k_begin, uint32_t k_end, const uint64_t* off,
               const double* eps_min_in, uint64_t* out_up, uint64_t* out_dn, double* rej_max) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t wpg = gridDim.x * kSelWarps;
  const int n = P.n_orbs;
  for (uint32_t k = k_begin + blockIdx.x * kSelWarps + (threadIdx.x >> 5); k < k_end; k += wpg) {
    const uint32_t i = P.pass + 5u * k;
    const double eps_min = eps_min_in[k - k_begin];
    const double eps_max = P.eps_tried[i];
    if (!(eps_min < eps_max)) continue;
    const uint64_t up = P.up[i], dn = P.dn[i];
    uint64_t base = off[k - k_begin];
    const int n_slots = P.n_elecs + P.n_pairs;
    const double diff = P.rej_on ? diff_from_hf(P, up, dn) : 0.0;
    double rmax = 0.0;  // largest rejected |H| seen by this lane
    for (int s0 = 0; s0 < n_slots; s0 += 32) {
      const int slot = s0 + lane;
      uint32_t lo = 0, c = 0;
      if (slot < n_slots) slot_range(P, up, dn, slot, eps_min, eps_max, &lo, &c);
      uint32_t inc = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, inc, o);
        if (lane >= (unsigned)o) inc += t;
      }
      const uint32_t total = __shfl_sync(kFull, inc, 31);
      for (uint32_t t0 = 0; t0 < total; t0 += 32) {
        const uint32_t t = t0 + lane;
        uint32_t ol = 0;
#pragma unroll
        for (uint32_t step = 16; step; step >>= 1) {
          const uint32_t v = __shfl_sync(kFull, inc, ol + step - 1);
          if (v <= t) ol += step;
        }
        const uint32_t o_inc = __shfl_sync(kFull, inc, ol);
        const uint32_t o_c = __shfl_sync(kFull, c, ol);
        const uint32_t o_lo = __shfl_sync(kFull, lo, ol);
        if (t >= total) continue;
        const int o_slot = s0 + (int)ol;
        const uint32_t e = o_lo + (t - (o_inc - o_c));
        uint64_t cu, cd;
        bool single;
        double hr;
        if (P.rej_on && second_rejected(P, up, dn, o_slot, e, diff, eps_min, &hr)) {
          rmax = fmax(rmax, hr);
          out_up[base + t] = kInvalid;
          out_dn[base + t] = kInvalid;
          continue;
        }
        bool ok = make_candidate(P, up, dn, o_slot, e, &cu, &cd, &single);
        // time_sym: the stored form has up <= dn (solver.h:452-454)
        const bool flip = P.time_sym && cu > cd;
        const uint64_t ru = flip ? cd : cu, rd = flip ? cu : cd;
        if (ok && in_set(P, ru, rd)) ok = false;
        if (ok && single) {  // small single excitations are filtered (solver.h:456-459)
          const double h = h_offdiag(P.I, up, dn, cu, cd);
          if (fabs(h) < eps_min) ok = false;
        }
        out_up[base + t] = ok ? ru : kInvalid;
        out_dn[base + t] = ok ? rd : kInvalid;
      }
      base += total;
    }
    if (P.rej_on) {
#pragma unroll
      for (int o = 16; o; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(kFull, rmax, o));
      if (lane == 0) rej_max[k - k_begin] = rmax;
    }
  }
}

__global__ void k_valid_flags(const uint64_t* up, size_t n, uint32_t* flags) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    flags[i] = up[i] != kInvalid ? 1u : 0u;
}

__global__ void k_compact2(const uint64_t* a, const uint64_t* b, const uint32_t* flags,
                           const uint32_t* pos, size_t n, uint64_t* oa, uint64_t* ob) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    if (flags[i]) {
      oa[pos[i]] = a[i];
      ob[pos[i]] = b[i];
    }
}

// flags[k] = 1 where (su, sd)[k] differs from its predecessor
__global__ void k_unique_flags(const uint64_t* su, const uint64_t* sd, size_t n, uint32_t* flags) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    flags[k] = (k == 0 || su[k] != su[k - 1] || sd[k] != sd[k - 1]) ? 1u : 0u;
}

__global__ void k_fill_coef(double* c, size_t from, size_t to, double v) {
  for (size_t i = from + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < to;
       i += (size_t)gridDim.x * blockDim.x)
    c[i] = v;
}

// Several states: the coefficient of largest magnitude over the states, the first one on
// ties (solver.h:440-444).
struct StatePtrs {
  const double* p[kMaxStates - 1];
};
__global__ void k_max_coef(const double* c0, StatePtrs xs, int n_extra, size_t n, double* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double m = c0[i];
    for (int k = 0; k < n_extra; k++) {
      const double v = xs.p[k][i];
      if (fabs(v) > fabs(m)) m = v;
    }
    out[i] = m;
  }
}

}  // namespace

namespace {

// out[g] = sum of vals[perm[k]] over segment g = [starts[g], starts[g+1]), in input order
// (one thread per segment: a fixed summation order, independent of scheduling).
__global__ void k_segsum(const uint32_t* starts, size_t nseg, size_t m, const uint32_t* perm,
                         const double* vals, double* out) {
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < nseg;
       g += (size_t)gridDim.x * blockDim.x) {
    const size_t e = g + 1 < nseg ? starts[g + 1] : m;
    double acc = 0.0;
    for (size_t k = starts[g]; k < e; k++) acc += vals[perm[k]];
    out[g] = acc;
  }
}

__global__ void k_seg_starts(const uint32_t* flags, const uint32_t* pos, size_t m,
                             uint32_t* starts) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < m;
       k += (size_t)gridDim.x * blockDim.x)
    if (flags[k]) starts[pos[k]] = static_cast<uint32_t>(k);
}

}  // namespace

// Sorts (up, dn) pairs held in a / b (length m) into ascending (a, b) order and removes
// duplicates; returns the unique count (left in a / b).  With vals (n_vals columns), the
// values of equal keys are summed (reduce by key) and left in the columns.  a_bits = bits
// of the a key (0: n_orbs); b keys always have n_orbs bits.
size_t sort_unique_pairs(shci_ctx* c, DevBuf<uint64_t>& a, DevBuf<uint64_t>& b, size_t m,
                         DevBuf<double>* vals, int n_vals, int a_bits) {
  if (m == 0) return 0;
  cudaStream_t s = c->stream;
  const int nb = c->I.n;
  c->u0.reserve(m, 1.25);
  c->u1.reserve(m, 1.25);
  c->u2.reserve(m, 1.25);
  c->k2.reserve(m, 1.25);
  // LSD over (dn, then up): sort indices by dn, gather up, sort by up
  DevBuf<uint64_t>& key = c->k2;
  SHCI_CUDA(cudaMemcpyAsync(key.p, b.p, m * 8, cudaMemcpyDeviceToDevice, s));
  iota_u32(c->u0.p, m, s);
  radix_sort_pairs(key, c->u0, m, 0, nb, s, c->sort);
  gather_u64(a.p, c->u0.p, key.p, m, s);
  radix_sort_pairs(key, c->u0, m, 0, a_bits > 0 ? a_bits : nb, s, c->sort);
  // key = sorted ups; gather dns
  DevBuf<uint64_t> sd;
  sd.mt = &c->mem;
  sd.resize(m);
  gather_u64(b.p, c->u0.p, sd.p, m, s);
  k_unique_flags<<<grid_for(m, 256), 256, 0, s>>>(key.p, sd.p, m, c->u1.p);
  SHCI_LAUNCH_CHECK();
  const uint32_t nu = exclusive_scan_u32(c->u1.p, c->u2.p, m, s, c->sort);
  if (vals && n_vals > 0) {
    DevBuf<uint32_t> starts;
    starts.mt = &c->mem;
    starts.resize(nu ? nu : 1);
    k_seg_starts<<<grid_for(m, 256), 256, 0, s>>>(c->u1.p, c->u2.p, m, starts.p);
    SHCI_LAUNCH_CHECK();
    DevBuf<double> sums;
    sums.mt = &c->mem;
    sums.resize(nu ? nu : 1);
    for (int v = 0; v < n_vals; v++) {
      k_segsum<<<grid_for(nu, 256), 256, 0, s>>>(starts.p, nu, m, c->u0.p, vals[v].p, sums.p);
      SHCI_LAUNCH_CHECK();
      SHCI_CUDA(cudaMemcpyAsync(vals[v].p, sums.p, nu * 8, cudaMemcpyDeviceToDevice, s));
    }
    SHCI_CUDA(cudaStreamSynchronize(s));
    c->launches += 1 + n_vals;
  }
  k_compact2<<<grid_for(m, 256), 256, 0, s>>>(key.p, sd.p, c->u1.p, c->u2.p, m, a.p, b.p);
  SHCI_LAUNCH_CHECK();
  c->launches += 8;
  return nu;
}

namespace {
__global__ void k_compact_vals(const double* v, const uint32_t* flags, const uint32_t* pos,
                               size_t n, double* ov) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    if (flags[i]) ov[pos[i]] = v[i];
}
}  // namespace

// Appends the entries of (a, b[, v columns]) whose a != kInvalid to (oa, ob[, ov columns])
// after *n_out (growing them); *n_out is advanced by the number appended.
void compact_valid(shci_ctx* c, const uint64_t* a, const uint64_t* b, const double* const* v,
                   int n_vals, size_t m, DevBuf<uint64_t>& oa, DevBuf<uint64_t>& ob,
                   DevBuf<double>* ov, size_t* n_out) {
  if (m == 0) return;
  cudaStream_t s = c->stream;
  c->u1.reserve(m, 1.25);
  c->u2.reserve(m, 1.25);
  k_valid_flags<<<grid_for(m, 256), 256, 0, s>>>(a, m, c->u1.p);
  SHCI_LAUNCH_CHECK();
  const uint32_t nv = exclusive_scan_u32(c->u1.p, c->u2.p, m, s, c->sort);
  c->launches += 3;
  if (!nv) return;
  const size_t at = *n_out;
  oa.n = ob.n = at;
  oa.grow_keep(at + nv, s);
  ob.grow_keep(at + nv, s);
  k_compact2<<<grid_for(m, 256), 256, 0, s>>>(a, b, c->u1.p, c->u2.p, m, oa.p + at, ob.p + at);
  SHCI_LAUNCH_CHECK();
  for (int k = 0; k < n_vals && ov; k++) {
    ov[k].n = at;
    ov[k].grow_keep(at + nv, s);
    k_compact_vals<<<grid_for(m, 256), 256, 0, s>>>(v[k], c->u1.p, c->u2.p, m, ov[k].p + at);
    SHCI_LAUNCH_CHECK();
  }
  *n_out = at + nv;
}

// Sorted copy of the whole det list, the membership set used by selection and PT2.
// Inserts det ids into the variational hash set (slot = fingerprint << 32 | id + 1, linear
// probing; the table is at most half full, so every insertion finds an empty slot).
__global__ void k_hash_insert(const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn,
                              size_t n, unsigned long long* table, uint64_t mask) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint64_t h = set_slot_hash(up[i], dn[i]);
    const unsigned long long v = ((h >> 32) << 32) | (static_cast<unsigned long long>(i) + 1ull);
    uint64_t p = h & mask;
    for (uint64_t probe = 0; probe <= mask; probe++) {
      if (atomicCAS(&table[p], 0ull, v) == 0ull) break;
      p = (p + 1) & mask;
    }
  }
}

void rebuild_det_set(shci_ctx* c) {
  const size_t n = c->up.size();
  cudaStream_t s = c->stream;
  c->set_up.mt = c->set_dn.mt = &c->mem;
  c->set_up.resize(n, 1.25);
  c->set_dn.resize(n, 1.25);
  SHCI_CUDA(cudaMemcpyAsync(c->set_up.p, c->d_up.p, n * 8, cudaMemcpyDeviceToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(c->set_dn.p, c->d_dn.p, n * 8, cudaMemcpyDeviceToDevice, s));
  const size_t nu = sort_unique_pairs(c, c->set_up, c->set_dn, n);
  if (nu != n) throw ArgError("the det list contains duplicates");
  // hash set over the det list: a power of two >= 2n slots
  size_t slots = 1024;
  while (slots < 2 * n) slots <<= 1;
  c->set_hash.mt = &c->mem;
  c->set_hash.resize(slots, 1.0);
  c->set_hash_mask = slots - 1;
  SHCI_CUDA(cudaMemsetAsync(c->set_hash.p, 0, slots * 8, s));
  k_hash_insert<<<grid_for(n, 256), 256, 0, s>>>(c->d_up.p, c->d_dn.p, n, c->set_hash.p,
                                                 c->set_hash_mask);
  SHCI_LAUNCH_CHECK();
  c->launches += 1;
}

size_t select_dets(shci_ctx* c, double eps_var, bool var_sd) {
  if (!c->Q.built) throw ArgError("heat-bath queues not built (call shci_build_queues)");
  sync_dets(c);
  cudaStream_t s = c->stream;
  const size_t n_dets = c->up.size();
  const int n = c->I.n;
  const int n_elecs = static_cast<int>(c->I.n_up + c->I.n_dn);
  // eps_tried_prev grows with INF for new dets (solver.h:431)
  c->eps_tried.resize(n_dets, 1.0e100);
  DevBuf<double> d_eps;
  d_eps.mt = &c->mem;
  d_eps.resize(n_dets);
  SHCI_CUDA(cudaMemcpyAsync(d_eps.p, c->eps_tried.data(), n_dets * 8, cudaMemcpyHostToDevice, s));
  std::vector<uint32_t> pairs;
  for (int a = 0; a < n_elecs; a++)
    for (int b = a + 1; b < n_elecs; b++) pairs.push_back(a | (b << 16));
  DevBuf<uint32_t> d_pairs;
  d_pairs.mt = &c->mem;
  d_pairs.resize(pairs.empty() ? 1 : pairs.size());
  if (!pairs.empty())
    SHCI_CUDA(cudaMemcpyAsync(d_pairs.p, pairs.data(), pairs.size() * 4, cudaMemcpyHostToDevice, s));
  rebuild_det_set(c);

  SelParams P{};
  P.I = c->dI;
  P.coef = c->d_coef.p;
  P.eps_tried = d_eps.p;
  P.d_off = c->Q.d_off.p;
  P.d_H = c->Q.d_H.p;
  P.d_rs = c->Q.d_rs.p;
  P.s_off = c->Q.s_off.p;
  P.s_S = c->Q.s_S.p;
  P.s_r = c->Q.s_r.p;
  P.pair_tab = d_pairs.p;
  P.eps_var = eps_var;
  P.max_hci = c->Q.max_hci;
  P.max_singles = c->Q.max_singles;
  P.n_orbs = n;
  P.n_up = static_cast<int>(c->I.n_up);
  P.n_elecs = n_elecs;
  P.n_pairs = static_cast<int>(pairs.size());
  P.var_sd = var_sd ? 1 : 0;
  P.n_src_total = static_cast<uint32_t>(n_dets);
  P.rej_on = c->second_rejection ? 1 : 0;
  P.rej_factor = c->second_rejection_factor;
  P.time_sym = c->time_sym ? 1 : 0;
  P.no_doubles = c->has_doubles ? 0 : 1;
  P.inactive = c->inactive_orbs;
  P.e_hf_1b = 0.0;
  if (c->second_rejection) {
    // ChemSystem::get_e_hf_1b (chem_system.cc:812-823) on dets[0]: alpha, then beta (doubled
    // alpha under time_sym)
    for (uint64_t m = c->up[0]; m; m &= m - 1) P.e_hf_1b += c->I.h(__builtin_ctzll(m), __builtin_ctzll(m));
    if (c->time_sym) {
      P.e_hf_1b *= 2.;
    } else {
      for (uint64_t m = c->dn[0]; m; m &= m - 1)
        P.e_hf_1b += c->I.h(__builtin_ctzll(m), __builtin_ctzll(m));
    }
  }

  // several states: the sources' thresholds use the largest |c| over the states
  DevBuf<double> d_selc;
  if (c->n_states > 1) {
    d_selc.mt = &c->mem;
    d_selc.resize(n_dets);
    StatePtrs xs{};
    for (unsigned k = 1; k < c->n_states; k++) xs.p[k - 1] = c->d_xcoef[k - 1].p;
    k_max_coef<<<grid_for(n_dets, 256), 256, 0, s>>>(c->d_coef.p, xs,
                                                     static_cast<int>(c->n_states - 1), n_dets,
                                                     d_selc.p);
    SHCI_LAUNCH_CHECK();
    c->launches += 1;
  }
  int sms = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const unsigned grid = static_cast<unsigned>(sms) * 8u;
  const uint64_t kCap = 1ull << 27;  // candidates per chunk
  size_t n_new_total = 0;
  DevBuf<uint64_t> cnt, pass_up, pass_dn, cu, cd;
  DevBuf<double> epsm, rejm;
  cnt.mt = pass_up.mt = pass_dn.mt = cu.mt = cd.mt = &c->mem;
  epsm.mt = rejm.mt = &c->mem;
  for (uint32_t pass = 0; pass < 5; pass++) {
    P.pass = pass;
    P.up = c->d_up.p;
    P.dn = c->d_dn.p;
    P.coef = c->n_states > 1 ? d_selc.p : c->d_coef.p;
    P.set_up = c->set_up.p;
    P.set_dn = c->set_dn.p;
    P.set_n = static_cast<uint32_t>(c->set_up.n);
    P.set_hash = c->set_hash.p;
    P.set_hash_mask = c->set_hash_mask;
    const uint32_t n_src = n_dets > pass ? static_cast<uint32_t>((n_dets - pass + 4) / 5) : 0;
    size_t pass_n = 0;
    pass_up.n = pass_dn.n = 0;
    if (n_src) {
      cnt.resize(n_src + 1, 1.25);
      epsm.resize(n_src, 1.25);
      if (P.rej_on) {
        rejm.resize(n_src, 1.25);
        SHCI_CUDA(cudaMemsetAsync(rejm.p, 0, n_src * 8, s));
      }
      k_sel_count<<<grid, kSelWarps * 32, 0, s>>>(P, 0, n_src, cnt.p, epsm.p);
      SHCI_LAUNCH_CHECK();
      std::vector<uint64_t> hc(n_src);
      SHCI_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, n_src * 8, cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
      // chunk the sources so each chunk emits at most kCap candidates
      uint32_t k0 = 0;
      while (k0 < n_src) {
        uint64_t tot = 0;
        uint32_t k1 = k0;
        while (k1 < n_src && (k1 == k0 || tot + hc[k1] <= kCap)) tot += hc[k1++];
        if (tot > 0) {
          std::vector<uint64_t> off(k1 - k0);
          uint64_t acc = 0;
          for (uint32_t k = k0; k < k1; k++) {
            off[k - k0] = acc;
            acc += hc[k];
          }
          DevBuf<uint64_t> d_off;
          d_off.mt = &c->mem;
          d_off.resize(off.size());
          SHCI_CUDA(cudaMemcpyAsync(d_off.p, off.data(), off.size() * 8, cudaMemcpyHostToDevice, s));
          cu.resize(tot, 1.25);
          cd.resize(tot, 1.25);
          {
            ProfScope ps(c->prof, s, "select_emit");
            k_sel_emit<<<grid, kSelWarps * 32, 0, s>>>(P, k0, k1, d_off.p, epsm.p + k0, cu.p, cd.p,
                                                       P.rej_on ? rejm.p + k0 : nullptr);
            SHCI_LAUNCH_CHECK();
          }
          // compact valid candidates, then sort + unique
          const size_t before = pass_n;
          compact_valid(c, cu.p, cd.p, nullptr, 0, tot, pass_up, pass_dn, nullptr, &pass_n);
          if (pass_n > before) {
            pass_n = sort_unique_pairs(c, pass_up, pass_dn, pass_n);
            pass_up.n = pass_dn.n = pass_n;
          }
          c->launches += 1;
        }
        k0 = k1;
      }
      k_sel_mark<<<grid_for(n_src, 256), 256, 0, s>>>(P, 0, n_src, epsm.p,
                                                      P.rej_on ? rejm.p : nullptr);
      SHCI_LAUNCH_CHECK();
      c->launches += 2;
    }
    if (pass_n) {
      // append this pass's new dets (ascending Det order) to the det list
      const size_t old = c->up.size();
      c->up.resize(old + pass_n);
      c->dn.resize(old + pass_n);
      c->coefs.resize(old + pass_n, 1e-16);
      SHCI_CUDA(cudaMemcpyAsync(c->up.data() + old, pass_up.p, pass_n * 8, cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaMemcpyAsync(c->dn.data() + old, pass_dn.p, pass_n * 8, cudaMemcpyDeviceToHost, s));
      c->d_up.grow_keep(old + pass_n, s);
      c->d_dn.grow_keep(old + pass_n, s);
      c->d_coef.grow_keep(old + pass_n, s);
      SHCI_CUDA(cudaMemcpyAsync(c->d_up.p + old, pass_up.p, pass_n * 8, cudaMemcpyDeviceToDevice, s));
      SHCI_CUDA(cudaMemcpyAsync(c->d_dn.p + old, pass_dn.p, pass_n * 8, cudaMemcpyDeviceToDevice, s));
      k_fill_coef<<<grid_for(pass_n, 256), 256, 0, s>>>(c->d_coef.p, old, old + pass_n, 1e-16);
      SHCI_LAUNCH_CHECK();
      // states 1..: 1e-16, except that while the list is small (<= 50 dets when this step
      // began) det k starts as state k's unit vector (solver.h:479-486)
      for (unsigned k = 1; k < c->n_states; k++) {
        auto& xc = c->d_xcoef[k - 1];
        xc.grow_keep(old + pass_n, s);
        k_fill_coef<<<grid_for(pass_n, 256), 256, 0, s>>>(xc.p, old, old + pass_n, 1e-16);
        SHCI_LAUNCH_CHECK();
        if (n_dets <= 50 && k >= old && k < old + pass_n)
          k_fill_coef<<<1, 32, 0, s>>>(xc.p, k, k + 1, 1.0);
      }
      SHCI_CUDA(cudaStreamSynchronize(s));
      n_new_total += pass_n;
      // the new dets join the membership set before the next pass
      rebuild_det_set(c);
    }
  }
  // eps_tried_prev back to the host mirror (only the sources of this step changed)
  SHCI_CUDA(cudaMemcpyAsync(c->eps_tried.data(), d_eps.p, n_dets * 8, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->eps_tried.resize(c->up.size(), 1.0e100);
  c->prof.flush();
  return n_new_total;
}

}  // namespace shci

// Heat-bath candidate generation shared by selection (select.cu) and PT2 (pt2.cu).
//
// The reference's ChemSystem::find_connected_dets (src/chem/chem_system.cc:289-402) walks
// singles_queue[p] and hci_queue[pq] (sorted by descending |H|) until the first entry below
// eps_min, skipping doubles with |H| >= eps_max.  The same queues sit in HBM in CSR form and
// a binary search gives each (det, slot) its exact entry range.  A det has n_elecs "single"
// slots (one per electron) and n_elecs (n_elecs - 1) / 2 "double" slots (one per electron
// pair, in the reference's p_id < q_id order).
#pragma once

#include "common.cuh"

namespace shci {

constexpr int kSelWarps = 8;
constexpr uint64_t kInvalid = ~0ull;

struct SelParams {
  DevIntegrals I;
  const uint64_t* up;
  const uint64_t* dn;
  const double* coef;
  double* eps_tried;
  const uint64_t* d_off;
  const double* d_H;
  const uint32_t* d_rs;
  const uint32_t* s_off;
  const double* s_S;
  const uint32_t* s_r;
  const uint32_t* pair_tab;  // pair k -> p_id | q_id << 16
  const uint64_t* set_up;    // sorted variational set
  const uint64_t* set_dn;
  uint32_t set_n;
  const unsigned long long* set_hash;  // hash set of the variational dets (see in_set)
  uint64_t set_hash_mask;
  double eps_var;
  double max_hci, max_singles;
  int n_orbs, n_up, n_elecs, n_pairs;
  int var_sd;
  uint32_t pass, n_src_total;  // sources are i = pass + 5 k, i < n_src_total
  // second rejection (chem_system.cc:300-308, 318-324, 364-370): off unless rej_on
  int rej_on;
  double rej_factor;  // second_rejection_factor
  double e_hf_1b;     // sum of h_pp over the HF det's electrons (chem_system.cc:812-823)
  int time_sym;       // time-reversal symmetry: list holds up <= dn, open dets stand for pairs
  // find_connected_dets options: no double excitations (has_double_excitation false,
  // chem_system.cc:345) and orbitals that may not be targets (the active space,
  // chem_system.cc:327-329, 383-387); 0 and 0 are the reference's defaults
  int no_doubles;
  uint64_t inactive;
};

constexpr double kSqrt2 = 1.4142135623730951;  // Util::SQRT2 (src/util.h:58)

__device__ __forceinline__ int nth_bit(uint64_t x, int k) {
  const unsigned lo = static_cast<unsigned>(x), hi = static_cast<unsigned>(x >> 32);
  const int cl = __popc(lo);
  if (k < cl) return __fns(lo, 0, k + 1);
  return 32 + __fns(hi, 0, k - cl + 1);
}

// spin-orbital index of electron e (up electrons first, then dn + n)
__device__ __forceinline__ int elec_orb(uint64_t up, uint64_t dn, int e, int n_up, int n) {
  return e < n_up ? nth_bit(up, e) : nth_bit(dn, e - n_up) + n;
}

// First k in [lo, hi) with a[k] < x, for a descending array of non-negative values and
// any x.  Non-negative doubles order like the integers of their bit patterns (a negative or
// NaN x compares false against every entry, as in FP64), so the comparisons run on the
// integer pipe (the FP64 pipe is slow on GB300) with the same result.
__device__ __forceinline__ uint32_t first_below(const double* a, uint32_t lo, uint32_t hi,
                                                double x) {
  long long xb = __double_as_longlong(x);
  if ((xb & 0x7fffffffffffffffll) > 0x7ff0000000000000ll) xb = -1;  // NaN: never above an entry
  const long long* ab = reinterpret_cast<const long long*>(a);
  // the usual cases: the window starts at the slot's largest entry or is empty
  if (lo < hi && ab[lo] < xb) return lo;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (ab[mid] < xb) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

__device__ __forceinline__ size_t c2(size_t a, size_t b) {
  return a > b ? (a * (a + 1)) / 2 + b : (b * (b + 1)) / 2 + a;
}

// Entry range [lo, lo + cnt) of slot `slot` for the det (eps window [eps_min, eps_max)).
// *orbs (optional) receives the slot's electron orbitals for make_candidate_at: the moved
// orbital of a single, or the two spin-orbitals p | q << 8 of a pair.
__device__ __forceinline__ void slot_range(const SelParams& P, uint64_t up, uint64_t dn, int slot,
                                           double eps_min, double eps_max, uint32_t* lo,
                                           uint32_t* cnt, uint32_t* orbs = nullptr) {
  *lo = 0;
  *cnt = 0;
  const int n = P.n_orbs;
  if (slot < P.n_elecs) {
    if (eps_min > P.max_singles) return;
    const int p = slot < P.n_up ? nth_bit(up, slot) : nth_bit(dn, slot - P.n_up);
    if (orbs) *orbs = static_cast<uint32_t>(p);
    const uint32_t a = P.s_off[p], b = P.s_off[p + 1];
    *lo = a;
    *cnt = first_below(P.s_S, a, b, eps_min) - a;
    return;
  }
  if (P.no_doubles || eps_min > P.max_hci) return;
  const uint32_t pr = P.pair_tab[slot - P.n_elecs];
  const int p = elec_orb(up, dn, pr & 0xffff, P.n_up, n);
  const int q = elec_orb(up, dn, pr >> 16, P.n_up, n);
  if (orbs) *orbs = static_cast<uint32_t>(p) | (static_cast<uint32_t>(q) << 8);
  int p2 = p, q2 = q;
  if (p >= n && q >= n) {
    p2 -= n;
    q2 -= n;
  } else if (p < n && q >= n && p > q - n) {
    p2 = q - n;
    q2 = p + n;
  }
  const size_t pq = c2(p2, q2);
  const uint32_t a = static_cast<uint32_t>(P.d_off[pq]), b = static_cast<uint32_t>(P.d_off[pq + 1]);
  const uint32_t s = first_below(P.d_H, a, b, eps_max);
  const uint32_t e = first_below(P.d_H, s, b, eps_min);
  *lo = s;
  *cnt = e - s;
}

// Slot hash of a det for the variational hash set (this set is internal: no other hash has
// to agree with it): the strings combined by one multiply, then a multiply-xorshift finaliser
// so that the low bits index the table and the high bits fingerprint.  About a dozen integer
// instructions, against about seventy for the reference's det hash plus a finaliser; every
// PT2 candidate and selection candidate pays it.
__host__ __device__ __forceinline__ uint64_t set_slot_hash(uint64_t u, uint64_t d) {
  uint64_t h = u * 0x9E3779B97F4A7C15ull + d;
  h ^= h >> 32;
  h *= 0xD6E8FEB86659FD93ull;
  h ^= h >> 29;
  return h;
}

// Is (u, d) a variational det?  With the hash set (slots hold fingerprint << 32 | det id + 1,
// linear probing, at most half full) one or two probes and a comparison against the det
// list; otherwise a binary search of the sorted set.
__device__ __forceinline__ bool in_set(const SelParams& P, uint64_t u, uint64_t d) {
  if (P.set_hash) {
    const uint64_t h = set_slot_hash(u, d);
    const uint32_t fp = static_cast<uint32_t>(h >> 32);
    uint64_t p = h & P.set_hash_mask;
    for (uint64_t probe = 0; probe <= P.set_hash_mask; probe++) {
      const unsigned long long v = P.set_hash[p];
      if (v == 0ull) return false;
      if (static_cast<uint32_t>(v >> 32) == fp) {
        const uint32_t id = static_cast<uint32_t>(v) - 1u;
        if (P.up[id] == u && P.dn[id] == d) return true;
      }
      p = (p + 1) & P.set_hash_mask;
    }
    return false;
  }
  uint32_t lo = 0, hi = P.set_n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const uint64_t su = P.set_up[mid], sd = P.set_dn[mid];
    if (su < u || (su == u && sd < d)) lo = mid + 1;
    else hi = mid;
  }
  return lo < P.set_n && P.set_up[lo] == u && P.set_dn[lo] == d;
}

__device__ __forceinline__ double src_eps_min(const SelParams& P, uint32_t i) {
  double e = P.eps_var / fabs(P.coef[i]);
  if (i == 0 && P.var_sd) e = 0.0;
  if (P.time_sym && P.up[i] != P.dn[i]) e *= kSqrt2;  // solver.h:447
  return e;
}


// Candidate det for entry e of slot `slot` of det (up, dn).  Returns false when the target
// orbitals are occupied (the reference's occupancy checks).  *single tells the slot kind.
__device__ __forceinline__ bool make_candidate(const SelParams& P, uint64_t up, uint64_t dn,
                                               int slot, uint32_t e, uint64_t* cu,
                                               uint64_t* cd, bool* single) {
  const int n = P.n_orbs;
  *cu = up;
  *cd = dn;
  if (slot < P.n_elecs) {
    *single = true;
    const bool is_up = slot < P.n_up;
    const int p = is_up ? nth_bit(up, slot) : nth_bit(dn, slot - P.n_up);
    const int r = static_cast<int>(P.s_r[e]);
    // an inactive target (active space) fails like an occupied one
    if (is_up) {
      if ((up | P.inactive) >> r & 1) return false;
      *cu = (up & ~(1ull << p)) | (1ull << r);
    } else {
      if ((dn | P.inactive) >> r & 1) return false;
      *cd = (dn & ~(1ull << p)) | (1ull << r);
    }
    return true;
  }
  *single = false;
  const uint32_t pr = P.pair_tab[slot - P.n_elecs];
  const int p = elec_orb(up, dn, pr & 0xffff, P.n_up, n);
  const int q = elec_orb(up, dn, pr >> 16, P.n_up, n);
  const uint32_t rs = P.d_rs[e];
  int r = rs & 0xffff, s = rs >> 16;
  if (p >= n && q >= n) {
    r += n;
    s += n;
  } else if (p < n && q >= n && p > q - n) {
    const int tmp = s - n;
    s = r + n;
    r = tmp;
  }
  // an inactive target (active space) fails like an occupied one
  const uint64_t bu = up | P.inactive, bd = dn | P.inactive;
  const bool occ_r = r < n ? (bu >> r & 1) : (bd >> (r - n) & 1);
  if (occ_r) return false;
  const bool occ_s = s < n ? (bu >> s & 1) : (bd >> (s - n) & 1);
  if (occ_s) return false;
  uint64_t u = up, d = dn;
  if (p < n) u &= ~(1ull << p); else d &= ~(1ull << (p - n));
  if (q < n) u &= ~(1ull << q); else d &= ~(1ull << (q - n));
  if (r < n) u |= 1ull << r; else d |= 1ull << (r - n);
  if (s < n) u |= 1ull << s; else d |= 1ull << (s - n);
  *cu = u;
  *cd = d;
  return true;
}

// make_candidate with the slot's electron orbitals already known (from slot_range).
__device__ __forceinline__ bool make_candidate_at(const SelParams& P, uint64_t up, uint64_t dn,
                                                  int slot, uint32_t orbs, uint32_t e,
                                                  uint64_t* cu, uint64_t* cd) {
  const int n = P.n_orbs;
  *cu = up;
  *cd = dn;
  if (slot < P.n_elecs) {
    const int p = static_cast<int>(orbs);
    const int r = static_cast<int>(P.s_r[e]);
    // an inactive target (active space) fails like an occupied one
    if (slot < P.n_up) {
      if ((up | P.inactive) >> r & 1) return false;
      *cu = (up & ~(1ull << p)) | (1ull << r);
    } else {
      if ((dn | P.inactive) >> r & 1) return false;
      *cd = (dn & ~(1ull << p)) | (1ull << r);
    }
    return true;
  }
  const int p = static_cast<int>(orbs & 0xffu), q = static_cast<int>(orbs >> 8);
  const uint32_t rs = P.d_rs[e];
  int r = rs & 0xffff, s = rs >> 16;
  if (p >= n && q >= n) {
    r += n;
    s += n;
  } else if (p < n && q >= n && p > q - n) {
    const int tmp = s - n;
    s = r + n;
    r = tmp;
  }
  // an inactive target (active space) fails like an occupied one
  const uint64_t bu = up | P.inactive, bd = dn | P.inactive;
  const bool occ_r = r < n ? (bu >> r & 1) : (bd >> (r - n) & 1);
  if (occ_r) return false;
  const bool occ_s = s < n ? (bu >> s & 1) : (bd >> (s - n) & 1);
  if (occ_s) return false;
  uint64_t u = up, d = dn;
  if (p < n) u &= ~(1ull << p); else d &= ~(1ull << (p - n));
  if (q < n) u &= ~(1ull << q); else d &= ~(1ull << (q - n));
  if (r < n) u |= 1ull << r; else d |= 1ull << (r - n);
  if (s < n) u |= 1ull << s; else d |= 1ull << (s - n);
  *cu = u;
  *cd = d;
  return true;
}

// Walks the candidates of one source det (a warp): the heat-bath slots' index ranges in the
// window [eps_min, eps_max) are flattened over the lanes 32 at a time, and f(slot, ok, cu,
// cd) is called by all lanes for each group of 32 (slot = the lane holds an index entry of
// the window, ok = that entry makes a valid candidate (cu, cd)).
template <class F>
__device__ __forceinline__ void pt_walk(const SelParams& P, uint64_t up, uint64_t dn,
                                        double eps_min, double eps_max, F&& f) {
  const unsigned lane = threadIdx.x & 31;
  const int n_slots = P.n_elecs + P.n_pairs;
  for (int s0 = 0; s0 < n_slots; s0 += 32) {
    const int slot = s0 + lane;
    uint32_t lo = 0, c = 0, orbs = 0;
    if (slot < n_slots) slot_range(P, up, dn, slot, eps_min, eps_max, &lo, &c, &orbs);
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
      const uint32_t o_orbs = __shfl_sync(kFull, orbs, ol);
      uint64_t cu = 0, cd = 0;
      bool ok = false;
      if (t < total) {
        const uint32_t e = o_lo + (t - (o_inc - o_c));
        ok = make_candidate_at(P, up, dn, s0 + (int)ol, o_orbs, e, &cu, &cd);
      }
      f(t < total, ok, cu, cd);
    }
  }
}

}  // namespace shci

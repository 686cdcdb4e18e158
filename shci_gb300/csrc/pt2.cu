// Epstein-Nesbet PT2 on the device: deterministic, pseudo-stochastic and stochastic stages
// (K6 in PT mode + K7).
//
// Reference: Solver<S>::get_energy_pt_dtm / _psto / _sto (src/solver/solver.h:636-1153) and
// mapreduce_sum (:1155-1177).  Each stage visits source dets i (all var dets, or a stochastic
// sample) and emits the connected dets a in the heat-bath window [eps / |c_i|, INF) that fall
// in the current hash batch (rehash(DetHasher(a)) % n_batches), are not variational and have
// |H_ai c_i| >= eps.  The reference accumulates (a -> sum) in a distributed hash map; here
// the (a, values) pairs are compacted, radix-sorted by det and reduced by key in a fixed
// order, and a second kernel forms each unique a's contribution with its diagonal H_aa.
//   dtm : value  = H_ai c_i                          contribution S0^2 / (E - H_aa)
//   psto: values = [hc, hc if |hc| >= eps_dtm]      contribution (S0^2 - S1^2) / (E - H_aa)
//   sto : values = the five sums of solver.h:1093-1103, contribution of :1117-1124
// Stochastic iterations are independent: the host draws every iteration's sample with the
// reference's generator and distributions (std::default_random_engine, alias tables of
// src/util.cc:128-175), a chunk of iterations is processed in one device pass with the
// iteration index stored above the orbital bits of the key, and the reference's stopping
// rules are then applied iteration by iteration.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <numeric>
#include <queue>
#include <random>
#include <future>
#include <stack>
#include <thread>
#include <unordered_map>

#include "ctx.h"
#include "heatbath.cuh"
#include "kernels.h"

namespace shci {

namespace {

constexpr int kPtWarps = 8;  // 8 warps per CTA; the walks are capped at 64 registers for
                              // four CTAs per SM (PT2 1.29 -> 1.26 s at n = 40)
enum : int { kDtm = 0, kPsto = 1, kSto = 2 };

struct PtParams {
  double eps;        // emission threshold |H_ai c_i| >= eps (and window eps / |c_i|)
  double eps_dtm;    // psto: second column threshold
  double eps_psto;   // sto: column split threshold
  uint64_t n_batches;
  uint64_t batch_magic;  // floor((2^64 - 1) / n_batches) for batch_of (set by set_batches)
  uint64_t batch;    // dtm / psto: the batch being computed
  double factor;     // sto: 1 / (n_samples - n_dtm - 1)
  int iter_shift;    // sto: bit position of the iteration index in the emitted up key
  int pilot;         // sto: sample-size pilot (only single excitations face the |H c| test)
};

// Stochastic sources: entry e = (det, iteration, count, weight, batch, deterministic?).  With
// ent_off, source m groups the entries [ent_off[m], ent_off[m+1]) of one det (its draws in the
// iterations of one device pass): the det's window is walked and each candidate hashed once,
// then tested against every entry's batch.  Without it, source m is entry m.
struct StoSources {
  const uint32_t* det;
  const uint32_t* iter;
  const double* count;
  const double* weight;
  const uint32_t* batch;
  const uint8_t* is_dtm;
  const uint32_t* remap;    // optional: launch source k' is source remap[k'] (re-runs)
  const uint32_t* ent_off;  // optional: entries of each source
};

__device__ __forceinline__ uint32_t src_index(const StoSources& S, uint32_t k) {
  return S.remap ? S.remap[k] : k;
}

__device__ __forceinline__ uint32_t ent_begin(const StoSources& S, uint32_t k) {
  return S.ent_off ? S.ent_off[k] : k;
}
__device__ __forceinline__ uint32_t ent_end(const StoSources& S, uint32_t k) {
  return S.ent_off ? S.ent_off[k + 1] : k + 1;
}

__device__ __forceinline__ uint32_t src_det(const StoSources& S, uint32_t k, int mode) {
  return mode == kSto ? S.det[ent_begin(S, k)] : k;
}

// h % n_batches exactly, without a 64-bit division: a mask for powers of two, else the
// quotient estimate floor(h * magic / 2^64) with magic = floor((2^64 - 1) / n_batches), which
// is at most 2 below the true quotient, corrected by subtraction.
__device__ __forceinline__ uint64_t batch_of(const PtParams& Q, uint64_t h) {
  const uint64_t nb = Q.n_batches;
  if ((nb & (nb - 1)) == 0) return h & (nb - 1);
  uint64_t r = h - __umul64hi(h, Q.batch_magic) * nb;
  if (r >= nb) r -= nb;
  if (r >= nb) r -= nb;
  return r;
}

// Candidate a of source i belongs to the batch being computed (the first test of the
// handler, solver.h:703-705: rehash(DetHasher(a)) % n_batches).  One batch: every candidate.
__device__ __forceinline__ bool in_batch(const PtParams& Q, uint64_t batch, uint64_t cu,
                                         uint64_t cd) {
  return Q.n_batches <= 1 || batch_of(Q, rehash(det_hash(cu, cd))) == batch;
}

void set_batches(PtParams& Q, uint64_t n_batches) {
  Q.n_batches = n_batches;
  Q.batch_magic = n_batches ? ~0ull / n_batches : 0;
}

__device__ __forceinline__ uint64_t src_batch(const PtParams& Q, const StoSources& S, uint32_t k,
                                              int mode) {
  return mode == kSto ? S.batch[k] : Q.batch;
}

// Output slots of each source: its candidates in the current batch.
template <int MODE>
__global__ void __launch_bounds__(kPtWarps * 32, 4)
    k_pt_count(SelParams P, PtParams Q, StoSources S, uint32_t n_src, uint64_t* cnt_out) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t wpg = gridDim.x * kPtWarps;
  for (uint32_t k = blockIdx.x * kPtWarps + (threadIdx.x >> 5); k < n_src; k += wpg) {
    const uint32_t kk = src_index(S, k);
    const uint32_t i = src_det(S, kk, MODE);
    const double ac = fabs(P.coef[i]);
    const double eps_min = Q.eps / ac;
    const double eps_max = 1.0e100 / ac;
    const uint64_t up = P.up[i], dn = P.dn[i];
    uint64_t tot = 0;
    if (Q.n_batches <= 1) {
      // every candidate counts: the slot ranges suffice
      const int n_slots = P.n_elecs + P.n_pairs;
      for (int s0 = 0; s0 < n_slots; s0 += 32) {
        uint32_t lo = 0, c = 0;
        if (s0 + (int)lane < n_slots) slot_range(P, up, dn, s0 + lane, eps_min, eps_max, &lo, &c);
        uint64_t cc = c;
#pragma unroll
        for (int o = 16; o; o >>= 1) cc += __shfl_xor_sync(kFull, cc, o);
        tot += cc;
      }
    } else if (MODE == kSto) {
      // every entry of the source whose batch the candidate falls in
      const uint32_t e0 = ent_begin(S, kk), e1 = ent_end(S, kk);
      pt_walk(P, up, dn, eps_min, eps_max, [&](bool, bool ok, uint64_t cu, uint64_t cd) {
        const uint64_t b = ok ? batch_of(Q, rehash(det_hash(cu, cd))) : ~0ull;
        uint32_t m = 0;
        for (uint32_t e = e0; e < e1; e++) m += b == S.batch[e] ? 1u : 0u;
        tot += __reduce_add_sync(kFull, m);
      });
    } else {
      const uint64_t batch = src_batch(Q, S, kk, MODE);
      pt_walk(P, up, dn, eps_min, eps_max, [&](bool, bool ok, uint64_t cu, uint64_t cd) {
        tot += __popc(__ballot_sync(kFull, ok && in_batch(Q, batch, cu, cd)));
      });
    }
    if (lane == 0) cnt_out[k] = tot;
  }
}

struct OutCols {
  double* v[5];
};

// Single-excitation elements in 64-bit fixed point.  H_ij of a single excitation p -> q is
// +-(h_pq + sum_o (pq|oo) [2 (pq|oo) for a doubly occupied o] - sum_o (po|oq)), about 2 n_e
// table entries (chem_system.cc:544-577); in FP64 that chain of dependent additions kept
// the FP64 pipe (about two operations per SM cycle on GB300) half busy in the emission.  Here
// every entry is rounded once to a multiple of 2^-s and the sum is exact on the integer pipe;
// |fixed - FP64| <= margin (entry rounding plus the FP64 evaluation's own rounding).  A
// value within margin |c_i| of a threshold is formed again in FP64, so every keep / split
// decision is the FP64 one; kept values differ from it by at most margin |c_i|.
struct SingleFix {
  const long long* h1;  // [n*n]
  const long long* d;   // [n^3] (pq|oo) at (p n + q) n + o
  const long long* x;   // [n^3] (po|oq) at (p n + q) n + o
  int n;
  double inv_scale;     // 2^-s
  double margin;
};

__device__ __forceinline__ double h_one_fix(const SingleFix& F, uint64_t ui, uint64_t di,
                                            uint64_t uj, uint64_t dj) {
  const uint64_t xu = ui ^ uj;
  const bool alpha = xu != 0;
  const uint64_t si = alpha ? ui : di, sj = alpha ? uj : dj;
  uint64_t oppo = alpha ? di : ui;
  const uint64_t x = si ^ sj;
  const int oi = ctz64(si & x), oj = ctz64(sj & x);
  const int n = F.n;
  const size_t row = (size_t)(oi * n + oj) * n;
  const long long* D = F.d + row;
  const long long* X = F.x + row;
  long long e = __ldg(F.h1 + oi * n + oj);
  for (uint64_t m = si & ~(1ull << oi) & ~(1ull << oj); m; m &= m - 1) {
    const int o = ctz64(m);
    e -= __ldg(X + o);
    const long long dd = __ldg(D + o);
    if (oppo >> o & 1) {
      oppo &= ~(1ull << o);
      e += 2 * dd;
    } else {
      e += dd;
    }
  }
  for (uint64_t m = oppo; m; m &= m - 1) e += __ldg(D + ctz64(m));
  return flip_sign(static_cast<double>(e) * F.inv_scale, move_parity(si, oi, oj));
}

constexpr uint32_t kPtQ = 64;  // per-warp queue of batch members (< 32 waiting + 32 pushed)
struct PtQueue {
  uint64_t u[kPtQ];
  uint64_t d[kPtQ];
  uint64_t pos[kPtQ];  // output slot of the member
  uint32_t src[kPtQ];  // its source (launch-relative index k - k_begin)
  uint8_t ent[kPtQ];   // stochastic stage: its entry within the source
};

// Emits the batch members of each source into its region [off[k], off[k + 1]) (one batch:
// every index entry of the window, as counted by slot ranges).  A warp walks its sources one
// after the other; members wait in a per-warp queue that carries them across sources (with
// their source and output slot) and are finished 32 at a time (variational-set test,
// H_ai c_i, the value columns), so the set search and the FP64 element run with full warps
// even when most sources have only a few members.  Slots of members rejected there, of
// entries that make no valid candidate, and the unused tail of a region are written invalid.
// Members keep their walk order within their source's region.  A region may be sized by an
// estimate (several batches): when the members do not fit, the queue is drained, the whole
// region is written invalid and overflow[k] is set, and the caller emits that source again
// with an exact count.
template <int MODE>
__global__ void __launch_bounds__(kPtWarps * 32, 4)
    k_pt_emit(SelParams P, PtParams Q, StoSources S, SingleFix F, uint32_t k_begin,
              uint32_t k_end, const uint64_t* off, uint64_t* out_up, uint64_t* out_dn,
              OutCols out, uint8_t* overflow) {
  __shared__ PtQueue qs[kPtWarps];
  PtQueue& q = qs[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t wpg = gridDim.x * kPtWarps;
  uint32_t qh = 0, qn = 0;  // warp-uniform ring state, kept across sources
  auto drain = [&](uint32_t m) {
    __syncwarp();
    if (lane < m) {
      const uint32_t sl = (qh + lane) & (kPtQ - 1);
      const uint64_t cu = q.u[sl], cd = q.d[sl], pos = q.pos[sl];
      const uint32_t kk = src_index(S, k_begin + q.src[sl]);
      const uint32_t i = src_det(S, kk, MODE);
      const uint64_t up = P.up[i], dn = P.dn[i];
      const double coef = P.coef[i];
      double count = 1.0, weight = 1.0;
      bool dtm_src = true;
      uint64_t iter_tag = 0;
      if (MODE == kSto) {
        const uint32_t e = ent_begin(S, kk) + q.ent[sl];
        dtm_src = S.is_dtm[e] != 0;
        count = dtm_src ? 1.0 : S.count[e];
        weight = dtm_src ? 1.0 : S.weight[e];
        iter_tag = static_cast<uint64_t>(S.iter[e]) << Q.iter_shift;
      }
      // handler order of solver.h:703-713: batch (done), variational set, |H_ai c_i|
      bool ok = cu != kInvalid && !in_set(P, cu, cd);
      double hc = 0.0;
      // the pilot's handler tests |H_ai c_i| for single excitations only (solver.h:958-962)
      const bool test = MODE != kSto || !Q.pilot || popc64(up ^ cu) + popc64(dn ^ cd) == 2;
      if (ok && test) {
        if (popc64(up ^ cu) + popc64(dn ^ cd) == 2) {  // single excitation
          hc = h_one_fix(F, up, dn, cu, cd) * coef;
          const double a = fabs(hc), m = F.margin * fabs(coef);
          bool near = fabs(a - Q.eps) <= m;
          if (MODE == kPsto) near = near || fabs(a - Q.eps_dtm) <= m;
          if (MODE == kSto) near = near || fabs(a - Q.eps_psto) <= m;
          if (near) hc = h_one(P.I, up, dn, cu, cd) * coef;
        } else {
          hc = h_two(P.I, up, dn, cu, cd) * coef;
        }
        if (fabs(hc) < Q.eps) ok = false;
      }
      out_up[pos] = ok ? (cu | iter_tag) : kInvalid;
      out_dn[pos] = ok ? cd : kInvalid;
      if (MODE == kDtm) {
        out.v[0][pos] = hc;
      } else if (MODE == kPsto) {
        out.v[0][pos] = hc;
        out.v[1][pos] = fabs(hc) >= Q.eps_dtm ? hc : 0.0;
      } else {
        // solver.h:1093-1103
        const double x = count * hc / weight;
        const bool above = fabs(hc) > Q.eps_psto;
        double v2 = 0.0, v3 = 0.0, v4 = 0.0;
        if (!dtm_src) {
          v2 = count * hc / weight * sqrt(Q.factor);
          if (above) v3 = v2;
          else v4 = x * x * (1. - weight / count + Q.factor);
        }
        out.v[0][pos] = x;
        out.v[1][pos] = above ? x : 0.0;
        out.v[2][pos] = v2;
        out.v[3][pos] = v3;
        out.v[4][pos] = v4;
      }
    }
    __syncwarp();
    qh += m;
    qn -= m;
  };
  for (uint32_t k = k_begin + blockIdx.x * kPtWarps + (threadIdx.x >> 5); k < k_end; k += wpg) {
    const uint32_t kl = k - k_begin;
    const uint32_t kk = src_index(S, k);
    const uint32_t i = src_det(S, kk, MODE);
    const double ac = fabs(P.coef[i]);
    const double eps_min = Q.eps / ac;
    const double eps_max = 1.0e100 / ac;
    const uint64_t up = P.up[i], dn = P.dn[i];
    const uint64_t batch = MODE == kSto ? 0 : src_batch(Q, S, kk, MODE);
    const uint32_t e0 = MODE == kSto ? ent_begin(S, kk) : 0u;
    const uint32_t e1 = MODE == kSto ? ent_end(S, kk) : 1u;
    const uint64_t start = off[kl], limit = off[kl + 1];
    uint64_t cnt = 0;   // members of this source so far (warp-uniform)
    bool over = false;  // warp-uniform
    // queue the lanes with mine set (members of entry ent), each with its output slot
    auto push = [&](bool mine, bool ok, uint64_t cu, uint64_t cd, uint32_t ent) {
      const unsigned bal = __ballot_sync(kFull, mine);
      if (!bal) return;
      const uint32_t nb = __popc(bal);
      if (start + cnt + nb > limit) over = true;
      if (!over && mine) {
        const uint32_t sl = (qh + qn + __popc(bal & lt)) & (kPtQ - 1);
        q.u[sl] = ok ? cu : kInvalid;
        q.d[sl] = ok ? cd : kInvalid;
        q.pos[sl] = start + cnt + __popc(bal & lt);
        q.src[sl] = kl;
        q.ent[sl] = static_cast<uint8_t>(ent);
      }
      if (!over) qn += nb;
      cnt += nb;
      if (qn >= 32u) drain(32u);
    };
    pt_walk(P, up, dn, eps_min, eps_max, [&](bool slot, bool ok, uint64_t cu, uint64_t cd) {
      if (MODE == kSto) {
        // hash once, then one member per entry whose batch the candidate falls in
        const uint64_t b =
            (ok && Q.n_batches > 1) ? batch_of(Q, rehash(det_hash(cu, cd))) : 0ull;
        for (uint32_t e = e0; e < e1; e++)
          push(Q.n_batches <= 1 ? slot : (ok && b == S.batch[e]), ok, cu, cd, e - e0);
        return;
      }
      push(Q.n_batches <= 1 ? slot : (ok && in_batch(Q, batch, cu, cd)), ok, cu, cd, 0u);
    });
    if (over) {
      // members of this source may still wait in the queue: finish them, then void the region
      while (qn) drain(qn < 32u ? qn : 32u);
      for (uint64_t p = start + lane; p < limit; p += 32) out_up[p] = kInvalid;
      if (lane == 0) overflow[kl] = 1;
    } else {
      // the region's unused tail (the members' slots are below start + cnt)
      for (uint64_t p = start + cnt + lane; p < limit; p += 32) out_up[p] = kInvalid;
    }
  }
  while (qn) drain(qn < 32u ? qn : 32u);
}

// Diagonal H_aa of the PT dets in 64-bit fixed point.  The diagonal is a sum of about
// n_e^2 / 2 table entries (h_pp, J - K for same-spin pairs, J for opposite-spin pairs,
// chem_system.cc:495-542); on GB300 the FP64 pipe retires about two operations per SM cycle,
// so ~300 FP64 additions per PT det made the contribution kernel FP64-bound.  Here every
// entry is rounded once to a multiple of 2^-s (s chosen so that no sum can reach 2^62) and the
// sum is an exact integer sum on the integer pipe: |error| <= (number of terms) * 2^-(s+1),
// about 1e-13 Ha at n = 40 (s = 51), where the FP64 sum carries a comparable rounding error.
struct DiagFix {
  const long long* tab;  // [n] h_pp, [n*n] J - K, [n*n] J
  int n;
  double inv_scale;      // 2^-s
  double e_core;
};

__device__ __forceinline__ double h_diag_fix(const DiagFix& F, uint64_t up, uint64_t dn) {
  const int n = F.n;
  const long long* h1 = F.tab;
  const long long* jk = F.tab + n;
  const long long* jj = F.tab + n + n * n;
  long long acc = 0;
  for (uint64_t m = up; m; m &= m - 1) {
    const int a = ctz64(m);
    acc += __ldg(h1 + a);
    const long long* row = jk + a * n;
    for (uint64_t m2 = m & (m - 1); m2; m2 &= m2 - 1) acc += __ldg(row + ctz64(m2));
    const long long* row2 = jj + a * n;
    for (uint64_t m3 = dn; m3; m3 &= m3 - 1) acc += __ldg(row2 + ctz64(m3));
  }
  for (uint64_t m = dn; m; m &= m - 1) {
    const int a = ctz64(m);
    acc += __ldg(h1 + a);
    const long long* row = jk + a * n;
    for (uint64_t m2 = m & (m - 1); m2; m2 &= m2 - 1) acc += __ldg(row + ctz64(m2));
  }
  return static_cast<double>(acc) * F.inv_scale + F.e_core;
}

// x[k] = contribution of unique PT det k (mapper of solver.h:727-732, 856-862, 1117-1124)
template <int MODE>
__global__ void k_pt_x(DiagFix D, const uint64_t* au, const uint64_t* ad, OutCols S,
                       size_t m, double e_var, double n_batches, uint64_t orb_mask, double* x) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < m;
       k += (size_t)gridDim.x * blockDim.x) {
    const double haa = h_diag_fix(D, au[k] & orb_mask, ad[k]);
    double v;
    if (MODE == kDtm) {
      v = S.v[0][k] * S.v[0][k] / (e_var - haa);
    } else if (MODE == kPsto) {
      const double d = S.v[0][k] * S.v[0][k] - S.v[1][k] * S.v[1][k];
      v = d / (e_var - haa);
    } else {
      const double f = n_batches / (e_var - haa);
      v = (S.v[0][k] * S.v[0][k] - S.v[1][k] * S.v[1][k] + S.v[2][k] * S.v[2][k] -
           S.v[3][k] * S.v[3][k] - S.v[4][k]) * f;
    }
    x[k] = v;
  }
}

// Sums of x and x^2 over segments [starts[g], starts[g+1]) in a fixed order (the map-reduce of
// solver.h:1155-1177, whose thread-local FP64 sums this replaces): pass 1 reduces chunks of
// kRedChunk elements of each segment (block (chunk, g)), pass 2 reduces each segment's chunk
// partials.  Every partial is a compensated double-double sum (Dd), so the result does not
// lose accuracy with the number of PT dets (1e8 and more); only the chunking fixes the order,
// so results are reproducible.
constexpr uint32_t kRedChunk = 1u << 16;

__device__ __forceinline__ void block_sum2(Dd* a, Dd* b) {
  __shared__ Dd s1[8], s2[8];
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    *a = dd_add(*a, dd_shfl_xor(*a, o));
    *b = dd_add(*b, dd_shfl_xor(*b, o));
  }
  if ((threadIdx.x & 31) == 0) {
    s1[threadIdx.x >> 5] = *a;
    s2[threadIdx.x >> 5] = *b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Dd ta, tb;
    for (int w = 0; w < 8; w++) {
      ta = dd_add(ta, s1[w]);
      tb = dd_add(tb, s2[w]);
    }
    *a = ta;
    *b = tb;
  }
}

__global__ void __launch_bounds__(256)
    k_seg_partial2(const double* __restrict__ x, const uint64_t* __restrict__ starts,
                   uint32_t n_chunks, double* part) {
  const uint32_t g = blockIdx.y, ch = blockIdx.x;
  const uint64_t b0 = starts[g] + (uint64_t)ch * kRedChunk;
  const uint64_t e = starts[g + 1];
  const uint64_t b1 = b0 + kRedChunk < e ? b0 + kRedChunk : e;
  Dd a, b;
  for (uint64_t k = b0 + threadIdx.x; k < b1; k += blockDim.x) {
    const double v = x[k];
    a = dd_add(a, v);
    // v^2 as an exact product pair: hi = v*v rounded, lo = its FMA error
    const double sq = v * v;
    Dd t;
    t.hi = sq;
    t.lo = fma(v, v, -sq);
    b = dd_add(b, t);
  }
  block_sum2(&a, &b);
  if (threadIdx.x == 0) {
    double* o = part + 4 * ((size_t)g * n_chunks + ch);
    o[0] = a.hi;
    o[1] = a.lo;
    o[2] = b.hi;
    o[3] = b.lo;
  }
}

__global__ void __launch_bounds__(256)
    k_seg_final2(const double* __restrict__ part, uint32_t n_chunks, double* out) {
  const uint32_t g = blockIdx.x;
  Dd a, b;
  for (uint32_t k = threadIdx.x; k < n_chunks; k += blockDim.x) {
    const double* p = part + 4 * ((size_t)g * n_chunks + k);
    Dd ta, tb;
    ta.hi = p[0];
    ta.lo = p[1];
    tb.hi = p[2];
    tb.lo = p[3];
    a = dd_add(a, ta);
    b = dd_add(b, tb);
  }
  block_sum2(&a, &b);
  if (threadIdx.x == 0) {
    out[2 * g] = a.hi + a.lo;
    out[2 * g + 1] = b.hi + b.lo;
  }
}

}  // namespace

// out[2g], out[2g+1] = sum, sum of squares of x over segment g (total length m).
void seg_reduce2(shci_ctx* c, const double* x, const uint64_t* starts, uint32_t nseg, size_t m,
                 double* out) {
  cudaStream_t s = c->stream;
  const uint32_t n_chunks = static_cast<uint32_t>((m + kRedChunk - 1) / kRedChunk) + 1;
  DevBuf<double> part;
  part.mt = &c->mem;
  part.resize(4 * (size_t)n_chunks * nseg);
  k_seg_partial2<<<dim3(n_chunks, nseg), 256, 0, s>>>(x, starts, n_chunks, part.p);
  SHCI_LAUNCH_CHECK();
  k_seg_final2<<<nseg, 256, 0, s>>>(part.p, n_chunks, out);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 2;
}

namespace {

// starts[it] = first k with (au[k] >> shift) >= it, for it = 0..n_it (au sorted ascending)
__global__ void k_iter_starts(const uint64_t* au, size_t m, int shift, uint32_t n_it,
                              uint64_t* starts) {
  const uint32_t it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it > n_it) return;
  size_t lo = 0, hi = m;
  while (lo < hi) {
    const size_t mid = (lo + hi) >> 1;
    if ((au[mid] >> shift) < it) lo = mid + 1;
    else hi = mid;
  }
  starts[it] = lo;
}

// Fixed-point diagonal tables of the context's integrals (built once per set of integrals).
DiagFix diag_fix(shci_ctx* c) {
  const auto& I = c->I;
  const int n = static_cast<int>(I.n);
  if (!c->dfix_valid) {
    std::vector<double> v(n + 2 * (size_t)n * n, 0.0);
    for (int p = 0; p < n; p++) v[p] = I.h(p, p);
    for (int a = 0; a < n; a++)
      for (int b = 0; b < n; b++) {
        const double J = I.g(a, a, b, b), K = I.g(a, b, b, a);
        v[n + (size_t)a * n + b] = J - K;
        v[n + (size_t)n * n + (size_t)a * n + b] = J;
      }
    double mx = 0.0;
    for (double x : v) mx = std::max(mx, std::fabs(x));
    const int n_e = static_cast<int>(I.n_up + I.n_dn);
    const double bound = (static_cast<double>(n_e) + static_cast<double>(n_e) * n_e) * mx;
    int s = 60;
    while (s > 0 && bound * std::ldexp(1.0, s) >= std::ldexp(1.0, 62)) s--;
    std::vector<long long> t(v.size());
    for (size_t k = 0; k < v.size(); k++) t[k] = std::llround(std::ldexp(v[k], s));
    c->dfix.mt = &c->mem;
    c->dfix.resize(t.size());
    SHCI_CUDA(cudaMemcpyAsync(c->dfix.p, t.data(), t.size() * 8, cudaMemcpyHostToDevice,
                              c->stream));
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
    c->dfix_scale = s;
    c->dfix_valid = true;
  }
  return DiagFix{c->dfix.p, n, std::ldexp(1.0, -c->dfix_scale), I.e_core};
}

// Fixed-point single-excitation tables (built with the diagonal tables, once per set of
// integrals).  Scale: the largest |sum| (h_pq plus at most 2 n_e entries, doubled ones
// counted twice) stays below 2^62.  margin = the rounding of the entries (2^-(s+1) each,
// twice for a doubled one) + the FP64 evaluation's rounding (each of its <= 2 n_e + 1
// additions within 2^-53 of a partial sum <= bound) + the final product by c_i, generously.
SingleFix single_fix(shci_ctx* c) {
  const auto& I = c->I;
  const int n = static_cast<int>(I.n);
  // new integrals invalidate the diagonal tables; rebuild these with them
  const bool stale = !c->dfix_valid || c->sfix.n != (size_t)n * n + 2 * (size_t)n * n * n;
  diag_fix(c);
  if (stale) {
    const size_t n2 = (size_t)n * n, n3 = n2 * n;
    std::vector<double> v(n2 + 2 * n3, 0.0);
    for (int p = 0; p < n; p++)
      for (int q = 0; q < n; q++) {
        v[(size_t)p * n + q] = I.h(p, q);
        for (int o = 0; o < n; o++) {
          v[n2 + ((size_t)p * n + q) * n + o] = I.g(p, q, o, o);
          v[n2 + n3 + ((size_t)p * n + q) * n + o] = I.g(p, o, o, q);
        }
      }
    double mh = 0.0, mt = 0.0;
    for (size_t k = 0; k < n2; k++) mh = std::max(mh, std::fabs(v[k]));
    for (size_t k = n2; k < v.size(); k++) mt = std::max(mt, std::fabs(v[k]));
    const int n_e = static_cast<int>(I.n_up + I.n_dn);
    const double terms = 3.0 * n_e + 1.0;  // bound on the number of entries, doubles twice
    const double bound = mh + terms * mt;
    int s = 60;
    while (s > 0 && bound * std::ldexp(1.0, s) >= std::ldexp(1.0, 62)) s--;
    std::vector<long long> t(v.size());
    for (size_t k = 0; k < v.size(); k++) t[k] = std::llround(std::ldexp(v[k], s));
    c->sfix.mt = &c->mem;
    c->sfix.resize(t.size());
    SHCI_CUDA(cudaMemcpyAsync(c->sfix.p, t.data(), t.size() * 8, cudaMemcpyHostToDevice,
                              c->stream));
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
    c->sfix_scale = s;
    c->sfix_margin = 4.0 * (terms * std::ldexp(1.0, -(s + 1)) + terms * bound * std::ldexp(1.0, -52));
  }
  const size_t n2 = (size_t)n * n, n3 = n2 * n;
  return SingleFix{c->sfix.p, c->sfix.p + n2, c->sfix.p + n2 + n3, n,
                   std::ldexp(1.0, -c->sfix_scale), c->sfix_margin};
}

struct PtSetup {
  SelParams P{};
  DevBuf<uint32_t> pairs;
  unsigned grid = 0;
};

void pt_setup(shci_ctx* c, PtSetup& st) {
  if (!c->Q.built) throw ArgError("heat-bath queues not built (call shci_build_queues)");
  HostScope hs(c->prof, "pt2_host_pt_setup");
  sync_dets(c);
  cudaStream_t s = c->stream;
  const int n_elecs = static_cast<int>(c->I.n_up + c->I.n_dn);
  rebuild_det_set(c);
  std::vector<uint32_t> pairs;
  for (int a = 0; a < n_elecs; a++)
    for (int b = a + 1; b < n_elecs; b++) pairs.push_back(a | (b << 16));
  st.pairs.mt = &c->mem;
  st.pairs.resize(pairs.empty() ? 1 : pairs.size());
  if (!pairs.empty())
    SHCI_CUDA(cudaMemcpyAsync(st.pairs.p, pairs.data(), pairs.size() * 4, cudaMemcpyHostToDevice, s));
  SelParams& P = st.P;
  P.I = c->dI;
  P.up = c->d_up.p;
  P.dn = c->d_dn.p;
  P.coef = c->d_coef.p;
  P.d_off = c->Q.d_off.p;
  P.d_H = c->Q.d_H.p;
  P.d_rs = c->Q.d_rs.p;
  P.s_off = c->Q.s_off.p;
  P.s_S = c->Q.s_S.p;
  P.s_r = c->Q.s_r.p;
  P.pair_tab = st.pairs.p;
  P.set_up = c->set_up.p;
  P.set_dn = c->set_dn.p;
  P.set_n = static_cast<uint32_t>(c->set_up.n);
  P.set_hash = c->set_hash.p;
  P.set_hash_mask = c->set_hash_mask;
  P.max_hci = c->Q.max_hci;
  P.max_singles = c->Q.max_singles;
  P.n_orbs = c->I.n;
  P.n_up = static_cast<int>(c->I.n_up);
  P.n_elecs = n_elecs;
  P.n_pairs = static_cast<int>(pairs.size());
  P.no_doubles = c->has_doubles ? 0 : 1;
  P.inactive = c->inactive_orbs;
  int sms = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  st.grid = static_cast<unsigned>(sms) * 8u;
}

template <int MODE>
constexpr int n_cols() {
  return MODE == kDtm ? 1 : MODE == kPsto ? 2 : 5;
}

// Emits the pairs of the sources [0, n_src) for one batch (or set of iterations), appending
// the valid ones to (bu, bd, bv) after the first *bn; slots[k] = the size of source k's
// region.  Sources whose region overflowed (regions sized by an estimate) are appended to
// *over as launch indices.  The accumulation is sorted and reduced in place whenever it
// grows past kCap, to keep it bounded.
template <int MODE>
void pt_emit_append(shci_ctx* c, PtSetup& st, const PtParams& Q, const StoSources& S,
                    uint32_t n_src, const std::vector<uint64_t>& slots, DevBuf<uint64_t>& bu,
                    DevBuf<uint64_t>& bd, DevBuf<double>* bv, size_t* bn, int a_bits,
                    std::vector<uint32_t>* over) {
  constexpr int NV = n_cols<MODE>();
  cudaStream_t s = c->stream;
  const uint64_t kCap = 1ull << 27;
  DevBuf<uint64_t> cu, cd;
  DevBuf<double> cv[NV];
  DevBuf<uint8_t> d_over;
  cu.mt = cd.mt = &c->mem;
  d_over.mt = &c->mem;
  for (int v = 0; v < NV; v++) cv[v].mt = &c->mem;
  uint32_t k0 = 0;
  while (k0 < n_src) {
    uint64_t tot = 0;
    uint32_t k1 = k0;
    while (k1 < n_src && (k1 == k0 || tot + slots[k1] <= kCap)) tot += slots[k1++];
    if (tot > 0) {
      HostScope hs_off(c->prof, "pt2_host_offsets");
      std::vector<uint64_t> off(k1 - k0 + 1);
      uint64_t acc = 0;
      for (uint32_t k = k0; k < k1; k++) {
        off[k - k0] = acc;
        acc += slots[k];
      }
      off[k1 - k0] = acc;
      DevBuf<uint64_t> d_off;
      d_off.mt = &c->mem;
      d_off.resize(off.size());
      SHCI_CUDA(cudaMemcpyAsync(d_off.p, off.data(), off.size() * 8, cudaMemcpyHostToDevice, s));
      hs_off.stop();
      d_over.resize(k1 - k0);
      SHCI_CUDA(cudaMemsetAsync(d_over.p, 0, k1 - k0, s));
      cu.resize(tot, 1.25);
      cd.resize(tot, 1.25);
      OutCols oc{};
      const double* vptr[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
      for (int v = 0; v < NV; v++) {
        cv[v].resize(tot, 1.25);
        oc.v[v] = cv[v].p;
        vptr[v] = cv[v].p;
      }
      {
        ProfScope ps(c->prof, s, "pt2_emit");
        k_pt_emit<MODE><<<st.grid, kPtWarps * 32, 0, s>>>(st.P, Q, S, single_fix(c), k0, k1,
                                                          d_off.p, cu.p, cd.p, oc, d_over.p);
        SHCI_LAUNCH_CHECK();
      }
      c->launches += 1;
      {
        ProfScope ps(c->prof, s, "pt2_compact");
        compact_valid(c, cu.p, cd.p, vptr, NV, tot, bu, bd, bv, bn);
      }
      std::vector<uint8_t> h_over(k1 - k0);
      SHCI_CUDA(cudaMemcpyAsync(h_over.data(), d_over.p, k1 - k0, cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
      for (uint32_t k = k0; k < k1; k++)
        if (h_over[k - k0]) over->push_back(k);
      if (*bn > kCap) {  // keep the accumulation buffer bounded
        *bn = sort_unique_pairs(c, bu, bd, *bn, bv, NV, a_bits);
        bu.n = bd.n = *bn;
      }
    }
    k0 = k1;
  }
}

template <int MODE>
std::vector<uint64_t> pt_counts(shci_ctx* c, PtSetup& st, const PtParams& Q, const StoSources& S,
                                uint32_t n_src);

// Emits and reduces the pairs of the sources [0, n_src) for one batch / set of iterations;
// returns the unique count, keys in (bu, bd) and value columns in bv[0..n_cols).  slots are
// exact counts or estimates; sources whose estimated region overflowed are emitted again,
// after the others, with exact counts.
template <int MODE>
size_t pt_emit_reduce(shci_ctx* c, PtSetup& st, const PtParams& Q, const StoSources& S,
                      uint32_t n_src, const std::vector<uint64_t>& slots, DevBuf<uint64_t>& bu,
                      DevBuf<uint64_t>& bd, DevBuf<double>* bv, int a_bits) {
  constexpr int NV = n_cols<MODE>();
  cudaStream_t s = c->stream;
  size_t bn = 0;
  std::vector<uint32_t> over;
  pt_emit_append<MODE>(c, st, Q, S, n_src, slots, bu, bd, bv, &bn, a_bits, &over);
  if (!over.empty()) {
    DevBuf<uint32_t> remap;
    remap.mt = &c->mem;
    remap.resize(over.size());
    SHCI_CUDA(cudaMemcpyAsync(remap.p, over.data(), over.size() * 4, cudaMemcpyHostToDevice, s));
    StoSources S2 = S;
    S2.remap = remap.p;
    const uint32_t n2 = static_cast<uint32_t>(over.size());
    const std::vector<uint64_t> exact = pt_counts<MODE>(c, st, Q, S2, n2);
    std::vector<uint32_t> over2;
    pt_emit_append<MODE>(c, st, Q, S2, n2, exact, bu, bd, bv, &bn, a_bits, &over2);
    if (!over2.empty()) throw std::logic_error("PT2 emission: exact regions overflowed");
  }
  {
    ProfScope ps(c->prof, s, "pt2_reduce");
    bn = sort_unique_pairs(c, bu, bd, bn, bv, NV, a_bits);
  }
  bu.n = bd.n = bn;
  return bn;
}

// Region sizes from bounds (each source's window entries, an exact count with one batch):
// with several batches a source's members are a binomial(bound, 1 / n_batches) count, and
// bound / n_batches * 1.3 + 64 exceeds its mean by many standard deviations (overflowing
// sources are re-run exactly).  SHCI_PT_SLOTS="slack,pad" replaces 1.3 and 64.
std::vector<uint64_t> region_slots(const std::vector<uint64_t>& bound, uint64_t n_batches,
                                   const std::vector<uint32_t>* mult = nullptr) {
  // mult[k]: entries of source k (a det walked once for several iterations)
  double slack = 1.3, pad = 64.0;
  if (const char* e = std::getenv("SHCI_PT_SLOTS")) std::sscanf(e, "%lf,%lf", &slack, &pad);
  std::vector<uint64_t> r(bound.size());
  for (size_t k = 0; k < bound.size(); k++) {
    const uint64_t full = bound[k] * (mult ? (*mult)[k] : 1u);
    if (n_batches <= 1) {
      r[k] = full;
      continue;
    }
    const double est = std::ceil(static_cast<double>(full) / n_batches * slack + pad);
    r[k] = std::min<uint64_t>(full, static_cast<uint64_t>(std::max(0.0, est)));
  }
  return r;
}

template <int MODE>
std::vector<uint64_t> pt_counts(shci_ctx* c, PtSetup& st, const PtParams& Q, const StoSources& S,
                                uint32_t n_src) {
  cudaStream_t s = c->stream;
  DevBuf<uint64_t> cnt;
  cnt.mt = &c->mem;
  cnt.resize(n_src ? n_src : 1);
  std::vector<uint64_t> hc(n_src);
  if (n_src) {
    {
      ProfScope ps(c->prof, s, "pt2_count");
      k_pt_count<MODE><<<st.grid, kPtWarps * 32, 0, s>>>(st.P, Q, S, n_src, cnt.p);
      SHCI_LAUNCH_CHECK();
    }
    SHCI_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, n_src * 8, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    c->launches += 1;
  }
  return hc;
}

// Sum and sum of squares of the contributions of one reduced batch (dtm / psto).
template <int MODE>
void pt_batch_sums(shci_ctx* c, DevBuf<uint64_t>& bu, DevBuf<uint64_t>& bd, DevBuf<double>* bv,
                   size_t bn, double e_var, double* sum, double* sumsq) {
  *sum = *sumsq = 0.0;
  if (!bn) return;
  cudaStream_t s = c->stream;
  DevBuf<double> x, out;
  DevBuf<uint64_t> starts;
  x.mt = out.mt = starts.mt = &c->mem;
  x.resize(bn);
  out.resize(2);
  starts.resize(2);
  OutCols oc{};
  for (int v = 0; v < n_cols<MODE>(); v++) oc.v[v] = bv[v].p;
  {
    ProfScope ps(c->prof, s, "pt2_contrib");
    k_pt_x<MODE><<<grid_for(bn, 256), 256, 0, s>>>(diag_fix(c), bu.p, bd.p, oc, bn, e_var, 1.0,
                                                   ~0ull, x.p);
    SHCI_LAUNCH_CHECK();
    const uint64_t st2[2] = {0, bn};
    SHCI_CUDA(cudaMemcpyAsync(starts.p, st2, 16, cudaMemcpyHostToDevice, s));
    seg_reduce2(c, x.p, starts.p, 1, bn, out.p);
  }
  double h[2];
  SHCI_CUDA(cudaMemcpyAsync(h, out.p, 16, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  *sum = h[0];
  *sumsq = h[1];
  c->launches += 2;
}

// Deterministic-style batched stage (dtm: MODE kDtm, psto: kPsto) with the batch accumulation,
// uncertainty and (psto) early stopping of solver.h:691-764, 818-895.
template <int MODE>
Pt2Out pt_batched(shci_ctx* c, double e_var, PtParams Q, size_t n_batches, double target_error,
                  double eps_pt) {
  PtSetup st;
  pt_setup(c, st);
  const uint32_t n_var = static_cast<uint32_t>(c->up.size());
  StoSources S{};
  // slots per source over all batches (sizes the automatic batch count)
  set_batches(Q, 1);
  Q.batch = 0;
  std::vector<uint64_t> hc = pt_counts<MODE>(c, st, Q, S, n_var);
  if (n_batches == 0) {
    // Automatic batch count: every candidate pair costs ~48 device bytes while a batch is
    // processed (keys, value columns, compaction, sort ping-pong); keep a batch within 40% of
    // the free HBM.  (The dtm energy does not depend on the batch count.)
    uint64_t tot = 0;
    for (uint64_t v : hc) tot += v;
    size_t free_b = 0, total_b = 0;
    SHCI_CUDA(cudaMemGetInfo(&free_b, &total_b));
    free_b += c->mem.cached;  // cached blocks return to the driver on demand
    const double per = 48.0 * (MODE == kDtm ? 1.0 : 1.3);
    n_batches = static_cast<size_t>(std::ceil(tot * per / (0.4 * free_b)));
    if (n_batches < 1) n_batches = 1;
  }
  set_batches(Q, n_batches);
  // regions per source: exact with one batch, estimated from the window counts otherwise
  const std::vector<uint64_t> slots = region_slots(hc, n_batches);
  Pt2Out out;
  double esum = 0.0, esq = 0.0;
  size_t n_sum = 0;
  DevBuf<uint64_t> bu, bd;
  DevBuf<double> bv[2];
  bu.mt = bd.mt = bv[0].mt = bv[1].mt = &c->mem;
  for (size_t batch = 0; batch < n_batches; batch++) {
    Q.batch = batch;
    bu.n = bd.n = 0;
    const size_t bn = pt_emit_reduce<MODE>(c, st, Q, S, n_var, slots, bu, bd, bv, 0);
    double bs, bsq;
    pt_batch_sums<MODE>(c, bu, bd, bv, bn, e_var, &bs, &bsq);
    n_sum += bn;
    esum += bs;
    esq += bsq;
    out.value = esum / (batch + 1) * n_batches;
    if (batch == n_batches - 1) {
      out.uncert = 0.0;
    } else {
      const double avg = esum / n_sum;
      const double sd = std::sqrt(esq / n_sum - avg * avg);
      if (MODE == kDtm) {
        out.uncert = sd * std::sqrt((double)n_sum) / (batch + 1) * (n_batches - batch - 1);
      } else {
        const double mean_sd = sd / std::sqrt((double)n_sum);
        out.uncert = mean_sd * n_sum / (batch + 1) * (n_batches - batch - 1);
      }
    }
    out.n_batches_done = batch + 1;
    if (MODE == kPsto) {
      if (out.uncert <= target_error * 0.5) break;
      if (Q.eps <= eps_pt && out.uncert <= target_error) break;
    }
  }
  out.n_pt_dets = n_sum;
  c->prof.flush();
  return out;
}

// f(begin, end) over [0, n) in contiguous chunks, one per host thread (chunk k on thread k).
template <class F>
void host_chunks(size_t n, F f) {
  const size_t k = std::max<size_t>(1, std::min<size_t>(host_threads(), (n + 65535) / 65536));
  std::vector<std::thread> th;
  for (size_t t = 1; t < k; t++) th.emplace_back(f, t, n * t / k, n * (t + 1) / k);
  f(size_t{0}, size_t{0}, n / k);
  for (auto& x : th) x.join();
}

// Vose alias tables, as src/util.cc:128-175.  The scaled probabilities and the initial
// small / large stacks are formed in chunks on the host threads (each chunk's indices in
// order, the chunks concatenated in order: the stacks the sequential pass would build); the
// pairing loop is sequential.
void alias_tables(const std::vector<double>& p, std::vector<double>& np, std::vector<size_t>& al) {
  const size_t L = p.size();
  np.assign(L, 0.0);
  al.assign(L, 0);
  std::vector<double> t(L);
  std::vector<size_t> small, large;  // used as stacks (back = top)
  std::vector<std::vector<size_t>> cs(host_threads()), cl(host_threads());
  host_chunks(L, [&](size_t k, size_t b, size_t e) {
    for (size_t i = b; i < e; i++) {
      t[i] = p[i] * L;
      if (t[i] < 1.) cs[k].push_back(i);
      else cl[k].push_back(i);
    }
  });
  small.reserve(L);
  large.reserve(L);
  for (auto& v : cs) small.insert(small.end(), v.begin(), v.end());
  for (auto& v : cl) large.insert(large.end(), v.begin(), v.end());
  while (!small.empty() && !large.empty()) {
    const size_t l = large.back(), s = small.back();
    np[s] = t[s];
    al[s] = l;
    t[l] = t[l] + t[s] - 1.;
    if (t[l] < 1.) {
      large.pop_back();
      small.back() = l;
    } else {
      small.pop_back();
    }
  }
  for (size_t i : large) np[i] = 1.;
  for (size_t i : small) np[i] = 1.;
}

}  // namespace

Pt2Out pt2_dtm(shci_ctx* c, double energy_var, double eps_pt_dtm, size_t n_batches) {
  PtParams Q{};
  Q.eps = eps_pt_dtm;
  return pt_batched<kDtm>(c, energy_var, Q, n_batches, 0.0, 0.0);
}

Pt2Out pt2_psto(shci_ctx* c, double energy_var, double eps_pt_dtm, double eps_pt_psto,
                size_t n_batches, double target_error, double eps_pt) {
  if (n_batches == 0) throw ArgError("n_batches must be >= 1");
  PtParams Q{};
  Q.eps = eps_pt_psto;
  Q.eps_dtm = eps_pt_dtm;
  return pt_batched<kPsto>(c, energy_var, Q, n_batches, target_error, eps_pt);
}

// Number of unique PT dets in hash batch 0 of 128 of the given sources (the sample-size
// pilot of solver.h:942-972; no |H_ai c_i| test on double excitations).
size_t pilot_pt_dets(shci_ctx* c, PtSetup& st, const std::vector<size_t>& src, double eps_pt,
                     int shift) {
  if (src.empty()) return 0;
  cudaStream_t s = c->stream;
  const uint32_t n_src = static_cast<uint32_t>(src.size());
  std::vector<uint32_t> h_det(src.begin(), src.end()), h_zero(n_src, 0u);
  std::vector<double> h_one(n_src, 1.0);
  std::vector<uint8_t> h_dtm(n_src, 1);
  DevBuf<uint32_t> d_det, d_zero;
  DevBuf<double> d_one;
  DevBuf<uint8_t> d_dtm;
  d_det.mt = d_zero.mt = d_one.mt = d_dtm.mt = &c->mem;
  d_det.resize(n_src);
  d_zero.resize(n_src);
  d_one.resize(n_src);
  d_dtm.resize(n_src);
  SHCI_CUDA(cudaMemcpyAsync(d_det.p, h_det.data(), n_src * 4, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(d_zero.p, h_zero.data(), n_src * 4, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(d_one.p, h_one.data(), n_src * 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(d_dtm.p, h_dtm.data(), n_src, cudaMemcpyHostToDevice, s));
  StoSources S{d_det.p, d_zero.p, d_one.p, d_one.p, d_zero.p, d_dtm.p};
  PtParams Q{};
  Q.eps = eps_pt;
  Q.eps_psto = eps_pt;
  Q.factor = 0.0;
  Q.iter_shift = shift;
  Q.pilot = 1;
  set_batches(Q, 128);
  PtParams Q1 = Q;
  set_batches(Q1, 1);
  const std::vector<uint64_t> hc = region_slots(pt_counts<kSto>(c, st, Q1, S, n_src), 128);
  DevBuf<uint64_t> bu, bd;
  DevBuf<double> bv[5];
  bu.mt = bd.mt = &c->mem;
  for (auto& b : bv) b.mt = &c->mem;
  return pt_emit_reduce<kSto>(c, st, Q, S, n_src, hc, bu, bd, bv, shift + 5);
}

size_t psto_auto_batches(shci_ctx* c, double eps_pt_psto, double pt_mem_avail, double mem_usage,
                         size_t* n_pilot) {
  const int shift = c->I.n;
  if (shift > 57) throw ArgError("the automatic psto batch count supports n_orbs <= 57");
  PtSetup st;
  pt_setup(c, st);
  std::vector<size_t> src;
  for (size_t i = 50; i < c->up.size(); i += 100) src.push_back(i);
  const size_t n_pt = pilot_pt_dets(c, st, src, eps_pt_psto, shift);
  if (n_pilot) *n_pilot = n_pt;
  const size_t bytes_per_entry = 2 * 16 + 16;  // solver.h:402, 774
  const double mem = static_cast<double>(static_cast<size_t>(pt_mem_avail)) * mem_usage;
  size_t nb = static_cast<size_t>(std::ceil(2.5 * 128 * 100 * static_cast<double>(n_pt) *
                                            static_cast<double>(bytes_per_entry) / mem));
  if (nb < 16) nb = 16;
  return nb;
}

// Stochastic stage (solver.h:898-1153).  n_dets_in_sample = 0: the sample size comes from
// the reference's 1,000-draw pilot and the PT memory pt_mem_avail (solver.h:942-1006);
// semisto: the variational dets above the quantile of the top quarter of the unique-sample
// target are summed deterministically in every iteration and the others sampled with
// renormalised weights (solver.h:1009-1036).  psto_uncert is the uncertainty of the preceding
// stage (it enters the second stopping rule).  info = {n_dets_in_sample, n_dtm,
// n_unique_target} of the run.
Pt2Out pt2_sto(shci_ctx* c, double energy_var, double eps_pt_psto, double eps_pt,
               size_t n_batches, size_t n_dets_in_sample, bool semisto, unsigned random_seed,
               size_t max_iterations, double target_error, double psto_uncert,
               double pt_mem_avail, double mem_usage, std::vector<double>* loops,
               size_t* info) {
  if (n_batches == 0) throw ArgError("n_batches must be >= 1");
  if (n_dets_in_sample == 1) throw ArgError("n_dets_in_sample_pt_sto must be 0 (automatic) or >= 2");
  if (semisto && n_dets_in_sample != 0)
    throw ArgError("semisto_sto with n_dets_in_sample_pt_sto set has no deterministic dets in "
                   "the reference (its 25% quantile heap is empty: solver.h:1009-1021); set "
                   "semisto_sto to false or leave n_dets_in_sample_pt_sto unset");
  const size_t n_var = c->up.size();
  std::vector<double> coefs(n_var);
  sync_dets(c);
  cudaStream_t s = c->stream;
  SHCI_CUDA(cudaMemcpyAsync(coefs.data(), c->d_coef.p, n_var * 8, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  const int shift = c->I.n;
  if (shift > 57) throw ArgError("stochastic PT2 supports n_orbs <= 57");
  const auto t_setup = std::chrono::steady_clock::now();
  // probabilities and their running sums (solver.h:921-933)
  double sum_w = 0.0;
  for (size_t i = 0; i < n_var; i++) sum_w += std::abs(coefs[i]);
  std::vector<double> probs(n_var), cum;
  host_chunks(n_var, [&](size_t, size_t b, size_t e) {
    for (size_t i = b; i < e; i++) probs[i] = std::abs(coefs[i]) / sum_w;
  });
  if (n_dets_in_sample == 0) {  // the pilot draws by inverse CDF
    cum.resize(n_var);
    for (size_t i = 0; i < n_var; i++) cum[i] = i > 0 ? probs[i] + cum[i - 1] : probs[i];
  }
  std::default_random_engine gen(random_seed);
  std::uniform_real_distribution<double> ur(0., 1.);
  PtSetup st;
  pt_setup(c, st);
  size_t n_target = 0;
  if (n_dets_in_sample == 0) {
    // pilot (solver.h:944-972): 1,000 inverse-CDF draws, PT dets of the unique ones in batch
    // 0 of 128, scaled to a batch of n_batches
    std::vector<uint8_t> seen(n_var, 0);
    std::vector<size_t> list;
    for (size_t k = 0; k < 1000; k++) {
      const size_t id = std::lower_bound(cum.begin(), cum.end(), ur(gen)) - cum.begin();
      if (id < n_var && !seen[id]) {
        seen[id] = 1;
        list.push_back(id);
      } else if (id >= n_var) {
        throw ArgError("coefficient weights do not sum to 1 (empty or non-finite wavefunction)");
      }
    }
    const size_t n_pt = pilot_pt_dets(c, st, list, eps_pt, shift);
    const size_t n_pt_batch = n_pt * 128 / n_batches;
    const size_t bytes_per_entry = 2 * 16 + 40;  // solver.h:402, 905 (two 64-bit chunks)
    const size_t cap = n_var / 8 + 1;
    // a pilot without PT dets is a division by zero in the reference; the cap is taken
    n_target = cap;
    if (n_pt_batch > 0) {
      const double t = static_cast<double>(static_cast<size_t>(pt_mem_avail)) * mem_usage *
                       static_cast<double>(list.size()) / static_cast<double>(bytes_per_entry) /
                       5.0 / static_cast<double>(n_pt_batch);
      n_target = static_cast<size_t>(t);
      if (n_target >= cap) n_target = cap;
    }
    // draws until the target of unique dets is met (solver.h:990-1000)
    std::fill(seen.begin(), seen.end(), 0);
    size_t n_unique = 0;
    while (n_unique < n_target) {
      const size_t id = std::lower_bound(cum.begin(), cum.end(), ur(gen)) - cum.begin();
      if (id >= n_var)
        throw ArgError("coefficient weights do not sum to 1 (empty or non-finite wavefunction)");
      if (!seen[id]) {
        seen[id] = 1;
        n_unique++;
      }
      n_dets_in_sample++;
    }
  }
  std::vector<uint32_t> dtm_list;
  if (semisto) {
    // the top n_target / 4 weights by a min-heap quantile (solver.h:1009-1036)
    const size_t n_heap = n_target / 4;
    if (n_heap == 0)
      throw ArgError("semistochastic PT2 needs a sample-size target of at least 4 (the "
                     "reference's quantile heap would be empty)");
    std::priority_queue<double, std::vector<double>, std::greater<double>> heap;
    for (size_t i = 0; i < n_heap; i++) heap.push(probs[i]);
    for (size_t i = n_heap; i < n_var; i++)
      if (heap.top() < probs[i]) {
        heap.pop();
        heap.push(probs[i]);
      }
    const double C = heap.top();
    double s2 = 0.0;
    for (size_t i = 0; i < n_var; i++) {
      if (probs[i] > C) {
        probs[i] = 0.;
        dtm_list.push_back(static_cast<uint32_t>(i));
      } else {
        s2 += probs[i];
      }
    }
    for (auto& p : probs) p /= s2;
  }
  const size_t n_dtm = dtm_list.size();
  if (n_dets_in_sample < n_dtm + 2)
    throw ArgError("stochastic PT2 sample too small for its deterministic part");
  if (info) {
    info[0] = n_dets_in_sample;
    info[1] = n_dtm;
    info[2] = n_target;
  }
  std::uniform_int_distribution<size_t> ui_var(0, n_var - 1);
  std::uniform_int_distribution<size_t> ui_batch(0, n_batches - 1);
  const double factor = 1. / (n_dets_in_sample - n_dtm - 1.);
  // Iterations per device pass: the first pass runs the 6 iterations before which the
  // stopping rules cannot fire, later passes 2 (results past the stop are discarded).
  const uint32_t kFirstChunk = 6, kNextChunk = 2;
  // A pass's random numbers in the reference's order (per iteration: its draws, then its
  // batch, solver.h:1048-1072).  They depend on nothing but the generator, so a helper thread
  // draws each pass ahead of it: the first while the alias tables are built, the next during
  // the current pass's device work (a pass that turns out not to be needed only advanced the
  // generator, which nothing uses afterwards).
  const size_t n_draw = n_dets_in_sample - n_dtm;
  struct PassDraws {
    std::vector<std::vector<size_t>> r1;
    std::vector<std::vector<double>> r2;
    std::vector<size_t> batch;
  };
  auto draw_pass = [&gen, &ur, &ui_var, &ui_batch, n_draw](uint32_t n_it) {
    PassDraws d;
    d.r1.assign(n_it, std::vector<size_t>(n_draw));
    d.r2.assign(n_it, std::vector<double>(n_draw));
    d.batch.resize(n_it);
    for (uint32_t it = 0; it < n_it; it++) {
      for (size_t k = 0; k < n_draw; k++) {
        d.r1[it][k] = ui_var(gen);
        d.r2[it][k] = ur(gen);
      }
      d.batch[it] = ui_batch(gen);
    }
    return d;
  };
  // one helper thread draws ahead unless the calling thread may use only one host thread
  const unsigned n_host = host_threads();
  const auto draw_policy = n_host > 1 ? std::launch::async : std::launch::deferred;
  std::future<PassDraws> next_draws;
  if (max_iterations > 0)
    next_draws = std::async(draw_policy, draw_pass,
                            static_cast<uint32_t>(std::min<size_t>(kFirstChunk, max_iterations)));
  // per-iteration sample counts, one array per iteration of a pass (zero between uses; set up
  // on a helper thread while the alias tables are built); which iterations of a pass drew
  // each det (zero between uses); the deterministic dets
  std::vector<std::vector<uint32_t>> cnts;
  std::vector<uint8_t> pass_mask, is_dtm;
  auto zeroed = std::async(n_host > 1 ? std::launch::async : std::launch::deferred, [&]() {
    const size_t k = std::min<size_t>(std::max<size_t>(kFirstChunk, kNextChunk), max_iterations);
    for (size_t it = 0; it < k; it++) cnts.emplace_back(n_var, 0u);
    pass_mask.assign(n_var, 0);
    is_dtm.assign(n_var, 0);
  });
  std::vector<double> aprob;
  std::vector<size_t> alias;
  alias_tables(probs, aprob, alias);
  zeroed.get();
  for (uint32_t i : dtm_list) is_dtm[i] = 1;
  static_assert(kFirstChunk <= 8 && kNextChunk <= 8, "iteration masks are 8 bits");
  if (c->prof.on)
    c->prof.host("pt2_host_setup", std::chrono::duration<double, std::milli>(
                                       std::chrono::steady_clock::now() - t_setup).count());
  Pt2Out out;
  std::vector<double> loop_vals;
  bool done = false;
  size_t iteration = 0;
  while (!done && iteration < max_iterations) {
    // draw the samples of the next chunk of iterations (solver.h:1048-1072)
    const uint32_t chunk = iteration == 0 ? kFirstChunk : kNextChunk;
    const uint32_t n_it = static_cast<uint32_t>(std::min<size_t>(chunk, max_iterations - iteration));
    std::vector<uint32_t> h_det, h_iter, h_batch, h_off;
    std::vector<double> h_count, h_weight;
    std::vector<uint8_t> h_dtm;
    {
      HostScope hs(c->prof, "pt2_host_sample");
      // the pass's random numbers (drawn ahead), then the next pass's, ahead of it
      HostScope hs_rng(c->prof, "pt2_host_sample_rng");
      PassDraws draws = next_draws.get();
      hs_rng.stop();
      const size_t it_next = iteration + n_it;
      if (it_next < max_iterations)
        next_draws = std::async(
            draw_policy, draw_pass,
            static_cast<uint32_t>(std::min<size_t>(kNextChunk, max_iterations - it_next)));
      const auto& r1s = draws.r1;
      const auto& r2s = draws.r2;
      const auto& batch_ids = draws.batch;
      // Per iteration and on a host thread of its own: the alias lookups (independent of one
      // another: one loop whose cache misses overlap, the table entries of a later draw
      // prefetched; the tables are far larger than the host caches), the sample counts per det
      // and the dets in order of first draw (the reference's unordered_map counts and
      // insertion-ordered list).
      while (cnts.size() < n_it) cnts.emplace_back(n_var, 0u);
      std::vector<std::vector<uint32_t>> lists(n_it);
      auto sample_one = [&](uint32_t it) {
        constexpr size_t kAhead = 32;
        const auto& r1 = r1s[it];
        const auto& r2 = r2s[it];
        auto& cnt = cnts[it];
        std::vector<uint32_t> ids(n_draw);
        for (size_t k = 0; k < n_draw; k++) {
          if (k + kAhead < n_draw) {
            __builtin_prefetch(&aprob[r1[k + kAhead]]);
            __builtin_prefetch(&alias[r1[k + kAhead]]);
          }
          ids[k] = static_cast<uint32_t>(r2[k] < aprob[r1[k]] ? r1[k] : alias[r1[k]]);
        }
        auto& list = lists[it];
        for (size_t k = 0; k < n_draw; k++) {
          if (k + kAhead < n_draw) __builtin_prefetch(&cnt[ids[k + kAhead]], 1);
          const uint32_t id = ids[k];
          if (cnt[id]++ == 0) list.push_back(id);
        }
      };
      {
        HostScope hs_look(c->prof, "pt2_host_sample_lookup");
        std::atomic<uint32_t> next_it{0};
        auto run = [&]() {
          for (uint32_t it; (it = next_it.fetch_add(1)) < n_it;) sample_one(it);
        };
        std::vector<std::thread> th;
        for (uint32_t t = 1; t < std::min<uint32_t>(n_it, n_host); t++) th.emplace_back(run);
        run();
        for (auto& t : th) t.join();
      }
      HostScope hs_group(c->prof, "pt2_host_sample_group");
      // The pass's entries grouped by det, dets in increasing order and a det's iterations in
      // order: a det drawn in several iterations is walked once (the heaviest dets, with the
      // widest windows, are drawn in nearly every iteration).  A bit mask per det marks the
      // iterations that drew it (all of them for a deterministic det: count and weight 1); one
      // scan of the masks in det order lays the entries out.
      const uint8_t all_it = static_cast<uint8_t>((1u << n_it) - 1u);
      size_t n_ent_pass = n_dtm * n_it;
      for (uint32_t it = 0; it < n_it; it++) {
        n_ent_pass += lists[it].size();
        for (uint32_t i : lists[it]) pass_mask[i] |= static_cast<uint8_t>(1u << it);
      }
      for (uint32_t i : dtm_list) pass_mask[i] = all_it;
      h_det.resize(n_ent_pass);
      h_iter.resize(n_ent_pass);
      h_batch.resize(n_ent_pass);
      h_count.resize(n_ent_pass);
      h_weight.resize(n_ent_pass);
      h_dtm.resize(n_ent_pass);
      h_off.clear();
      size_t k = 0;
      for (size_t i = 0; i < n_var; i++) {
        const uint32_t m = pass_mask[i];
        if (!m) continue;
        pass_mask[i] = 0;
        h_off.push_back(static_cast<uint32_t>(k));
        const bool dt = is_dtm[i] != 0;
        for (uint32_t it = 0; it < n_it; it++) {
          if (!(m >> it & 1u)) continue;
          h_det[k] = static_cast<uint32_t>(i);
          h_iter[k] = it;
          h_batch[k] = static_cast<uint32_t>(batch_ids[it]);
          if (dt) {
            h_count[k] = 1.0;
            h_weight[k] = 1.0;
            h_dtm[k] = 1;
          } else {
            h_count[k] = static_cast<double>(cnts[it][i]);
            cnts[it][i] = 0;
            h_weight[k] = (n_dets_in_sample - n_dtm) * probs[i];
            h_dtm[k] = 0;
          }
          k++;
        }
      }
      h_off.push_back(static_cast<uint32_t>(k));
    }
    const uint32_t n_ent = static_cast<uint32_t>(h_det.size());
    const uint32_t n_src = static_cast<uint32_t>(h_off.size() - 1);  // dets of the pass
    DevBuf<uint32_t> d_det, d_iter, d_batch;
    DevBuf<double> d_count, d_weight;
    DevBuf<uint8_t> d_dtm;
    DevBuf<uint32_t> d_off;
    d_det.mt = d_iter.mt = d_batch.mt = d_count.mt = d_weight.mt = d_dtm.mt = &c->mem;
    d_off.mt = &c->mem;
    d_off.resize(n_src + 1);
    SHCI_CUDA(cudaMemcpyAsync(d_off.p, h_off.data(), (n_src + 1) * 4, cudaMemcpyHostToDevice, s));
    d_det.resize(n_ent);
    d_iter.resize(n_ent);
    d_batch.resize(n_ent);
    d_count.resize(n_ent);
    d_weight.resize(n_ent);
    d_dtm.resize(n_ent);
    SHCI_CUDA(cudaMemcpyAsync(d_det.p, h_det.data(), n_ent * 4, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(d_iter.p, h_iter.data(), n_ent * 4, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(d_batch.p, h_batch.data(), n_ent * 4, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(d_count.p, h_count.data(), n_ent * 8, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(d_weight.p, h_weight.data(), n_ent * 8, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(d_dtm.p, h_dtm.data(), n_ent, cudaMemcpyHostToDevice, s));
    StoSources S{d_det.p, d_iter.p, d_count.p, d_weight.p, d_batch.p, d_dtm.p, nullptr, d_off.p};
    PtParams Q{};
    Q.eps = eps_pt;
    Q.eps_psto = eps_pt_psto;
    set_batches(Q, n_batches);
    Q.factor = factor;
    Q.iter_shift = shift;
    PtParams Q1 = Q;
    set_batches(Q1, 1);
    std::vector<uint32_t> mult(n_src);
    for (uint32_t g = 0; g < n_src; g++) mult[g] = h_off[g + 1] - h_off[g];
    const std::vector<uint64_t> hc =
        region_slots(pt_counts<kSto>(c, st, Q1, S, n_src), n_batches, &mult);
    DevBuf<uint64_t> bu, bd;
    DevBuf<double> bv[5];
    bu.mt = bd.mt = &c->mem;
    for (auto& b : bv) b.mt = &c->mem;
    const size_t bn = pt_emit_reduce<kSto>(c, st, Q, S, n_src, hc, bu, bd, bv, shift + 5);
    // per-iteration sums of the contributions
    std::vector<double> it_sum(n_it, 0.0);
    if (bn) {
      DevBuf<double> x, o;
      DevBuf<uint64_t> starts;
      x.mt = o.mt = starts.mt = &c->mem;
      x.resize(bn);
      o.resize(2 * n_it);
      starts.resize(n_it + 1);
      OutCols oc{};
      for (int v = 0; v < 5; v++) oc.v[v] = bv[v].p;
      const uint64_t mask = shift == 64 ? ~0ull : ((1ull << shift) - 1ull);
      {
        ProfScope ps(c->prof, s, "pt2_contrib");
        k_pt_x<kSto><<<grid_for(bn, 256), 256, 0, s>>>(diag_fix(c), bu.p, bd.p, oc, bn,
                                                       energy_var, static_cast<double>(n_batches),
                                                       mask, x.p);
        SHCI_LAUNCH_CHECK();
        k_iter_starts<<<1, 128, 0, s>>>(bu.p, bn, shift, n_it, starts.p);
        SHCI_LAUNCH_CHECK();
        seg_reduce2(c, x.p, starts.p, n_it, bn, o.p);
      }
      std::vector<double> h(2 * n_it);
      SHCI_CUDA(cudaMemcpyAsync(h.data(), o.p, h.size() * 8, cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
      for (uint32_t it = 0; it < n_it; it++) it_sum[it] = h[2 * it];
      c->launches += 3;
    }
    out.n_pt_dets += bn;
    // statistics and stopping rules, iteration by iteration (solver.h:1126-1147)
    for (uint32_t it = 0; it < n_it && !done; it++) {
      loop_vals.push_back(it_sum[it]);
      const double n = static_cast<double>(loop_vals.size());
      double sm = 0.0, sq = 0.0;
      for (double v : loop_vals) {
        sm += v;
        sq += v * v;
      }
      out.value = sm / n;
      out.uncert = std::sqrt((sq - sm * sm / n) / (n - 1)) / std::sqrt(n);
      iteration++;
      if (iteration >= 6 && out.uncert <= target_error * 0.7) done = true;
      if (iteration >= 10 &&
          std::sqrt(out.uncert * out.uncert + psto_uncert * psto_uncert) <= target_error)
        done = true;
    }
  }
  out.n_batches_done = iteration;
  if (loops) *loops = loop_vals;
  c->prof.flush();
  return out;
}

}  // namespace shci

// Deterministic Epstein-Nesbet PT2 (K6 in PT mode + K7).
//
// Reference: Solver<S>::get_energy_pt_dtm (src/solver/solver.h:636-764) and mapreduce_sum
// (:1155-1177).  For batch b of n_batches, every var det i emits the connected dets a
// (heat-bath window [eps_pt_dtm / |c_i|, INF)) with rehash(DetHasher(a)) % n_batches == b,
// a not variational, and |H_ai c_i| >= eps_pt_dtm, as (a, H_ai c_i) pairs.  The reference
// accumulates them in a distributed hash map; here the pairs are compacted, radix-sorted by
// det and reduced by key (a fixed-order segmented sum), and a second kernel forms
// (sum_i H_ai c_i)^2 / (E_var - H_aa) per unique a and reduces the contributions and their
// squares in a fixed order.
#include <cmath>

#include "ctx.h"
#include "heatbath.cuh"
#include "kernels.h"

namespace shci {

namespace {

constexpr int kPtWarps = 8;

__global__ void __launch_bounds__(kPtWarps * 32)
    k_pt_count(SelParams P, double eps_pt, uint32_t n_src, uint64_t* cnt_out) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t wpg = gridDim.x * kPtWarps;
  for (uint32_t i = blockIdx.x * kPtWarps + (threadIdx.x >> 5); i < n_src; i += wpg) {
    const double ac = fabs(P.coef[i]);
    const double eps_min = eps_pt / ac;
    const double eps_max = 1.0e100 / ac;
    const uint64_t up = P.up[i], dn = P.dn[i];
    const int n_slots = P.n_elecs + P.n_pairs;
    uint64_t tot = 0;
    for (int s0 = 0; s0 < n_slots; s0 += 32) {
      uint32_t lo = 0, c = 0;
      if (s0 + (int)lane < n_slots) slot_range(P, up, dn, s0 + lane, eps_min, eps_max, &lo, &c);
      uint64_t cc = c;
#pragma unroll
      for (int o = 16; o; o >>= 1) cc += __shfl_xor_sync(kFull, cc, o);
      tot += cc;
    }
    if (lane == 0) cnt_out[i] = tot;
  }
}

__global__ void __launch_bounds__(kPtWarps * 32)
    k_pt_emit(SelParams P, double eps_pt, uint64_t n_batches, uint64_t batch, uint32_t k_begin,
              uint32_t k_end, const uint64_t* off, uint64_t* out_up, uint64_t* out_dn,
              double* out_v) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t wpg = gridDim.x * kPtWarps;
  for (uint32_t i = k_begin + blockIdx.x * kPtWarps + (threadIdx.x >> 5); i < k_end; i += wpg) {
    const double coef = P.coef[i];
    const double ac = fabs(coef);
    const double eps_min = eps_pt / ac;
    const double eps_max = 1.0e100 / ac;
    const uint64_t up = P.up[i], dn = P.dn[i];
    uint64_t base = off[i - k_begin];
    const int n_slots = P.n_elecs + P.n_pairs;
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
        const uint32_t e = o_lo + (t - (o_inc - o_c));
        uint64_t cu, cd;
        bool single;
        bool ok = make_candidate(P, up, dn, s0 + (int)ol, e, &cu, &cd, &single);
        double hc = 0.0;
        // handler order of solver.h:703-713: batch, variational set, |H_ai c_i|
        if (ok && rehash(det_hash(cu, cd)) % n_batches != batch) ok = false;
        if (ok && in_set(P, cu, cd)) ok = false;
        if (ok) {
          const double h = h_offdiag(P.I, up, dn, cu, cd);
          hc = h * coef;
          if (fabs(hc) < eps_pt) ok = false;
        }
        out_up[base + t] = ok ? cu : kInvalid;
        out_dn[base + t] = ok ? cd : kInvalid;
        out_v[base + t] = hc;
      }
      base += total;
    }
  }
}

// Per unique PT det: x = S^2 / (E_var - H_aa); partial sums of x and x^2 per block.
__global__ void __launch_bounds__(256)
    k_pt_contrib(DevIntegrals I, const uint64_t* au, const uint64_t* ad, const double* S,
                 size_t m, double e_var, double* partial) {
  double sx = 0.0, sxx = 0.0;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < m;
       k += (size_t)gridDim.x * blockDim.x) {
    const double haa = h_diag(I, au[k], ad[k]);
    const double x = S[k] * S[k] / (e_var - haa);
    sx += x;
    sxx += x * x;
  }
  __shared__ double s1[8], s2[8];
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    sx += __shfl_xor_sync(kFull, sx, o);
    sxx += __shfl_xor_sync(kFull, sxx, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s1[threadIdx.x >> 5] = sx;
    s2[threadIdx.x >> 5] = sxx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < 8; w++) {
      a += s1[w];
      b += s2[w];
    }
    partial[2 * blockIdx.x] = a;
    partial[2 * blockIdx.x + 1] = b;
  }
}

}  // namespace

Pt2Out pt2_dtm(shci_ctx* c, double energy_var, double eps_pt, size_t n_batches) {
  if (!c->Q.built) throw ArgError("heat-bath queues not built (call shci_build_queues)");
  if (n_batches == 0) throw ArgError("n_batches must be >= 1");
  sync_dets(c);
  cudaStream_t s = c->stream;
  const size_t n_var = c->up.size();
  const int n_elecs = static_cast<int>(c->I.n_up + c->I.n_dn);
  rebuild_det_set(c);
  std::vector<uint32_t> pairs;
  for (int a = 0; a < n_elecs; a++)
    for (int b = a + 1; b < n_elecs; b++) pairs.push_back(a | (b << 16));
  DevBuf<uint32_t> d_pairs;
  d_pairs.mt = &c->mem;
  d_pairs.resize(pairs.empty() ? 1 : pairs.size());
  if (!pairs.empty())
    SHCI_CUDA(cudaMemcpyAsync(d_pairs.p, pairs.data(), pairs.size() * 4, cudaMemcpyHostToDevice, s));
  SelParams P{};
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
  P.pair_tab = d_pairs.p;
  P.set_up = c->set_up.p;
  P.set_dn = c->set_dn.p;
  P.set_n = static_cast<uint32_t>(c->set_up.n);
  P.max_hci = c->Q.max_hci;
  P.max_singles = c->Q.max_singles;
  P.n_orbs = c->I.n;
  P.n_up = static_cast<int>(c->I.n_up);
  P.n_elecs = n_elecs;
  P.n_pairs = static_cast<int>(pairs.size());

  int sms = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const unsigned grid = static_cast<unsigned>(sms) * 8u;
  DevBuf<uint64_t> cnt, cu, cd, bu, bd;
  DevBuf<double> cv, bv, partial;
  cnt.mt = cu.mt = cd.mt = bu.mt = bd.mt = &c->mem;
  cv.mt = bv.mt = partial.mt = &c->mem;
  cnt.resize(n_var ? n_var : 1);
  k_pt_count<<<grid, kPtWarps * 32, 0, s>>>(P, eps_pt, (uint32_t)n_var, cnt.p);
  SHCI_LAUNCH_CHECK();
  std::vector<uint64_t> hc(n_var);
  SHCI_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, n_var * 8, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 1;
  const uint64_t kCap = 1ull << 27;
  const unsigned cgrid = static_cast<unsigned>(sms) * 4u;
  partial.resize(2 * cgrid);
  Pt2Out out;
  double esum = 0.0, esq = 0.0;
  size_t n_sum = 0;
  for (size_t batch = 0; batch < n_batches; batch++) {
    size_t bn = 0;
    uint32_t k0 = 0;
    while (k0 < n_var) {
      uint64_t tot = 0;
      uint32_t k1 = k0;
      while (k1 < n_var && (k1 == k0 || tot + hc[k1] <= kCap)) tot += hc[k1++];
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
        cv.resize(tot, 1.25);
        {
          ProfScope ps(c->prof, s, "pt2_emit");
          k_pt_emit<<<grid, kPtWarps * 32, 0, s>>>(P, eps_pt, n_batches, batch, k0, k1, d_off.p,
                                                   cu.p, cd.p, cv.p);
          SHCI_LAUNCH_CHECK();
        }
        c->launches += 1;
        compact_valid(c, cu.p, cd.p, cv.p, tot, bu, bd, &bv, &bn);
        // keep the batch buffer bounded: reduce by key when it grows large
        if (bn > kCap) {
          bn = sort_unique_pairs(c, bu, bd, bn, &bv);
          bu.n = bd.n = bv.n = bn;
        }
      }
      k0 = k1;
    }
    {
      ProfScope ps(c->prof, s, "pt2_reduce");
      bn = sort_unique_pairs(c, bu, bd, bn, &bv);
    }
    bu.n = bd.n = bv.n = bn;
    double bs = 0.0, bsq = 0.0;
    if (bn) {
      {
        ProfScope ps(c->prof, s, "pt2_contrib");
        k_pt_contrib<<<cgrid, 256, 0, s>>>(c->dI, bu.p, bd.p, bv.p, bn, energy_var, partial.p);
        SHCI_LAUNCH_CHECK();
      }
      std::vector<double> hp(2 * cgrid);
      SHCI_CUDA(cudaMemcpyAsync(hp.data(), partial.p, hp.size() * 8, cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
      for (unsigned b = 0; b < cgrid; b++) {
        bs += hp[2 * b];
        bsq += hp[2 * b + 1];
      }
      c->launches += 1;
    }
    // batch accumulation and uncertainty as solver.h:733-743
    n_sum += bn;
    esum += bs;
    esq += bsq;
    out.value = esum / (batch + 1) * n_batches;
    if (batch == n_batches - 1) {
      out.uncert = 0.0;
    } else {
      const double avg = esum / n_sum;
      const double sd = std::sqrt(esq / n_sum - avg * avg);
      out.uncert = sd * std::sqrt((double)n_sum) / (batch + 1) * (n_batches - batch - 1);
    }
  }
  out.n_pt_dets = n_sum;
  c->prof.flush();
  return out;
}

}  // namespace shci

// Batched connected-determinant enumeration: BaseSystem::find_connected_dets
// (src/base_system.h:57-62) as ChemSystem implements it (src/chem/chem_system.cc:289-402),
// with second rejection off, for many dets in one call.
//
// A warp owns one det and walks its heat-bath slots (pt_walk, heatbath.cuh): one slot per
// electron for single excitations, one per electron pair for doubles, each slot's window of
// its queue in the reference's order.  The candidates that pass the occupancy checks are the
// dets the reference's handler would receive, in the handler's order.  A count pass sizes
// each det's output; an emit pass writes (up, dn, n_excite) at the det's offset.
#include <vector>

#include "ctx.h"
#include "heatbath.cuh"
#include "kernels.h"

namespace shci {

namespace {

constexpr int kConnWarps = 8;

// Window of det k: the reference returns before any handler call when eps_max < eps_min
// (chem_system.cc:295).
__device__ __forceinline__ bool conn_window(const double* eps_max, const double* eps_min,
                                            uint32_t k, double* lo, double* hi) {
  *lo = eps_min[k];
  *hi = eps_max[k];
  return !(*hi < *lo);
}

__global__ void __launch_bounds__(kConnWarps * 32)
    k_conn_count(SelParams P, const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn,
                 const double* __restrict__ eps_max, const double* __restrict__ eps_min,
                 uint32_t n, uint64_t* cnt) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t wpg = gridDim.x * kConnWarps;
  for (uint32_t k = blockIdx.x * kConnWarps + (threadIdx.x >> 5); k < n; k += wpg) {
    double lo, hi;
    uint64_t tot = 0;
    if (conn_window(eps_max, eps_min, k, &lo, &hi))
      pt_walk(P, up[k], dn[k], lo, hi, [&](bool, bool ok, uint64_t, uint64_t) {
        tot += __popc(__ballot_sync(kFull, ok));
      });
    if (lane == 0) cnt[k] = tot;
  }
}

__global__ void __launch_bounds__(kConnWarps * 32)
    k_conn_emit(SelParams P, const uint64_t* __restrict__ up, const uint64_t* __restrict__ dn,
                const double* __restrict__ eps_max, const double* __restrict__ eps_min,
                uint32_t n, const uint64_t* __restrict__ off, uint64_t* out_up,
                uint64_t* out_dn, uint8_t* out_nx) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t wpg = gridDim.x * kConnWarps;
  for (uint32_t k = blockIdx.x * kConnWarps + (threadIdx.x >> 5); k < n; k += wpg) {
    double lo, hi;
    if (!conn_window(eps_max, eps_min, k, &lo, &hi)) continue;
    const uint64_t u = up[k], d = dn[k];
    uint64_t pos = off[k];
    pt_walk(P, u, d, lo, hi, [&](bool, bool ok, uint64_t cu, uint64_t cd) {
      const unsigned bal = __ballot_sync(kFull, ok);
      if (ok) {
        const uint64_t q = pos + __popc(bal & lt);
        out_up[q] = cu;
        out_dn[q] = cd;
        out_nx[q] = static_cast<uint8_t>((__popcll(u ^ cu) + __popcll(d ^ cd)) >> 1);
      }
      pos += __popc(bal);
    });
  }
}

SelParams conn_params(shci_ctx* c, DevBuf<uint32_t>& pairs) {
  if (!c->Q.built) upload_queues(c);
  const int n_elecs = static_cast<int>(c->I.n_up + c->I.n_dn);
  std::vector<uint32_t> pr;
  for (int a = 0; a < n_elecs; a++)
    for (int b = a + 1; b < n_elecs; b++) pr.push_back(a | (b << 16));
  pairs.mt = &c->mem;
  pairs.resize(pr.empty() ? 1 : pr.size());
  if (!pr.empty())
    SHCI_CUDA(cudaMemcpyAsync(pairs.p, pr.data(), pr.size() * 4, cudaMemcpyHostToDevice,
                              c->stream));
  SelParams P{};
  P.I = c->dI;
  P.d_off = c->Q.d_off.p;
  P.d_H = c->Q.d_H.p;
  P.d_rs = c->Q.d_rs.p;
  P.s_off = c->Q.s_off.p;
  P.s_S = c->Q.s_S.p;
  P.s_r = c->Q.s_r.p;
  P.pair_tab = pairs.p;
  P.max_hci = c->Q.max_hci;
  P.max_singles = c->Q.max_singles;
  P.n_orbs = c->I.n;
  P.n_up = static_cast<int>(c->I.n_up);
  P.n_elecs = n_elecs;
  P.n_pairs = static_cast<int>(pr.size());
  P.no_doubles = c->has_doubles ? 0 : 1;
  P.inactive = c->inactive_orbs;
  return P;
}

}  // namespace

void find_connected(shci_ctx* c, const uint64_t* up, const uint64_t* dn, const double* eps_max,
                    const double* eps_min, size_t n, uint64_t* offsets, uint64_t* out_up,
                    uint64_t* out_dn, uint8_t* n_excite) {
  if (n == 0) {
    if (offsets) offsets[0] = 0;
    return;
  }
  if (n >= 0xffffffffull) throw ArgError("more than 2^32-1 dets in one call");
  if (!up || !dn || !eps_max || !eps_min || !offsets) throw ArgError("null input pointer");
  const bool emit = out_up != nullptr;
  if (emit && (!out_dn || !n_excite)) throw ArgError("null output pointer");
  const int n_up = static_cast<int>(c->I.n_up), n_dn = static_cast<int>(c->I.n_dn);
  for (size_t k = 0; k < n; k++)
    if (__builtin_popcountll(up[k]) != n_up || __builtin_popcountll(dn[k]) != n_dn)
      throw ArgError("det " + std::to_string(k) + " does not have the system's electron counts");
  cudaStream_t s = c->stream;
  DevBuf<uint32_t> pairs;
  const SelParams P = conn_params(c, pairs);
  DevBuf<uint64_t> d_up, d_dn, d_cnt;
  DevBuf<double> d_hi, d_lo;
  d_up.mt = d_dn.mt = d_cnt.mt = &c->mem;
  d_hi.mt = d_lo.mt = &c->mem;
  d_up.resize(n);
  d_dn.resize(n);
  d_hi.resize(n);
  d_lo.resize(n);
  d_cnt.resize(n + 1);
  SHCI_CUDA(cudaMemcpyAsync(d_up.p, up, n * 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(d_dn.p, dn, n * 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(d_hi.p, eps_max, n * 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(d_lo.p, eps_min, n * 8, cudaMemcpyHostToDevice, s));
  int sms = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const unsigned grid = grid_for((size_t)n * 32, kConnWarps * 32, (unsigned)sms * 8u);
  const uint32_t n32 = static_cast<uint32_t>(n);
  if (!emit) {
    k_conn_count<<<grid, kConnWarps * 32, 0, s>>>(P, d_up.p, d_dn.p, d_hi.p, d_lo.p, n32,
                                                   d_cnt.p);
    SHCI_LAUNCH_CHECK();
    std::vector<uint64_t> cnt(n);
    SHCI_CUDA(cudaMemcpyAsync(cnt.data(), d_cnt.p, n * 8, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    offsets[0] = 0;
    for (size_t k = 0; k < n; k++) offsets[k + 1] = offsets[k] + cnt[k];
    c->launches += 1;
    return;
  }
  // the emit pass writes each det's list at its offset: the offsets must be the count call's,
  // so the counts are taken again and compared (a region too small would be overrun)
  k_conn_count<<<grid, kConnWarps * 32, 0, s>>>(P, d_up.p, d_dn.p, d_hi.p, d_lo.p, n32,
                                                 d_cnt.p);
  SHCI_LAUNCH_CHECK();
  std::vector<uint64_t> cnt(n);
  SHCI_CUDA(cudaMemcpyAsync(cnt.data(), d_cnt.p, n * 8, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  if (offsets[0] != 0) throw ArgError("offsets[0] must be 0 (pass the count call's offsets)");
  for (size_t k = 0; k < n; k++)
    if (offsets[k + 1] < offsets[k] || offsets[k + 1] - offsets[k] != cnt[k])
      throw ArgError("offsets do not match the connected-det counts (pass the count call's "
                     "offsets)");
  const uint64_t total = offsets[n];
  SHCI_CUDA(cudaMemcpyAsync(d_cnt.p, offsets, (n + 1) * 8, cudaMemcpyHostToDevice, s));
  DevBuf<uint64_t> o_up, o_dn;
  DevBuf<uint8_t> o_nx;
  o_up.mt = o_dn.mt = &c->mem;
  o_nx.mt = &c->mem;
  o_up.resize(total ? total : 1);
  o_dn.resize(total ? total : 1);
  o_nx.resize(total ? total : 1);
  k_conn_emit<<<grid, kConnWarps * 32, 0, s>>>(P, d_up.p, d_dn.p, d_hi.p, d_lo.p, n32, d_cnt.p,
                                                o_up.p, o_dn.p, o_nx.p);
  SHCI_LAUNCH_CHECK();
  if (total) {
    SHCI_CUDA(cudaMemcpyAsync(out_up, o_up.p, total * 8, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaMemcpyAsync(out_dn, o_dn.p, total * 8, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaMemcpyAsync(n_excite, o_nx.p, total, cudaMemcpyDeviceToHost, s));
  }
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 2;
}

}  // namespace shci

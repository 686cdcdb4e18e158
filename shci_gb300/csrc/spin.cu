// <S^2> of the variational wavefunction: ChemSystem::get_s2 (src/chem/chem_system.cc:745-798),
// computed when the config sets "s2" (post_variation, :627-634), from the first state.
//
//   <S^2> = sum_i c_i^2 (n_up/2 - n_doubly_occupied + n_dn/2 + (n_up^2 + n_dn^2)/4
//                        - n_up n_dn / 2)
//         - 2 sum_i sum_(a, b) c_i c_i' perm_up perm_dn
//
// where for det i the pairs (a, b) run over a beta-only orbital a and an alpha-only orbital
// b > a, i' is det i with the alpha electron moved b -> a and the beta electron a -> b (the
// term is skipped when i' is not in the wavefunction), and perm_up, perm_dn are the
// permutation factors of those moves (HalfDet::diff, src/det/half_det.cc:120-206: the parity
// of the electrons strictly between a and b in each string).
//
// A warp per det: the lanes take its (a, b) pairs, look the partner up in the hash set of the
// det list, and the warp's sum plus the diagonal term is the det's share; the shares are then
// summed in a fixed, compensated order (the reference sums in OpenMP reduction order).
#include "ctx.h"
#include "heatbath.cuh"
#include "kernels.h"

namespace shci {

namespace {

// Id of det (u, d) in the hash set of the det list, or -1.
__device__ __forceinline__ long long set_index(const SelParams& P, uint64_t u, uint64_t d) {
  const uint64_t h = set_slot_hash(u, d);
  const uint32_t fp = static_cast<uint32_t>(h >> 32);
  uint64_t p = h & P.set_hash_mask;
  for (uint64_t probe = 0; probe <= P.set_hash_mask; probe++) {
    const unsigned long long v = P.set_hash[p];
    if (v == 0ull) return -1;
    if (static_cast<uint32_t>(v >> 32) == fp) {
      const uint32_t id = static_cast<uint32_t>(v) - 1u;
      if (P.up[id] == u && P.dn[id] == d) return id;
    }
    p = (p + 1) & P.set_hash_mask;
  }
  return -1;
}

__global__ void k_s2(SelParams P, const double* __restrict__ coef, uint32_t n, double nu,
                     double nd, double* __restrict__ out) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  const double diag0 = 0.5 * nu + 0.5 * nd + 0.25 * (nu * nu + nd * nd) - 0.5 * nu * nd;
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const uint64_t up = P.up[i], dn = P.dn[i];
    const double ci = coef[i];
    const uint64_t A = dn & ~up, B = up & ~dn;  // beta-only and alpha-only orbitals
    const uint32_t na = static_cast<uint32_t>(__popcll(A)), nb = static_cast<uint32_t>(__popcll(B));
    double acc = 0.0;
    for (uint32_t t = lane; t < na * nb; t += 32) {
      const int a = nth_bit(A, static_cast<int>(t / nb));
      const int b = nth_bit(B, static_cast<int>(t % nb));
      if (b <= a) continue;
      const uint64_t u2 = (up & ~(1ull << b)) | (1ull << a);
      const uint64_t d2 = (dn & ~(1ull << a)) | (1ull << b);
      const long long id = set_index(P, u2, d2);
      if (id < 0) continue;
      const int par = move_parity(up, a, b) + move_parity(dn, a, b);
      const double v = -2.0 * coef[id] * ci;
      acc += (par & 1) ? -v : v;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if (lane == 0) {
      const double diag = (diag0 - static_cast<double>(__popcll(up & dn))) * (ci * ci);
      out[i] = diag + acc;
    }
  }
}

}  // namespace

double get_s2(shci_ctx* c) {
  sync_dets(c);
  const size_t n = c->up.size();
  if (n == 0) throw ArgError("no dets");
  if (n >= 0xffffffffull) throw ArgError("more than 2^32-1 dets");
  rebuild_det_set(c);
  cudaStream_t s = c->stream;
  SelParams P{};
  P.up = c->d_up.p;
  P.dn = c->d_dn.p;
  P.set_hash = c->set_hash.p;
  P.set_hash_mask = c->set_hash_mask;
  if (!P.set_hash) throw std::logic_error("S^2: the det list has no hash set");
  DevBuf<double> x, out;
  DevBuf<uint64_t> starts;
  x.mt = out.mt = starts.mt = &c->mem;
  x.resize(n);
  out.resize(2);
  starts.resize(2);
  k_s2<<<grid_for(n * 32, 256), 256, 0, s>>>(P, c->d_coef.p, static_cast<uint32_t>(n),
                                              static_cast<double>(c->I.n_up),
                                              static_cast<double>(c->I.n_dn), x.p);
  SHCI_LAUNCH_CHECK();
  const uint64_t st2[2] = {0, n};
  SHCI_CUDA(cudaMemcpyAsync(starts.p, st2, 16, cudaMemcpyHostToDevice, s));
  seg_reduce2(c, x.p, starts.p, 1, n, out.p);
  double h[2];
  SHCI_CUDA(cudaMemcpyAsync(h, out.p, 16, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 2;
  return h[0];
}

}  // namespace shci

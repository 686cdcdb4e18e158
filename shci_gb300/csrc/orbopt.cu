// Orbital-optimisation inputs from the device RDMs: the generalized Fock matrix of
// Optimization::get_generalized_Fock / generalized_Fock_element (src/chem/optimization.cc:
// 620-650, Helgaker 10.8.24) and, on the host side of the ABI, the orbital gradient
// 2 (F_pq - F_qp) of Optimization::gradient (:565-578).
//
//   F(m, n) = sum_q gamma(m, q) h(n, q) + sum_{q,r,s} Gamma(m, r, s, q) (nq|rs)
//
// for orbitals of equal irrep (0 otherwise), with Gamma(p, q, r, s) = <a+_p a+_q a_r a_s> in the
// reference's half storage (pair a = p n + s, pair b = q n + r, element [max(a,b)
// (max(a,b)+1)/2 + min(a,b)], rdm.cc:233-241).  With n_states > 1 the RDMs sum over the states
// (rdm.cc:222-231, 648-657), as the reference's Optimization receives them.
//
// One CTA per (m, n): its threads walk the n^3 terms (q, r, s) with consecutive (r, s) on
// consecutive threads, so the (nq|rs) row of the dense integral table is read coalesced and
// the RDM row (m n + q) from L2; the partial sums reduce in a fixed order (bit-reproducible).
// Work n^5 FP64 multiply-adds: 0.1 G at n = 38, 1.1 G at n = 64.
#include <vector>

#include "ctx.h"
#include "kernels.h"

namespace shci {

namespace {

constexpr int kFockThreads = 256;

__global__ void __launch_bounds__(kFockThreads)
    k_gen_fock(const double* __restrict__ g1, const double* __restrict__ half,
               const double* __restrict__ h1, const double* __restrict__ g2,
               const unsigned* __restrict__ sym, int n, double* __restrict__ F) {
  const int m = blockIdx.x / n, nn = blockIdx.x % n;
  if (sym[m] != sym[nn]) {
    if (threadIdx.x == 0) F[m * n + nn] = 0.0;
    return;
  }
  const size_t n2 = (size_t)n * n, n3 = n2 * n;
  double acc = 0.0;
  for (size_t j = threadIdx.x; j < n3; j += kFockThreads) {
    const size_t q = j / n2, t = j - q * n2;  // t = r n + s
    const size_t a = (size_t)m * n + q;
    const size_t hi = a > t ? a : t, lo = a > t ? t : a;
    acc += half[hi * (hi + 1) / 2 + lo] * g2[((size_t)nn * n + q) * n2 + t];
  }
  // one-body part (:639-641) on the first n threads
  if (threadIdx.x < (unsigned)n) acc += g1[m * n + threadIdx.x] * h1[nn * n + threadIdx.x];
  __shared__ double red[kFockThreads / 32];
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < kFockThreads / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if (threadIdx.x == 0) F[m * n + nn] = v;
  }
}

__global__ void k_add(double* __restrict__ a, const double* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    a[i] += b[i];
}

}  // namespace

void generalized_fock(shci_ctx* c, double* F_host) {
  const int n = c->I.n;
  const size_t nn = (size_t)n * n, hs = nn * (nn + 1) / 2;
  cudaStream_t s = c->stream;
  DevBuf<double> g1, half, t1, th, F;
  DevBuf<unsigned> sym;
  g1.mt = half.mt = t1.mt = th.mt = F.mt = &c->mem;
  sym.mt = &c->mem;
  g1.resize(nn);
  half.resize(hs);
  F.resize(nn);
  sym.resize(n);
  SHCI_CUDA(cudaMemcpyAsync(sym.p, c->I.orb_sym.data(), n * sizeof(unsigned),
                            cudaMemcpyHostToDevice, s));
  sync_dets(c);
  for (unsigned k = 0; k < c->n_states; k++) {  // sum over the states
    if (k) c->d_coef.swap(c->d_xcoef[k - 1]);
    try {
      if (k == 0) {
        rdm1_dev(c, g1.p);
        rdm2_dev(c, half.p);
      } else {
        t1.resize(nn);
        th.resize(hs);
        rdm1_dev(c, t1.p);
        rdm2_dev(c, th.p);
        k_add<<<grid_for(nn, 256), 256, 0, s>>>(g1.p, t1.p, nn);
        SHCI_LAUNCH_CHECK();
        k_add<<<grid_for(hs, 256), 256, 0, s>>>(half.p, th.p, hs);
        SHCI_LAUNCH_CHECK();
        c->launches += 2;
      }
    } catch (...) {
      if (k) c->d_coef.swap(c->d_xcoef[k - 1]);
      throw;
    }
    if (k) c->d_coef.swap(c->d_xcoef[k - 1]);
  }
  {
    ProfScope ps(c->prof, s, "gen_fock");
    k_gen_fock<<<static_cast<unsigned>(nn), kFockThreads, 0, s>>>(g1.p, half.p, c->h1.p, c->g2.p,
                                                                  sym.p, n, F.p);
    SHCI_LAUNCH_CHECK();
  }
  SHCI_CUDA(cudaMemcpyAsync(F_host, F.p, nn * 8, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->prof.flush();
  c->launches += 1;
}

}  // namespace shci

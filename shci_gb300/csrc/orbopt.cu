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
#include <algorithm>
#include <cmath>
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

// 1-RDM and half-stored 2-RDM of the context's wavefunction, summed over the states
// (rdm.cc:222-231).
void state_rdms(shci_ctx* c, DevBuf<double>& g1, DevBuf<double>& half) {
  const int n = c->I.n;
  const size_t nn = (size_t)n * n, hs = nn * (nn + 1) / 2;
  cudaStream_t s = c->stream;
  DevBuf<double> t1, th;
  t1.mt = th.mt = &c->mem;
  sync_dets(c);
  for (unsigned k = 0; k < c->n_states; k++) {
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
}

// F (device, n x n) from the RDMs; also copied to F_host.
void generalized_fock_from(shci_ctx* c, DevBuf<double>& g1, DevBuf<double>& half,
                           DevBuf<double>& F, double* F_host) {
  const int n = c->I.n;
  const size_t nn = (size_t)n * n;
  cudaStream_t s = c->stream;
  DevBuf<unsigned> sym;
  sym.mt = &c->mem;
  sym.resize(n);
  SHCI_CUDA(cudaMemcpyAsync(sym.p, c->I.orb_sym.data(), n * sizeof(unsigned),
                            cudaMemcpyHostToDevice, s));
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

void generalized_fock(shci_ctx* c, double* F_host) {
  const int n = c->I.n;
  const size_t nn = (size_t)n * n, hs = nn * (nn + 1) / 2;
  DevBuf<double> g1, half, F;
  g1.mt = half.mt = F.mt = &c->mem;
  g1.resize(nn);
  half.resize(hs);
  F.resize(nn);
  state_rdms(c, g1, half);
  generalized_fock_from(c, g1, half, F, F_host);
}

// ---------------------------------------------------------------- natural orbitals, rotation
// Optimization::get_natorb_rotation_matrix (optimization.cc:6-79): the 1-RDM diagonalised
// within each irrep; column j of an irrep's block of rot is the eigenvector of its j-th
// largest occupation, occ[inds[i]] = the i-th largest eigenvalue.  Optimization::
// rotate_integrals / rewrite_integrals (:81-240): (pq|rs) -> sum U_ip U_jq U_kr U_ls (ij|kl)
// one index at a time, h -> U^T h U, and the rewritten tables keep, for each 8-fold (2-fold)
// class of equal integrals, the first value of largest magnitude in (p, q, r, s) order, as the
// reference's hash storage does.
namespace {

// out[..., c_axis, ...] = sum_i U[i, c_axis] in[..., i, ...]; stride = n^(3 - axis)
__global__ void k_rot_axis(const double* __restrict__ in, double* __restrict__ out,
                           const double* __restrict__ U, int n, size_t stride) {
  const size_t total = (size_t)n * n * n * n;
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < total;
       id += (size_t)gridDim.x * blockDim.x) {
    const int c = static_cast<int>((id / stride) % n);
    const size_t base = id - (size_t)c * stride;
    double acc = 0.0;
    for (int i = 0; i < n; i++) acc = fma(U[i * n + c], in[base + (size_t)i * stride], acc);
    out[id] = acc;
  }
}

}  // namespace

void natural_orbitals(shci_ctx* c, const double* g1, double* rot, double* occ) {
  const auto& I = c->I;
  const int n = static_cast<int>(I.n);
  unsigned n_irreps = 0;
  for (unsigned s : I.orb_sym) n_irreps = std::max(n_irreps, s);
  std::fill(rot, rot + (size_t)n * n, 0.0);
  for (unsigned irrep = 1; irrep <= n_irreps; irrep++) {
    std::vector<int> inds;
    for (int i = 0; i < n; i++)
      if (I.orb_sym[i] == irrep) inds.push_back(i);
    const int k = static_cast<int>(inds.size());
    if (!k) continue;
    std::vector<double> sub((size_t)k * k), ev(k), evec((size_t)k * k);
    for (int i = 0; i < k; i++)
      for (int j = 0; j < k; j++) sub[i * k + j] = g1[inds[i] * n + inds[j]];
    jacobi_eig(k, sub.data(), k, ev.data(), evec.data());  // ascending
    for (int i = 0; i < k; i++) {
      occ[inds[i]] = ev[k - 1 - i];
      for (int j = 0; j < k; j++) rot[inds[i] * n + inds[j]] = evec[i * k + (k - 1 - j)];
    }
  }
}

void rotate_integrals(shci_ctx* c, const double* rot) {
  auto& I = c->I;
  const int n = static_cast<int>(I.n);
  const size_t n4 = (size_t)n * n * n * n;
  cudaStream_t s = c->stream;
  DevBuf<double> a, b, u;
  a.mt = b.mt = u.mt = &c->mem;
  a.resize(n4);
  b.resize(n4);
  u.resize((size_t)n * n);
  SHCI_CUDA(cudaMemcpyAsync(a.p, I.g2.data(), n4 * 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(u.p, rot, (size_t)n * n * 8, cudaMemcpyHostToDevice, s));
  // p, q, r, s in the reference's order
  const size_t strides[4] = {(size_t)n * n * n, (size_t)n * n, (size_t)n, 1};
  for (int axis = 0; axis < 4; axis++) {
    k_rot_axis<<<grid_for(n4, 256), 256, 0, s>>>(a.p, b.p, u.p, n, strides[axis]);
    SHCI_LAUNCH_CHECK();
    a.swap(b);
  }
  std::vector<double> g(n4);
  SHCI_CUDA(cudaMemcpyAsync(g.data(), a.p, n4 * 8, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 4;
  // h -> U^T h U, first index then second (:175-199), on the host (n^3)
  std::vector<double> t((size_t)n * n, 0.0), h((size_t)n * n, 0.0);
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++) {
      double v = 0.0;
      for (int i = 0; i < n; i++) v += rot[i * n + p] * I.h1[i * n + q];
      t[p * n + q] = v;
    }
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++) {
      double v = 0.0;
      for (int i = 0; i < n; i++) v += rot[i * n + q] * t[p * n + i];
      h[p * n + q] = v;
    }
  // the rewritten tables: one value per class, the first of largest magnitude (:204-240)
  auto c2 = [](size_t x, size_t y) { return x > y ? x * (x + 1) / 2 + y : y * (y + 1) / 2 + x; };
  const size_t nn = (size_t)n * n;
  std::vector<double> cls(c2(nn, nn) + 1, 0.0);
  std::vector<uint8_t> seen(cls.size(), 0);
  auto put = [](double& a, uint8_t& f, double v) {
    if (!f || std::fabs(a) < std::fabs(v)) a = v;
    f = 1;
  };
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++)
      for (int r = 0; r < n; r++)
        for (int s2 = 0; s2 < n; s2++) {
          const size_t key = c2(c2(p, q), c2(r, s2));
          put(cls[key], seen[key], g[((size_t)(p * n + q) * n + r) * n + s2]);
        }
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++)
      for (int r = 0; r < n; r++)
        for (int s2 = 0; s2 < n; s2++)
          I.g2[((size_t)(p * n + q) * n + r) * n + s2] = cls[c2(c2(p, q), c2(r, s2))];
  std::vector<double> cls1(c2(n, n) + 1, 0.0);
  std::vector<uint8_t> seen1(cls1.size(), 0);
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++) put(cls1[c2(p, q)], seen1[c2(p, q)], h[p * n + q]);
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++) I.h1[p * n + q] = cls1[c2(p, q)];
  screen_linear(I);
}


// ---------------------------------------------------------------- Newton-type step inputs
// Optimization::hessian_diagonal / hessian_part / Y_matrix (optimization.cc:605-618, 652-676,
// Helgaker 10.8.50-53) for the parameter pairs (p, q), and fill_rot_matrix_with_parameters
// (:524-563): rot = exp(X), X_pq = -kappa, X_qp = kappa, formed from the eigenvectors W and
// eigenvalues -tau^2 of X^2 as W cos(tau) W^T + W sinc(tau) W^T X.
namespace {

__device__ __forceinline__ double gam(const double* half, int n, int P, int Q, int R, int S) {
  const size_t a = (size_t)P * n + S, b = (size_t)Q * n + R;
  const size_t hi = a > b ? a : b, lo = a > b ? b : a;
  return half[hi * (hi + 1) / 2 + lo];
}

// Y(a, b, c, d) = sum_mn (G(a,c,n,m) + G(a,n,c,m)) (bm|nd) + G(a,m,n,c) (bd|mn)
__device__ __forceinline__ double y_term(const double* half, const double* g2, int n, int a,
                                         int b, int c, int d, int m, int k) {
  const size_t n2 = (size_t)n * n;
  return (gam(half, n, a, c, k, m) + gam(half, n, a, k, c, m)) *
             g2[((size_t)b * n + m) * n2 + (size_t)k * n + d] +
         gam(half, n, a, m, k, c) * g2[((size_t)b * n + d) * n2 + (size_t)m * n + k];
}

__global__ void __launch_bounds__(kFockThreads)
    k_hess_diag(const double* __restrict__ g1, const double* __restrict__ half,
                const double* __restrict__ F, const double* __restrict__ h1,
                const double* __restrict__ g2, int n, const unsigned* __restrict__ pp,
                const unsigned* __restrict__ qq, double* __restrict__ out) {
  const int p = static_cast<int>(pp[blockIdx.x]), q = static_cast<int>(qq[blockIdx.x]);
  double y1 = 0.0, y2 = 0.0, y3 = 0.0;
  for (int t = threadIdx.x; t < n * n; t += kFockThreads) {
    const int m = t / n, k = t % n;
    y1 += y_term(half, g2, n, p, q, p, q, m, k);
    y2 += y_term(half, g2, n, p, q, q, p, m, k);
    y3 += y_term(half, g2, n, q, p, q, p, m, k);
  }
  __shared__ double red[3][kFockThreads / 32];
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    y1 += __shfl_xor_sync(kFull, y1, o);
    y2 += __shfl_xor_sync(kFull, y2, o);
    y3 += __shfl_xor_sync(kFull, y3, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = y1;
    red[1][threadIdx.x >> 5] = y2;
    red[2][threadIdx.x >> 5] = y3;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double Y1 = 0.0, Y2 = 0.0, Y3 = 0.0;
    for (int w = 0; w < kFockThreads / 32; w++) {
      Y1 += red[0][w];
      Y2 += red[1][w];
      Y3 += red[2][w];
    }
    // hessian_part(p,q,p,q) - 2 hessian_part(p,q,q,p) + hessian_part(q,p,q,p)
    const double a = 2 * g1[p * n + p] * h1[q * n + q] - 2 * F[p * n + p] + 2 * Y1;
    const double b = 2 * g1[p * n + q] * h1[q * n + p] + 2 * Y2;
    const double c = 2 * g1[q * n + q] * h1[p * n + p] - 2 * F[q * n + q] + 2 * Y3;
    out[blockIdx.x] = a - 2 * b + c;
  }
}

}  // namespace

void orbital_hessian_diagonal(shci_ctx* c, const unsigned* p, const unsigned* q, size_t n_param,
                              double* hdiag) {
  const int n = c->I.n;
  const size_t nn = (size_t)n * n, hs = nn * (nn + 1) / 2;
  cudaStream_t s = c->stream;
  DevBuf<double> g1, half, F, out;
  DevBuf<unsigned> dp, dq;
  g1.mt = half.mt = F.mt = out.mt = &c->mem;
  dp.mt = dq.mt = &c->mem;
  g1.resize(nn);
  half.resize(hs);
  F.resize(nn);
  state_rdms(c, g1, half);
  std::vector<double> Fh(nn);
  generalized_fock_from(c, g1, half, F, Fh.data());
  if (!n_param) return;
  dp.resize(n_param);
  dq.resize(n_param);
  out.resize(n_param);
  SHCI_CUDA(cudaMemcpyAsync(dp.p, p, n_param * 4, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(dq.p, q, n_param * 4, cudaMemcpyHostToDevice, s));
  k_hess_diag<<<static_cast<unsigned>(n_param), kFockThreads, 0, s>>>(g1.p, half.p, F.p, c->h1.p,
                                                                      c->g2.p, n, dp.p, dq.p,
                                                                      out.p);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaMemcpyAsync(hdiag, out.p, n_param * 8, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 1;
}

void rotation_from_parameters(int n, const unsigned* p, const unsigned* q, const double* kappa,
                              size_t n_param, double* rot) {
  std::vector<double> X((size_t)n * n, 0.0), X2((size_t)n * n, 0.0);
  for (size_t k = 0; k < n_param; k++) {
    X[p[k] * n + q[k]] = -kappa[k];
    X[q[k] * n + p[k]] = kappa[k];
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      double v = 0.0;
      for (int l = 0; l < n; l++) v += X[i * n + l] * X[l * n + j];
      X2[i * n + j] = v;
    }
  std::vector<double> tau2(n), W((size_t)n * n), WX((size_t)n * n, 0.0);
  jacobi_eig(n, X2.data(), n, tau2.data(), W.data());  // W[i * n + k]: component i of vector k
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++) {
      double v = 0.0;
      for (int l = 0; l < n; l++) v += W[l * n + k] * X[l * n + j];
      WX[k * n + j] = v;
    }
  for (int i = 0; i < n * n; i++) rot[i] = 0.0;
  for (int k = 0; k < n; k++) {
    double cs = 1.0, sc = 1.0;
    if (std::fabs(tau2[k]) >= 1e-10) {
      const double tau = std::sqrt(-tau2[k]);
      cs = std::cos(tau);
      sc = std::sin(tau) / tau;
    }
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        rot[i * n + j] += cs * W[i * n + k] * W[j * n + k] + sc * W[i * n + k] * WX[k * n + j];
  }
}

}  // namespace shci

// Uploads of integrals / queues / dets, and batched matrix-element evaluation.
#include <cstring>

#include "ctx.h"
#include "kernels.h"

namespace shci {

namespace {

__global__ void k_widen(const uint32_t* in, uint64_t* out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

__global__ void k_elems(DevIntegrals I, const uint64_t* ui, const uint64_t* di, const uint64_t* uj,
                        const uint64_t* dj, size_t n, double* out) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    if (ui[k] == uj[k] && di[k] == dj[k]) out[k] = h_diag(I, ui[k], di[k]);
    else out[k] = h_offdiag(I, ui[k], di[k], uj[k], dj[k]);
  }
}

template <class T>
void upload(DevBuf<T>& b, const std::vector<T>& v, cudaStream_t s, MemTracker* mt) {
  b.mt = mt;
  b.resize(v.empty() ? 1 : v.size());
  if (!v.empty())
    SHCI_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  b.n = v.size();
}

}  // namespace

void widen_u32_u64(const uint32_t* in, uint64_t* out, size_t n, cudaStream_t s) {
  k_widen<<<grid_for(n, 256), 256, 0, s>>>(in, out, n);
  SHCI_LAUNCH_CHECK();
}

void upload_integrals(shci_ctx* c) {
  const auto& I = c->I;
  const size_t n = I.n;
  std::vector<double> d(n * n * n), x(n * n * n), j(n * n), k(n * n);
  for (size_t a = 0; a < n; a++)
    for (size_t b = 0; b < n; b++) {
      j[a * n + b] = I.g(a, a, b, b);
      k[a * n + b] = I.g(a, b, b, a);
      for (size_t o = 0; o < n; o++) {
        d[(a * n + b) * n + o] = I.g(a, b, o, o);
        x[(a * n + b) * n + o] = I.g(a, o, o, b);
      }
    }
  cudaStream_t s = c->stream;
  upload(c->h1, I.h1, s, &c->mem);
  upload(c->g2, I.g2, s, &c->mem);
  upload(c->dtab, d, s, &c->mem);
  upload(c->xtab, x, s, &c->mem);
  upload(c->jtab, j, s, &c->mem);
  upload(c->ktab, k, s, &c->mem);
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->dI = DevIntegrals{static_cast<int>(n), I.e_core, c->h1.p, c->g2.p, c->dtab.p,
                       c->xtab.p, c->jtab.p, c->ktab.p};
  c->energy_hf = host_diag(I, I.hf_up, I.hf_dn);
}

void upload_queues(shci_ctx* c) {
  HostQueues Q;
  build_queues(c->I, Q);
  cudaStream_t s = c->stream;
  auto& D = c->Q;
  upload(D.d_off, Q.d_off, s, &c->mem);
  upload(D.d_H, Q.d_H, s, &c->mem);
  upload(D.d_rs, Q.d_rs, s, &c->mem);
  upload(D.s_off, Q.s_off, s, &c->mem);
  upload(D.s_S, Q.s_S, s, &c->mem);
  upload(D.s_r, Q.s_r, s, &c->mem);
  SHCI_CUDA(cudaStreamSynchronize(s));
  D.n_pairs = Q.d_off.size() - 1;
  D.max_hci = Q.max_hci;
  D.max_singles = Q.max_singles;
  D.n_hci = Q.d_H.size();
  D.n_singles = Q.s_S.size();
  D.built = true;
}

void sync_dets(shci_ctx* c) {
  if (!c->dets_dirty) return;
  cudaStream_t s = c->stream;
  upload(c->d_up, c->up, s, &c->mem);
  upload(c->d_dn, c->dn, s, &c->mem);
  upload(c->d_coef, c->coefs, s, &c->mem);
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->dets_dirty = false;
}

void hamiltonian_elems(shci_ctx* c, const uint64_t* ui, const uint64_t* di, const uint64_t* uj,
                       const uint64_t* dj, size_t n, double* out) {
  if (n == 0) return;
  cudaStream_t s = c->stream;
  DevBuf<uint64_t> b;
  b.mt = &c->mem;
  b.resize(4 * n);
  DevBuf<double> o;
  o.mt = &c->mem;
  o.resize(n);
  SHCI_CUDA(cudaMemcpyAsync(b.p, ui, n * 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(b.p + n, di, n * 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(b.p + 2 * n, uj, n * 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(b.p + 3 * n, dj, n * 8, cudaMemcpyHostToDevice, s));
  k_elems<<<grid_for(n, 128), 128, 0, s>>>(c->dI, b.p, b.p + n, b.p + 2 * n, b.p + 3 * n, n, o.p);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaMemcpyAsync(out, o.p, n * 8, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 1;
}

}  // namespace shci

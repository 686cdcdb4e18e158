// Uploads of integrals / queues / dets, and batched matrix-element evaluation.
#include <algorithm>
#include <cstring>
#include <vector>

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

// Packed copy of the element store: row i of the source [row_ptr[i], + row_len[i]) goes to
// [ptr[i], ptr[i+1]); values as FP64 (FP64 store, or FP32 value + FP32 residual).
__global__ void k_pack_rows(const uint64_t* __restrict__ row_ptr, const uint32_t* __restrict__ row_len,
                            const uint64_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                            const double* __restrict__ v64, const float* __restrict__ v32,
                            const float* __restrict__ r32, uint32_t n, uint32_t* out_col,
                            double* out_val) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const uint64_t a = row_ptr[i], b = ptr[i];
    for (uint32_t k = lane; k < row_len[i]; k += 32) {
      out_col[b + k] = col[a + k];
      out_val[b + k] = v64 ? v64[a + k]
                           : static_cast<double>(v32[a + k]) + static_cast<double>(r32[a + k]);
    }
  }
}

// Rows rows[k] of the element store into [off[k], off[k+1]) (values as FP64).
__global__ void k_gather_rows(const uint64_t* __restrict__ row_ptr,
                              const uint32_t* __restrict__ row_len,
                              const uint32_t* __restrict__ rows, uint32_t m,
                              const uint64_t* __restrict__ off, const uint32_t* __restrict__ col,
                              const double* __restrict__ v64, const float* __restrict__ v32,
                              const float* __restrict__ r32, uint32_t* out_col, double* out_val) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < m; k += warps) {
    const uint32_t i = rows[k];
    const uint64_t a = row_ptr[i], b = off[k];
    for (uint32_t t = lane; t < row_len[i]; t += 32) {
      out_col[b + t] = col[a + t];
      out_val[b + t] = v64 ? v64[a + t]
                           : static_cast<double>(v32[a + t]) + static_cast<double>(r32[a + t]);
    }
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

void pack_hamiltonian(shci_ctx* c, DevBuf<uint64_t>& ptr, DevBuf<uint32_t>& col,
                      DevBuf<double>& val) {
  const auto& H = c->H;
  const size_t n = H.n;
  cudaStream_t s = c->stream;
  ptr.resize(n + 1);
  widen_u32_u64(H.row_cnt.p, ptr.p, n, s);
  const uint64_t tot = exclusive_scan_u64(ptr.p, ptr.p, n, s, c->sort);
  SHCI_CUDA(cudaMemcpyAsync(ptr.p + n, &tot, 8, cudaMemcpyHostToDevice, s));
  col.resize(tot ? tot : 1);
  val.resize(tot ? tot : 1);
  const bool fp64 = H.precision == SHCI_PREC_FP64;
  k_pack_rows<<<grid_for(n * 32, 256), 256, 0, s>>>(H.row_ptr.p, H.row_cnt.p, ptr.p, H.col.p,
                                                   fp64 ? H.val64.p : nullptr,
                                                   fp64 ? nullptr : H.val32.p,
                                                   fp64 ? nullptr : H.res32.p,
                                                   static_cast<uint32_t>(n), col.p, val.p);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->launches += 2;
}

void get_rows(shci_ctx* c, const uint64_t* rows, size_t m, uint64_t* offsets, uint32_t* cols,
              double* vals) {
  const auto& H = c->H;
  if (!H.valid) throw ArgError("no Hamiltonian built");
  const size_t n = H.n;
  for (size_t k = 0; k < m; k++)
    if (rows[k] >= n) throw ArgError("row index out of range");
  cudaStream_t s = c->stream;
  const auto segs = segments(H);
  const bool fp64 = H.precision == SHCI_PREC_FP64;
  // per segment: the requested rows' lengths (rows beyond a segment's range are empty)
  std::vector<std::vector<uint64_t>> soff(segs.size(), std::vector<uint64_t>(m + 1, 0));
  for (size_t g = 0; g < segs.size(); g++) {
    std::vector<uint32_t> len(segs[g].n);
    if (segs[g].n)
      SHCI_CUDA(cudaMemcpyAsync(len.data(), segs[g].row_cnt, segs[g].n * 4,
                                cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    for (size_t k = 0; k < m; k++)
      soff[g][k + 1] = soff[g][k] + (rows[k] < segs[g].n ? len[rows[k]] : 0u);
  }
  offsets[0] = 0;
  for (size_t k = 0; k < m; k++) {
    uint64_t l = 0;
    for (size_t g = 0; g < segs.size(); g++) l += soff[g][k + 1] - soff[g][k];
    offsets[k + 1] = offsets[k] + l;
  }
  if (!cols && !vals) return;
  if (m == 0 || offsets[m] == 0) return;
  // gather each segment's part of the rows, then merge per row in increasing column order
  std::vector<std::vector<uint32_t>> hc(segs.size());
  std::vector<std::vector<double>> hv(segs.size());
  for (size_t g = 0; g < segs.size(); g++) {
    const uint64_t tot = soff[g][m];
    if (tot == 0) continue;
    std::vector<uint32_t> r32;
    std::vector<uint64_t> o;
    for (size_t k = 0; k < m; k++)
      if (rows[k] < segs[g].n) {
        r32.push_back(static_cast<uint32_t>(rows[k]));
        o.push_back(soff[g][k]);
      }
    o.push_back(tot);
    DevBuf<uint32_t> d_rows, o_col;
    DevBuf<uint64_t> d_off;
    DevBuf<double> o_val;
    d_rows.mt = o_col.mt = &c->mem;
    d_off.mt = &c->mem;
    o_val.mt = &c->mem;
    d_rows.resize(r32.size());
    d_off.resize(o.size());
    o_col.resize(tot);
    o_val.resize(tot);
    SHCI_CUDA(cudaMemcpyAsync(d_rows.p, r32.data(), r32.size() * 4, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(d_off.p, o.data(), o.size() * 8, cudaMemcpyHostToDevice, s));
    k_gather_rows<<<grid_for(r32.size() * 32, 256), 256, 0, s>>>(
        segs[g].row_ptr, segs[g].row_cnt, d_rows.p, static_cast<uint32_t>(r32.size()), d_off.p,
        segs[g].col, fp64 ? segs[g].val64 : nullptr, fp64 ? nullptr : segs[g].val32,
        fp64 ? nullptr : segs[g].res32, o_col.p, o_val.p);
    SHCI_LAUNCH_CHECK();
    hc[g].resize(tot);
    hv[g].resize(tot);
    SHCI_CUDA(cudaMemcpyAsync(hc[g].data(), o_col.p, tot * 4, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaMemcpyAsync(hv[g].data(), o_val.p, tot * 8, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    c->launches += 1;
  }
  std::vector<std::pair<uint32_t, double>> row;
  for (size_t k = 0; k < m; k++) {
    row.clear();
    for (size_t g = 0; g < segs.size(); g++)
      for (uint64_t t = soff[g][k]; t < soff[g][k + 1]; t++) row.emplace_back(hc[g][t], hv[g][t]);
    std::sort(row.begin(), row.end(),
              [](const std::pair<uint32_t, double>& a, const std::pair<uint32_t, double>& b) {
                return a.first < b.first;
              });
    for (size_t t = 0; t < row.size(); t++) {
      if (cols) cols[offsets[k] + t] = row[t].first;
      if (vals) vals[offsets[k] + t] = row[t].second;
    }
  }
}

void upload_integrals(shci_ctx* c) {
  const auto& I = c->I;
  const size_t n = I.n;
  c->dfix_valid = false;  // also marks the single-excitation tables (built with it)
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
  std::vector<double> stot(Q.s_off.size() - 1, 0.0), dtot(Q.d_off.size() - 1, 0.0);
  for (size_t p = 0; p + 1 < Q.s_off.size(); p++)
    for (size_t e = Q.s_off[p]; e < Q.s_off[p + 1]; e++) stot[p] += Q.s_S[e];
  for (size_t pq = 0; pq + 1 < Q.d_off.size(); pq++)
    for (size_t e = Q.d_off[pq]; e < Q.d_off[pq + 1]; e++) dtot[pq] += Q.d_H[e];
  upload(D.s_tot, stot, s, &c->mem);
  upload(D.d_tot, dtot, s, &c->mem);
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

// One- and two-body reduced density matrices of the variational wavefunction (K8): the
// adjoint of the energy, dE_var/dh and dE_var/dg.
//
// Reference: RDM::get_1rdm (src/chem/rdm.cc:12-131), RDM::get_2rdm over the Hamiltonian
// connections (:333-371, 397-433), get_2rdm_elements (:435-642), permfac_ccaa (:243-269) and
// the half storage of write_in_2rdm / combine4_2rdm (:233-241, 644-657); time_sym = false.
//  1-RDM: a thread per det i visits every single excitation p -> r of the same symmetry
//         (r = p included), finds the target det by binary search in the sorted det list and
//         accumulates c_i c_j sign into a per-block n x n tile in shared memory; the block
//         tiles are summed in a fixed order.
//  2-RDM: a warp per row walks the row's stored connections (diagonal included, as the
//         reference's connection lists do) and applies the reference's case table, adding
//         c_i c_j f into the half-stored array (a = p n + s, b = q n + r, kept when a >= b)
//         with FP64 atomics (the array is L2 resident for the sizes of interest).
#include <cmath>

#include "ctx.h"
#include "heatbath.cuh"
#include "kernels.h"

namespace shci {

namespace {

constexpr int kRdmBlocks = 304;

__device__ __forceinline__ int parity_move(uint64_t h, int p, uint64_t nh, int r) {
  // sign of src/det/half_det.cc:120-206 for h -> nh moving p -> r
  return ((popc64(h & below(p)) + popc64(nh & below(r))) & 1) ? -1 : 1;
}

__global__ void __launch_bounds__(256)
    k_rdm1(const uint64_t* up, const uint64_t* dn, const double* coef, uint32_t n_dets,
           const unsigned* orb_sym, int n, const uint64_t* set_up, const uint64_t* set_dn,
           const uint32_t* set_perm, double* partial) {
  extern __shared__ double tile[];
  for (int k = threadIdx.x; k < n * n; k += blockDim.x) tile[k] = 0.0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_dets; i += gridDim.x * blockDim.x) {
    const uint64_t u = up[i], d = dn[i];
    const double ci = coef[i];
    for (int spin = 0; spin < 2; spin++) {
      const uint64_t h = spin ? d : u;
      for (uint64_t m = h; m; m &= m - 1) {
        const int p = ctz64(m);
        for (int r = 0; r < n; r++) {
          if (orb_sym[p] != orb_sym[r]) continue;
          if (p != r && (h >> r & 1)) continue;
          const uint64_t nh = (h & ~(1ull << p)) | (1ull << r);
          const uint64_t tu = spin ? u : nh, td = spin ? nh : d;
          uint32_t lo = 0, hi = n_dets;
          while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            const uint64_t su = set_up[mid], sd = set_dn[mid];
            if (su < tu || (su == tu && sd < td)) lo = mid + 1;
            else hi = mid;
          }
          if (lo >= n_dets || set_up[lo] != tu || set_dn[lo] != td) continue;
          const uint32_t j = set_perm[lo];
          atomicAdd(&tile[p * n + r], ci * coef[j] * parity_move(h, p, nh, r));
        }
      }
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n * n; k += blockDim.x)
    partial[(size_t)blockIdx.x * n * n + k] = tile[k];
}

__global__ void k_rdm1_sum(const double* partial, int nb, int nn, double* out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nb; b++) s += partial[(size_t)b * nn + k];
    out[k] = s;
  }
}

struct Rdm2Writer {
  double* half;
  int n;
  double cc;  // c_i c_j
  __device__ __forceinline__ void operator()(int p, int q, int r, int s, double f) const {
    const uint64_t a = (uint64_t)p * n + s, b = (uint64_t)q * n + r;
    if (a >= b) atomicAdd(&half[a * (a + 1) / 2 + b], cc * f);
  }
};

__device__ __forceinline__ int bit_till(uint64_t h, int p) { return popc64(h & below(p)); }

// rdm.cc:243-269
__device__ __forceinline__ int permfac_ccaa(uint64_t h, int p, int q, int r, int s) {
  int c = bit_till(h, s);
  h &= ~(1ull << s);
  c += bit_till(h, r);
  h &= ~(1ull << r);
  c += bit_till(h, q);
  h |= 1ull << q;
  c += bit_till(h, p);
  return (c & 1) ? -1 : 1;
}

// diff(a, b) of one spin string: left = in a only, right = in b only (ascending), sign
struct Diff1 {
  int n;
  int l0, l1, r0, r1;
  int perm;
};
__device__ __forceinline__ Diff1 diff1(uint64_t a, uint64_t b) {
  Diff1 d{};
  const uint64_t x = a ^ b;
  d.n = popc64(x) >> 1;
  if (d.n == 0 || d.n > 2) {
    d.perm = 1;
    return d;
  }
  const uint64_t la = a & x, rb = b & x;
  d.l0 = ctz64(la);
  d.r0 = ctz64(rb);
  int par = bit_till(a, d.l0) + bit_till(b, d.r0);
  if (d.n == 2) {
    d.l1 = ctz64(la & (la - 1));
    d.r1 = ctz64(rb & (rb - 1));
    par += bit_till(a, d.l1) + bit_till(b, d.r1);
  }
  d.perm = (par & 1) ? -1 : 1;
  return d;
}

// get_2rdm_elements (rdm.cc:435-642) for this det (tu, td) and connected det (cu, cd), tr = 1
__device__ void rdm2_elements(uint64_t cu, uint64_t cd, uint64_t tu, uint64_t td,
                              const Rdm2Writer& W) {
  const double tr = 1.0;
  if (tu == cu) {
    if (td == cd) {
      for (uint64_t m = tu; m; m &= m - 1) {
        const int s = ctz64(m);
        for (uint64_t m2 = m & (m - 1); m2; m2 &= m2 - 1) {
          const int r = ctz64(m2);
          W(s, r, r, s, tr);
          W(s, r, s, r, -tr);
          W(r, s, s, r, tr);
          W(r, s, r, s, -tr);
        }
      }
      for (uint64_t m = td; m; m &= m - 1) {
        const int s = ctz64(m);
        for (uint64_t m2 = m & (m - 1); m2; m2 &= m2 - 1) {
          const int r = ctz64(m2);
          W(s, r, r, s, tr);
          W(s, r, s, r, -tr);
          W(r, s, s, r, tr);
          W(r, s, r, s, -tr);
        }
      }
      for (uint64_t m = tu; m; m &= m - 1) {
        const int s = ctz64(m);
        for (uint64_t m2 = td; m2; m2 &= m2 - 1) {
          const int r = ctz64(m2);
          W(s, r, r, s, tr);
          W(r, s, s, r, tr);
        }
      }
      return;
    }
    const Diff1 dc = diff1(cd, td), dt = diff1(td, cd);
    if (dc.n == 1) {
      const int b1 = dc.r0, b2 = dc.l0;
      for (uint64_t m = td; m; m &= m - 1) {
        const int p = ctz64(m);
        if (p != b1 && p != b2) {
          double sf = tr * permfac_ccaa(td, p, b2, b1, p);
          W(p, b2, b1, p, sf);
          W(b2, p, b1, p, -sf);
          W(p, b2, p, b1, -sf);
          W(b2, p, p, b1, sf);
          sf = tr * permfac_ccaa(cd, p, b1, b2, p);
          W(p, b1, b2, p, sf);
          W(b1, p, b2, p, -sf);
          W(p, b1, p, b2, -sf);
          W(b1, p, p, b2, sf);
        }
      }
      for (uint64_t m = tu; m; m &= m - 1) {
        const int p = ctz64(m);
        double sf = tr * dc.perm;
        W(p, b2, b1, p, sf);
        W(b2, p, p, b1, sf);
        sf = tr * dt.perm;
        W(p, b1, b2, p, sf);
        W(b1, p, p, b2, sf);
      }
    } else if (dc.n == 2) {
      const int b1 = dc.r0, b2 = dc.r1, b3 = dc.l0, b4 = dc.l1;
      double sf = tr * dc.perm;
      W(b3, b4, b2, b1, sf);
      W(b3, b4, b1, b2, -sf);
      W(b4, b3, b2, b1, -sf);
      W(b4, b3, b1, b2, sf);
      sf = tr * dt.perm;
      W(b1, b2, b4, b3, sf);
      W(b1, b2, b3, b4, -sf);
      W(b2, b1, b4, b3, -sf);
      W(b2, b1, b3, b4, sf);
    }
    return;
  }
  const Diff1 cuD = diff1(cu, tu), tuD = diff1(tu, cu);
  if (cuD.n == 1) {
    if (td == cd) {
      const int a1 = cuD.r0, a2 = cuD.l0;
      for (uint64_t m = tu; m; m &= m - 1) {
        const int p = ctz64(m);
        if (p != a1 && p != a2) {
          double sf = tr * permfac_ccaa(tu, p, a2, a1, p);
          W(p, a2, a1, p, sf);
          W(p, a2, p, a1, -sf);
          W(a2, p, a1, p, -sf);
          W(a2, p, p, a1, sf);
          sf = tr * permfac_ccaa(cu, p, a1, a2, p);
          W(p, a1, a2, p, sf);
          W(p, a1, p, a2, -sf);
          W(a1, p, a2, p, -sf);
          W(a1, p, p, a2, sf);
        }
      }
      for (uint64_t m = td; m; m &= m - 1) {
        const int p = ctz64(m);
        double sf = tr * cuD.perm;
        W(a2, p, p, a1, sf);
        W(p, a2, a1, p, sf);
        sf = tr * tuD.perm;
        W(a1, p, p, a2, sf);
        W(p, a1, a2, p, sf);
      }
    } else {
      const Diff1 cdD = diff1(cd, td), tdD = diff1(td, cd);
      if (cdD.n == 1) {
        const int a1 = cuD.r0, a2 = cuD.l0, b1 = cdD.r0, b2 = cdD.l0;
        double sf = tr * cuD.perm * cdD.perm;
        W(a2, b2, b1, a1, sf);
        W(b2, a2, a1, b1, sf);
        sf = tr * tuD.perm * tdD.perm;
        W(a1, b1, b2, a2, sf);
        W(b1, a1, a2, b2, sf);
      }
    }
  } else if (cuD.n == 2) {
    if (td == cd) {
      const int a1 = cuD.r0, a2 = cuD.r1, a3 = cuD.l0, a4 = cuD.l1;
      double sf = tr * cuD.perm;
      W(a3, a4, a2, a1, sf);
      W(a3, a4, a1, a2, -sf);
      W(a4, a3, a2, a1, -sf);
      W(a4, a3, a1, a2, sf);
      sf = tr * tuD.perm;
      W(a1, a2, a4, a3, sf);
      W(a1, a2, a3, a4, -sf);
      W(a2, a1, a4, a3, -sf);
      W(a2, a1, a3, a4, sf);
    }
  }
}

__global__ void __launch_bounds__(256)
    k_rdm2(const uint64_t* up, const uint64_t* dn, const double* coef, uint32_t n_dets,
           const uint64_t* row_ptr, const uint32_t* row_len, const uint32_t* col, int n,
           bool with_diag, double* half) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n_dets; i += warps) {
    const uint64_t tu = up[i], td = dn[i];
    const double ci = coef[i];
    if (with_diag && lane == 0) rdm2_elements(tu, td, tu, td, Rdm2Writer{half, n, ci * ci});
    for (uint64_t k = row_ptr[i] + lane; k < row_ptr[i] + row_len[i]; k += 32) {
      const uint32_t j = col[k];
      rdm2_elements(up[j], dn[j], tu, td, Rdm2Writer{half, n, ci * coef[j]});
    }
  }
}

// sorted (up, dn) list with the det index of each sorted position
void sorted_set_with_perm(shci_ctx* c, DevBuf<uint64_t>& su, DevBuf<uint64_t>& sd,
                          DevBuf<uint32_t>& perm) {
  const size_t n = c->up.size();
  cudaStream_t s = c->stream;
  su.resize(n);
  sd.resize(n);
  perm.resize(n);
  c->k0.resize(n, 1.25);
  SHCI_CUDA(cudaMemcpyAsync(c->k0.p, c->d_dn.p, n * 8, cudaMemcpyDeviceToDevice, s));
  iota_u32(c->u0.p, n, s);
  radix_sort_pairs(c->k0, c->u0, n, 0, c->I.n, s, c->sort);
  gather_u64(c->d_up.p, c->u0.p, c->k0.p, n, s);
  radix_sort_pairs(c->k0, c->u0, n, 0, c->I.n, s, c->sort);
  SHCI_CUDA(cudaMemcpyAsync(su.p, c->k0.p, n * 8, cudaMemcpyDeviceToDevice, s));
  gather_u64(c->d_dn.p, c->u0.p, sd.p, n, s);
  SHCI_CUDA(cudaMemcpyAsync(perm.p, c->u0.p, n * 4, cudaMemcpyDeviceToDevice, s));
  c->launches += 6;
}

}  // namespace

void rdm1(shci_ctx* c, double* out) {
  const int n = c->I.n;
  DevBuf<double> res;
  res.mt = &c->mem;
  res.resize((size_t)n * n);
  rdm1_dev(c, res.p);
  SHCI_CUDA(cudaMemcpyAsync(out, res.p, (size_t)n * n * 8, cudaMemcpyDeviceToHost, c->stream));
  SHCI_CUDA(cudaStreamSynchronize(c->stream));
}

void rdm1_dev(shci_ctx* c, double* res_dev) {
  sync_dets(c);
  const size_t n_dets = c->up.size();
  const int n = c->I.n;
  cudaStream_t s = c->stream;
  c->u0.reserve(n_dets, 1.25);
  DevBuf<uint64_t> su, sd;
  DevBuf<uint32_t> perm;
  DevBuf<unsigned> sym;
  DevBuf<double> partial;
  su.mt = sd.mt = &c->mem;
  perm.mt = sym.mt = &c->mem;
  partial.mt = &c->mem;
  sorted_set_with_perm(c, su, sd, perm);
  sym.resize(n);
  SHCI_CUDA(cudaMemcpyAsync(sym.p, c->I.orb_sym.data(), n * sizeof(unsigned), cudaMemcpyHostToDevice, s));
  partial.resize((size_t)kRdmBlocks * n * n);
  {
    ProfScope ps(c->prof, s, "rdm1");
    k_rdm1<<<kRdmBlocks, 256, (size_t)n * n * sizeof(double), s>>>(
        c->d_up.p, c->d_dn.p, c->d_coef.p, (uint32_t)n_dets, sym.p, n, su.p, sd.p, perm.p,
        partial.p);
    SHCI_LAUNCH_CHECK();
    k_rdm1_sum<<<grid_for((size_t)n * n, 256), 256, 0, s>>>(partial.p, kRdmBlocks, n * n, res_dev);
    SHCI_LAUNCH_CHECK();
  }
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->prof.flush();
  c->launches += 2;
}

void rdm2(shci_ctx* c, double* out_half) {
  const size_t nn = (size_t)c->I.n * c->I.n, size = nn * (nn + 1) / 2;
  DevBuf<double> half;
  half.mt = &c->mem;
  half.resize(size);
  rdm2_dev(c, half.p);
  SHCI_CUDA(cudaMemcpyAsync(out_half, half.p, size * 8, cudaMemcpyDeviceToHost, c->stream));
  SHCI_CUDA(cudaStreamSynchronize(c->stream));
}

void rdm2_dev(shci_ctx* c, double* half_dev) {
  auto& H = c->H;
  if (!H.valid || H.n != c->up.size()) throw ArgError("the 2-RDM needs the current Hamiltonian");
  sync_dets(c);
  const int n = c->I.n;
  const size_t nn = (size_t)n * n, size = nn * (nn + 1) / 2;
  cudaStream_t s = c->stream;
  SHCI_CUDA(cudaMemsetAsync(half_dev, 0, size * 8, s));
  int sms = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  {
    ProfScope ps(c->prof, s, "rdm2");
    const auto segs = segments(H);
    for (size_t k = 0; k < segs.size(); k++) {
      const SegView& g = segs[k];
      // diagonal terms once, with the current segment (which covers every row)
      k_rdm2<<<static_cast<unsigned>(sms) * 8u, 256, 0, s>>>(
          c->d_up.p, c->d_dn.p, c->d_coef.p, (uint32_t)g.n, g.row_ptr, g.row_cnt, g.col, n,
          k + 1 == segs.size(), half_dev);
      SHCI_LAUNCH_CHECK();
      c->launches += 1;
    }
  }
  SHCI_CUDA(cudaStreamSynchronize(s));
  c->prof.flush();
  c->launches += 1;
}

}  // namespace shci

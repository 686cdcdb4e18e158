// Davidson eigensolver on the device (K5).
//
// Follows Davidson::diagonalize (src/solver/davidson.cc:8-196).  davidson(): n_states = 1, at
// most five stored vectors, a restart that collapses onto the current Ritz vector, the
// diagonal preconditioner with the 1e-8 cut, Gram-Schmidt, the <= 5x5 subspace eigenproblem
// (solved on the host in FP64 by cyclic Jacobi) with the Ritz vector's first component made
// non-negative, and convergence |lambda - lambda_prev| <= tol.  davidson_states(): the same
// for n_states > 1 (5 n_states stored vectors, one preconditioned vector per step for the
// states in turn, a subspace solve after the last state's vector, convergence state by state).
// All vector work is FP64 on the device; dot products reduce in a fixed order so results do
// not depend on timing.
#include <algorithm>
#include <cmath>
#include <numeric>

#include "ctx.h"
#include "kernels.h"

namespace shci {

namespace {

constexpr int kDotBlocks = 304;
constexpr int kDotThreads = 256;

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double s[kDotThreads / 32];
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < kDotThreads / 32 ? s[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(kFull, t, o);
  }
  __syncthreads();
  return t;
}

struct Ptrs6 {
  const double* p[6];
};

// partial[m * kDotBlocks + b] = block b's share of <x, ys[m]>
__global__ void __launch_bounds__(kDotThreads)
    k_mdot_partial(const double* __restrict__ x, Ptrs6 ys, int m, size_t n,
                   double* __restrict__ partial) {
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double xi = x[i];
    for (int k = 0; k < m; k++) acc[k] += xi * ys.p[k][i];
  }
  for (int k = 0; k < m; k++) {
    const double t = block_sum(acc[k]);
    if (threadIdx.x == 0) partial[k * kDotBlocks + blockIdx.x] = t;
  }
}

__global__ void k_mdot_final(const double* __restrict__ partial, int m, double* out) {
  for (int k = 0; k < m; k++) {
    double v = 0.0;
    for (int b = threadIdx.x; b < kDotBlocks; b += blockDim.x) v += partial[k * kDotBlocks + b];
    const double t = block_sum(v);
    if (threadIdx.x == 0) out[k] = t;
  }
}

// v -= (*coef) * u
__global__ void k_axpy_dev(double* __restrict__ v, const double* __restrict__ u,
                           const double* __restrict__ coef, size_t n) {
  const double a = *coef;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    v[i] -= a * u[i];
}

__global__ void k_scale(double* __restrict__ v, double s, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    v[i] = v[i] / s;
}

// v = (Hw - lambda w) / (lambda - d), 0 where |lambda - d| < 1e-8  (davidson.cc:135-143)
__global__ void k_precond(double* __restrict__ v, const double* __restrict__ Hw,
                          const double* __restrict__ w, const double* __restrict__ diag,
                          double lambda, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double d = lambda - diag[i];
    v[i] = fabs(d) < 1.0e-8 ? 0.0 : (Hw[i] - lambda * w[i]) / d;
  }
}

// w = sum_k e_k v_k, Hw = sum_k e_k Hv_k  (davidson.cc:184-194)
struct Comb {
  const double* v[5];
  const double* hv[5];
  double e[5];
  int k;
};
__global__ void k_combine(double* __restrict__ w, double* __restrict__ hw, Comb cb, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < cb.k; k++) {
      a += cb.v[k][i] * cb.e[k];
      b += cb.hv[k][i] * cb.e[k];
    }
    w[i] = a;
    hw[i] = b;
  }
}

// w = sum_k e_k v_k, Hw = sum_k e_k Hv_k over up to 5 * kMaxStates vectors
struct CombN {
  const double* v[5 * kMaxStates];
  const double* hv[5 * kMaxStates];
  double e[5 * kMaxStates];
  int k;
};
__global__ void k_combine_n(double* __restrict__ w, double* __restrict__ hw, CombN cb, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < cb.k; k++) {
      a += cb.v[k][i] * cb.e[k];
      b += cb.hv[k][i] * cb.e[k];
    }
    w[i] = a;
    hw[i] = b;
  }
}

class Dots {
 public:
  Dots(shci_ctx* c) : c_(c) {
    c->dav.partial.reserve(6 * kDotBlocks);
    c->dav.scal.reserve(16);
  }
  // out_dev[k] = <x, ys[k]>, k < m (stays on the device)
  void mdot(const double* x, std::initializer_list<const double*> ys, size_t n, double* out_dev) {
    Ptrs6 p{};
    int m = 0;
    for (auto y : ys) p.p[m++] = y;
    mdot(x, p, m, n, out_dev);
  }
  void mdot(const double* x, const Ptrs6& p, int m, size_t n, double* out_dev) {
    k_mdot_partial<<<kDotBlocks, kDotThreads, 0, c_->stream>>>(x, p, m, n, c_->dav.partial.p);
    SHCI_LAUNCH_CHECK();
    k_mdot_final<<<1, kDotThreads, 0, c_->stream>>>(c_->dav.partial.p, m, out_dev);
    SHCI_LAUNCH_CHECK();
    c_->launches += 2;
  }
  double dot_host(const double* a, const double* b, size_t n) {
    mdot(a, {b}, n, c_->dav.scal.p);
    double r = 0.0;
    SHCI_CUDA(cudaMemcpyAsync(&r, c_->dav.scal.p, 8, cudaMemcpyDeviceToHost, c_->stream));
    SHCI_CUDA(cudaStreamSynchronize(c_->stream));
    return r;
  }

 private:
  shci_ctx* c_;
};

}  // namespace

// Cyclic Jacobi on the lower triangle of a k x k matrix: eigenvalues ascending, eigenvectors
// in columns (evecs[r*k + c]).
void jacobi_eig(int k, const double* lower, int ld, double* evals, double* evecs) {
  std::vector<double> a(static_cast<size_t>(k) * k), v(static_cast<size_t>(k) * k);
  for (int i = 0; i < k; i++)
    for (int j = 0; j < k; j++) {
      a[i * k + j] = i >= j ? lower[i * ld + j] : lower[j * ld + i];
      v[i * k + j] = i == j ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < k * k; i++) tot += a[i] * a[i];
    for (int i = 0; i < k; i++)
      for (int j = 0; j < k; j++)
        if (i != j) off += a[i * k + j] * a[i * k + j];
    if (off == 0.0 || off <= 1e-30 * tot) break;
    for (int p = 0; p < k; p++)
      for (int q = p + 1; q < k; q++) {
        const double apq = a[p * k + q];
        if (apq == 0.0) continue;
        const double th = (a[q * k + q] - a[p * k + p]) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int r = 0; r < k; r++) {
          const double x = a[r * k + p], y = a[r * k + q];
          a[r * k + p] = cs * x - sn * y;
          a[r * k + q] = sn * x + cs * y;
        }
        for (int r = 0; r < k; r++) {
          const double x = a[p * k + r], y = a[q * k + r];
          a[p * k + r] = cs * x - sn * y;
          a[q * k + r] = sn * x + cs * y;
        }
        for (int r = 0; r < k; r++) {
          const double x = v[r * k + p], y = v[r * k + q];
          v[r * k + p] = cs * x - sn * y;
          v[r * k + q] = sn * x + cs * y;
        }
      }
  }
  std::vector<int> idx(k);
  std::iota(idx.begin(), idx.end(), 0);
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return a[x * k + x] < a[y * k + y]; });
  for (int c = 0; c < k; c++) {
    evals[c] = a[idx[c] * k + idx[c]];
    for (int r = 0; r < k; r++) evecs[r * k + c] = v[r * k + idx[c]];
  }
}

__global__ void k_vec_differs(const double* __restrict__ a, const double* __restrict__ b, size_t n,
                              double* flag) {
  bool d = false;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    d |= __double_as_longlong(a[i]) != __double_as_longlong(b[i]);
  if (__any_sync(kFull, d) && (threadIdx.x & 31) == 0) *flag = 1.0;
}

DavidsonOut davidson(shci_ctx* c, double tol) {
  DavidsonOut out;
  auto& D = c->dav;
  D.ritz = false;
  const size_t n = c->H.n;
  cudaStream_t s = c->stream;
  const unsigned g = grid_for(n, 256, 152 * 16);
  Dots dots(c);
  if (n == 1) {
    SHCI_CUDA(cudaMemcpyAsync(&out.eval, c->H.diag.p, 8, cudaMemcpyDeviceToHost, s));
    const double one = 1.0;
    SHCI_CUDA(cudaMemcpyAsync(c->d_coef.p, &one, 8, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    out.converged = true;
    return out;
  }
  const size_t store = std::min<size_t>(n, 5);
  for (size_t k = 0; k < store; k++) {
    D.v[k].mt = D.Hv[k].mt = &c->mem;
    D.v[k].resize(n, 1.1);
    D.Hv[k].resize(n, 1.1);
  }
  D.w.mt = D.Hw.mt = &c->mem;
  D.w.resize(n, 1.1);
  D.Hw.resize(n, 1.1);
  // v0 = init / |init|
  SHCI_CUDA(cudaMemcpyAsync(D.v[0].p, c->d_coef.p, n * 8, cudaMemcpyDeviceToDevice, s));
  double nrm = std::sqrt(dots.dot_host(D.v[0].p, D.v[0].p, n));
  k_scale<<<g, 256, 0, s>>>(D.v[0].p, nrm, n);
  SHCI_LAUNCH_CHECK();
  spmv(c, D.v[0].p, D.Hv[0].p, false);
  out.n_matvec++;
  double lambda = dots.dot_host(D.v[0].p, D.Hv[0].p, n);
  double hk[5 * 5] = {0};
  hk[0] = lambda;
  SHCI_CUDA(cudaMemcpyAsync(D.w.p, D.v[0].p, n * 8, cudaMemcpyDeviceToDevice, s));
  SHCI_CUDA(cudaMemcpyAsync(D.Hw.p, D.Hv[0].p, n * 8, cudaMemcpyDeviceToDevice, s));
  out.trace.push_back(lambda);
  double lambda_prev = lambda;
  bool converged = false;
  double* scal = D.scal.p;
  for (size_t it = 1; it < store * 2; it++) {
    const size_t ic = it % store;
    if (it >= store && ic == 0) {  // restart (davidson.cc:115-131)
      SHCI_CUDA(cudaMemcpyAsync(D.v[0].p, D.w.p, n * 8, cudaMemcpyDeviceToDevice, s));
      SHCI_CUDA(cudaMemcpyAsync(D.Hv[0].p, D.Hw.p, n * 8, cudaMemcpyDeviceToDevice, s));
      lambda = dots.dot_host(D.v[0].p, D.Hv[0].p, n);
      hk[0] = lambda;
      continue;
    }
    k_precond<<<g, 256, 0, s>>>(D.v[ic].p, D.Hw.p, D.w.p, c->H.diag.p, lambda, n);
    SHCI_LAUNCH_CHECK();
    for (size_t i = 0; i < ic; i++) {  // Gram-Schmidt (davidson.cc:146-152)
      dots.mdot(D.v[ic].p, {D.v[i].p}, n, scal);
      k_axpy_dev<<<g, 256, 0, s>>>(D.v[ic].p, D.v[i].p, scal, n);
      SHCI_LAUNCH_CHECK();
    }
    nrm = std::sqrt(dots.dot_host(D.v[ic].p, D.v[ic].p, n));
    if (nrm < 1e-12) {
      converged = true;
      break;
    }
    k_scale<<<g, 256, 0, s>>>(D.v[ic].p, nrm, n);
    SHCI_LAUNCH_CHECK();
    spmv(c, D.v[ic].p, D.Hv[ic].p, false);
    out.n_matvec++;
    Ptrs6 p{};
    for (size_t i = 0; i <= ic; i++) p.p[i] = D.v[i].p;
    dots.mdot(D.Hv[ic].p, p, (int)ic + 1, n, scal);
    double row[6];
    SHCI_CUDA(cudaMemcpyAsync(row, scal, (ic + 1) * 8, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    for (size_t i = 0; i <= ic; i++) hk[ic * 5 + i] = row[i];
    const int k = static_cast<int>(ic + 1);
    double ev[5], evec[25];
    jacobi_eig(k, hk, 5, ev, evec);
    lambda = ev[0];
    const double factor = evec[0] < 0 ? -1.0 : 1.0;
    Comb cb{};
    cb.k = k;
    for (int i = 0; i < k; i++) {
      cb.v[i] = D.v[i].p;
      cb.hv[i] = D.Hv[i].p;
      cb.e[i] = evec[i * k] * factor;
    }
    k_combine<<<g, 256, 0, s>>>(D.w.p, D.Hw.p, cb, n);
    SHCI_LAUNCH_CHECK();
    c->launches += 4 + 2 * ic;
    out.trace.push_back(lambda);
    if (std::fabs(lambda - lambda_prev) <= tol) converged = true;
    if (!converged) lambda_prev = lambda;
    if (converged) break;
  }
  SHCI_CUDA(cudaMemcpyAsync(c->d_coef.p, D.w.p, n * 8, cudaMemcpyDeviceToDevice, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  D.ritz = true;
  D.ritz_h = c->H.build_id;
  out.eval = lambda;
  out.converged = converged;
  c->prof.flush();
  return out;
}

double* state_coef(shci_ctx* c, unsigned s) {
  return s == 0 ? c->d_coef.p : c->d_xcoef[s - 1].p;
}

// davidson.cc:8-196 for n_states = c->n_states > 1.  The subspace matrix starts with only its
// diagonal set (:62-77); the initial vectors are normalised and orthogonalised in order.
DavidsonStatesOut davidson_states(shci_ctx* c, double tol) {
  DavidsonStatesOut out;
  auto& D = c->dav;
  D.ritz = false;
  const size_t n = c->H.n;
  cudaStream_t s = c->stream;
  const unsigned g = grid_for(n, 256, 152 * 16);
  const unsigned req = c->n_states;
  const unsigned ns = static_cast<unsigned>(std::min<size_t>(n, req));
  out.evals.assign(req, 0.0);
  Dots dots(c);
  if (n == 1) {
    SHCI_CUDA(cudaMemcpyAsync(&out.evals[0], c->H.diag.p, 8, cudaMemcpyDeviceToHost, s));
    const double one = 1.0, zero = 0.0;
    SHCI_CUDA(cudaMemcpyAsync(c->d_coef.p, &one, 8, cudaMemcpyHostToDevice, s));
    for (unsigned k = 1; k < req; k++)
      SHCI_CUDA(cudaMemcpyAsync(state_coef(c, k), &zero, 8, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    out.converged = true;
    return out;
  }
  const size_t nis = std::min<size_t>(n, 5);
  const size_t m = ns * nis;
  for (size_t k = 0; k < m; k++) {
    D.sv[k].mt = D.sHv[k].mt = &c->mem;
    D.sv[k].resize(n, 1.1);
    D.sHv[k].resize(n, 1.1);
  }
  for (unsigned k = 0; k < ns; k++) {
    D.sw[k].mt = D.sHw[k].mt = &c->mem;
    D.sw[k].resize(n, 1.1);
    D.sHw[k].resize(n, 1.1);
  }
  double* scal = D.scal.p;
  auto host_dots = [&](const double* x, const std::vector<const double*>& ys, double* outv) {
    for (size_t b = 0; b < ys.size(); b += 6) {
      Ptrs6 p{};
      const int mm = static_cast<int>(std::min<size_t>(6, ys.size() - b));
      for (int q = 0; q < mm; q++) p.p[q] = ys[b + q];
      dots.mdot(x, p, mm, n, scal);
      SHCI_CUDA(cudaMemcpyAsync(outv + b, scal, mm * 8, cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
    }
  };
  // initial vectors (:44-60)
  for (unsigned k = 0; k < ns; k++) {
    SHCI_CUDA(cudaMemcpyAsync(D.sv[k].p, state_coef(c, k), n * 8, cudaMemcpyDeviceToDevice, s));
    double nrm = std::sqrt(dots.dot_host(D.sv[k].p, D.sv[k].p, n));
    k_scale<<<g, 256, 0, s>>>(D.sv[k].p, nrm, n);
    SHCI_LAUNCH_CHECK();
    if (k > 0) {
      for (unsigned q = 0; q < k; q++) {
        dots.mdot(D.sv[k].p, {D.sv[q].p}, n, scal);
        k_axpy_dev<<<g, 256, 0, s>>>(D.sv[k].p, D.sv[q].p, scal, n);
        SHCI_LAUNCH_CHECK();
      }
      nrm = std::sqrt(dots.dot_host(D.sv[k].p, D.sv[k].p, n));
      k_scale<<<g, 256, 0, s>>>(D.sv[k].p, nrm, n);
      SHCI_LAUNCH_CHECK();
    }
  }
  std::vector<double> hk(m * m, 0.0), lam(ns), lam_prev(ns);
  for (unsigned k = 0; k < ns; k++) {
    spmv(c, D.sv[k].p, D.sHv[k].p, false);
    out.n_matvec++;
    lam[k] = dots.dot_host(D.sv[k].p, D.sHv[k].p, n);
    hk[k * m + k] = lam[k];
    SHCI_CUDA(cudaMemcpyAsync(D.sw[k].p, D.sv[k].p, n * 8, cudaMemcpyDeviceToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(D.sHw[k].p, D.sHv[k].p, n * 8, cudaMemcpyDeviceToDevice, s));
  }
  lam_prev = lam;
  bool converged = false;
  size_t n_conv = 0, pre = 0;
  for (size_t it = ns; it < m * 2; it++) {
    const size_t ic = it % m;
    if (it >= m) {  // restart onto the Ritz vectors (:86-103)
      if (ic < ns - 1) continue;
      if (ic == ns - 1) {
        for (unsigned k = 0; k < ns; k++) {
          SHCI_CUDA(cudaMemcpyAsync(D.sv[k].p, D.sw[k].p, n * 8, cudaMemcpyDeviceToDevice, s));
          SHCI_CUDA(cudaMemcpyAsync(D.sHv[k].p, D.sHw[k].p, n * 8, cudaMemcpyDeviceToDevice, s));
        }
        for (unsigned k = 0; k < ns; k++) {
          lam[k] = dots.dot_host(D.sv[k].p, D.sHv[k].p, n);
          hk[k * m + k] = lam[k];
          for (unsigned q = k + 1; q < ns; q++) {
            const double e = dots.dot_host(D.sv[k].p, D.sHv[q].p, n);
            hk[k * m + q] = e;
            hk[q * m + k] = e;
          }
        }
        continue;
      }
    }
    // preconditioned residual of state `pre` (:133-143)
    k_precond<<<g, 256, 0, s>>>(D.sv[ic].p, D.sHw[pre].p, D.sw[pre].p, c->H.diag.p, lam[pre], n);
    SHCI_LAUNCH_CHECK();
    for (size_t i = 0; i < ic; i++) {  // (:145-152)
      dots.mdot(D.sv[ic].p, {D.sv[i].p}, n, scal);
      k_axpy_dev<<<g, 256, 0, s>>>(D.sv[ic].p, D.sv[i].p, scal, n);
      SHCI_LAUNCH_CHECK();
    }
    const double nrm = std::sqrt(dots.dot_host(D.sv[ic].p, D.sv[ic].p, n));
    if (nrm < 1e-12) {
      converged = true;
      break;
    }
    k_scale<<<g, 256, 0, s>>>(D.sv[ic].p, nrm, n);
    SHCI_LAUNCH_CHECK();
    spmv(c, D.sv[ic].p, D.sHv[ic].p, false);
    out.n_matvec++;
    {  // row ic of the subspace matrix (:163-167)
      std::vector<const double*> ys(ic + 1);
      for (size_t i = 0; i <= ic; i++) ys[i] = D.sv[i].p;
      std::vector<double> row(ic + 1);
      host_dots(D.sHv[ic].p, ys, row.data());
      for (size_t i = 0; i <= ic; i++) hk[ic * m + i] = row[i];
    }
    c->launches += 4 + 2 * ic;
    if (pre + 1 == ns) {  // subspace solve (:169-172) and Ritz vectors (:173-194)
      const int k = static_cast<int>(ic + 1);
      std::vector<double> ev(k), evec(static_cast<size_t>(k) * k);
      jacobi_eig(k, hk.data(), static_cast<int>(m), ev.data(), evec.data());
      for (unsigned st = 0; st < ns; st++) {
        lam[st] = ev[st];
        const double factor = evec[st] < 0 ? -1.0 : 1.0;
        CombN cb{};
        cb.k = k;
        for (int i = 0; i < k; i++) {
          cb.v[i] = D.sv[i].p;
          cb.hv[i] = D.sHv[i].p;
          cb.e[i] = evec[i * k + st] * factor;
        }
        k_combine_n<<<g, 256, 0, s>>>(D.sw[st].p, D.sHw[st].p, cb, n);
        SHCI_LAUNCH_CHECK();
        c->launches += 1;
      }
      for (unsigned st = static_cast<unsigned>(n_conv); st < ns; st++) {  // (:180-186)
        if (std::fabs(lam[st] - lam_prev[st]) > tol) break;
        n_conv++;
      }
      if (n_conv == ns) converged = true;
      if (!converged) lam_prev = lam;
      if (converged) break;
    }
    pre++;
    if (pre >= ns) pre = n_conv;
  }
  for (unsigned k = 0; k < ns; k++) {
    SHCI_CUDA(cudaMemcpyAsync(state_coef(c, k), D.sw[k].p, n * 8, cudaMemcpyDeviceToDevice, s));
    out.evals[k] = lam[k];
  }
  SHCI_CUDA(cudaStreamSynchronize(s));
  out.converged = converged;
  c->prof.flush();
  return out;
}

// Rayleigh quotient of d_coef with value + residual.  When d_coef is still the Ritz vector w
// of the last Davidson call on this (mixed) Hamiltonian, w^T H w = w^T Hw + w^T R w with Hw =
// H32 w kept by Davidson (FP32 values, FP64 diagonal), so only the residual store R is read
// (2 sum_i w_i (R w)_i over its upper triangle: one gather per element, no atomics);
// otherwise H w is formed from value + residual.
double rayleigh_fp64(shci_ctx* c) {
  const size_t n = c->H.n;
  auto& D = c->dav;
  cudaStream_t s = c->stream;
  Dots dots(c);
  if (n > 1 && D.ritz && D.ritz_h == c->H.build_id && c->H.precision != SHCI_PREC_FP64 &&
      D.w.n == n && c->d_coef.n >= n) {
    D.scal.reserve(8);
    SHCI_CUDA(cudaMemsetAsync(D.scal.p, 0, 8, s));
    k_vec_differs<<<grid_for(n, 256, 152 * 8), 256, 0, s>>>(c->d_coef.p, D.w.p, n, D.scal.p);
    SHCI_LAUNCH_CHECK();
    double differs = 0.0;
    SHCI_CUDA(cudaMemcpyAsync(&differs, D.scal.p, 8, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    if (differs == 0.0) {
      D.rt.mt = &c->mem;
      D.rt.resize(n, 1.1);
      residual_rows(c, D.w.p, D.rt.p);
      const double num = dots.dot_host(D.w.p, D.Hw.p, n) + 2.0 * dots.dot_host(D.w.p, D.rt.p, n);
      const double den = dots.dot_host(D.w.p, D.w.p, n);
      c->launches += 1;
      return num / den;
    }
  }
  return rayleigh_fp64_of(c, c->d_coef.p);
}

double rayleigh_fp64_of(shci_ctx* c, const double* x) {
  const size_t n = c->H.n;
  auto& D = c->dav;
  Dots dots(c);
  D.ritz = false;  // Hw is overwritten below
  D.Hw.mt = &c->mem;
  D.Hw.resize(n, 1.1);
  spmv(c, x, D.Hw.p, true);
  const double num = dots.dot_host(x, D.Hw.p, n);
  const double den = dots.dot_host(x, x, n);
  return num / den;
}

}  // namespace shci

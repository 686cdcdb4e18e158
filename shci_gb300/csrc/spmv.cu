// Symmetric sparse H*v over the upper-triangle store (K4).
//
// Replaces SparseMatrix::mul (src/solver/sparse_matrix.cc:28-56): y = H x with H stored as
// its strict upper triangle plus an FP64 diagonal.  One warp per row i streams the row's
// (col, val) pairs once: the row part y_i += H_ij x_j is reduced in registers and the
// transpose part y_j += H_ij x_i goes out as atomics (y is L2 resident).
//
// FP64 storage: FP64 products and FP64 atomics (the exact path).
//
// Mixed storage (FP32 value, optional FP32 residual): GB300 runs FP64 at 1/64 of the FP32
// rate, and one FP64 multiply-add per stored element already made this kernel FP64-bound, so
// the mixed kernel uses no FP64 per element:
//   * x is split into float pairs x = xh + xl (relative error 2^-48);
//   * products v * (xh + xl) are formed as float pairs with an exact FMA error term, so each
//     is accurate to about 2^-47 relative (far below the FP32 rounding of the stored value);
//   * the row part is accumulated as a float pair; each transpose contribution, and each
//     row's total, is converted to a 64-bit fixed-point integer with round-to-nearest and
//     added with an integer atomic.  The fixed-point scale 2^s is chosen per call from the
//     bound B = max_i sum_j |H_ij| * max_i |x_i| >= max_i |y_i| >= any single term, so that
//     B * 2^s < 2^61: every converted term and every final y_i fits, and integer additions
//     (modulo 2^64) are exact and order-independent.  The result does not depend on the
//     order of the atomics, so mixed H*v is bit-reproducible.  The absolute resolution of
//     y is 2^-s ~ B * 2^-61.
// The row abs-sum bound is computed once per matrix (float atomics; inflated by 5% against
// their rounding).
#include <cmath>
#include <cstring>

#include "ctx.h"
#include "kernels.h"

namespace shci {

namespace {

// FP64 store: FP64 products, FP64 atomics.
__global__ void __launch_bounds__(256)
    k_spmv(const uint64_t* __restrict__ row_ptr, const uint32_t* __restrict__ row_len,
           const uint32_t* __restrict__ col, const double* __restrict__ v64,
           const double* __restrict__ diag, const double* __restrict__ x, double* __restrict__ y,
           uint32_t n) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const uint64_t rs = row_ptr[i], re = rs + row_len[i];
    const double xi = x[i];
    double acc = 0.0;
    for (uint64_t k = rs + lane; k < re; k += 32) {
      const uint32_t j = col[k];
      const double v = v64[k];
      acc += v * x[j];
      atomicAdd(&y[j], v * xi);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if (lane == 0) atomicAdd(&y[i], diag ? acc + diag[i] * xi : acc);
  }
}

// ---------------------------------------------------------------- mixed: fixed point
// f * 2^s rounded to the nearest integer (ties away from zero), for |f| * 2^s < 2^63.
// Subnormal floats (< 1.2e-38) count as zero.
__device__ __forceinline__ long long f2fix(float f, int s) {
  const unsigned b = __float_as_uint(f);
  const int ex = static_cast<int>((b >> 23) & 0xffu);
  const unsigned m = ex ? ((b & 0x7fffffu) | 0x800000u) : 0u;  // value = m * 2^(ex - 150)
  const int sh = ex - 150 + s;
  const int rs = min(max(-sh, 1), 30);
  const long long left = static_cast<long long>(m) << max(sh, 0);
  const long long right = static_cast<long long>((m + (1u << (rs - 1))) >> rs);
  const long long r = sh >= 0 ? left : right;
  return (b >> 31) ? -r : r;
}

// Exact float-pair sum (a + b = s + e): Knuth's two-sum.
__device__ __forceinline__ void two_sum(float a, float b, float* s, float* e) {
  const float t = a + b;
  const float z = t - a;
  *e = (a - (t - z)) + (b - z);
  *s = t;
}

// v * (xh + xl) (+ r * xh) as a float pair p + e.
template <bool RES>
__device__ __forceinline__ void prod2(float v, float r, float xh, float xl, float* p, float* e) {
  const float q = v * xh;
  float t = fmaf(v, xh, -q);
  t = fmaf(v, xl, t);
  if (RES) t = fmaf(r, xh, t);
  *p = q;
  *e = t;
}

// Scale exponent s with B * 2^s < 2^61 (B > 0), from the bound's binary exponent.
__device__ __forceinline__ int fix_scale(double B) {
  if (!(B > 0.0)) return 0;
  const int e = static_cast<int>((__double_as_longlong(B) >> 52) & 0x7ff) - 1022;  // B < 2^e
  return 61 - e;
}

// x -> float pairs; max |x| (as ordered bits of a non-negative double) into *xmax_bits.
__global__ void k_split_x(const double* __restrict__ x, uint32_t n, float2* xs,
                          unsigned long long* xmax_bits) {
  unsigned long long mx = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = x[i];
    const float h = static_cast<float>(v);
    const float l = static_cast<float>(v - static_cast<double>(h));
    xs[i] = make_float2(h, l);
    const unsigned long long a = static_cast<unsigned long long>(__double_as_longlong(fabs(v)));
    mx = a > mx ? a : mx;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(kFull, mx, o);
    mx = t > mx ? t : mx;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(xmax_bits, mx);
}

// Off-diagonal row abs sums of the full symmetric matrix, in float.
template <bool RES>
__global__ void __launch_bounds__(256)
    k_rowabs(const uint64_t* __restrict__ row_ptr, const uint32_t* __restrict__ row_len,
             const uint32_t* __restrict__ col,
             const float* __restrict__ v32, const float* __restrict__ r32,
             const double* __restrict__ diag, float* rowabs, uint32_t n) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const uint64_t rs = row_ptr[i], re = rs + row_len[i];
    float acc = 0.0f;
    for (uint64_t k = rs + lane; k < re; k += 32) {
      const float a = fabsf(v32[k]) + (RES ? fabsf(r32[k]) : 0.0f);
      acc += a;
      atomicAdd(&rowabs[col[k]], a);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if (lane == 0) atomicAdd(&rowabs[i], acc);
  }
}

// max_i (rowabs_i + |diag_i|), as the bits of a non-negative float.
__global__ void k_max_bound(const float* __restrict__ a, const double* __restrict__ diag,
                            uint32_t n, unsigned* max_bits) {
  unsigned mx = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    mx = max(mx, __float_as_uint(a[i] + __double2float_ru(fabs(diag[i]))));
#pragma unroll
  for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(max_bits, mx);
}

// Mixed H*v: float-pair products, fixed-point accumulation (off-diagonal part only).
template <bool RES>
__global__ void __launch_bounds__(256)
    k_spmv_fix(const uint64_t* __restrict__ row_ptr, const uint32_t* __restrict__ row_len,
               const uint32_t* __restrict__ col,
               const float* __restrict__ v32, const float* __restrict__ r32,
               const float2* __restrict__ xs, const double* __restrict__ scal,
               unsigned long long* __restrict__ yfix, uint32_t n) {
  const int s = fix_scale(scal[0] * __longlong_as_double(static_cast<long long>(
                                        reinterpret_cast<const unsigned long long*>(scal)[1])));
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const uint64_t rs = row_ptr[i], re = rs + row_len[i];
    const float2 xi = xs[i];
    float ah = 0.0f, al = 0.0f;
    for (uint64_t k = rs + lane; k < re; k += 32) {
      const uint32_t j = col[k];
      const float v = v32[k];
      const float r = RES ? r32[k] : 0.0f;
      const float2 xj = xs[j];
      float p, e, t, te;
      prod2<RES>(v, r, xj.x, xj.y, &p, &e);
      two_sum(ah, p, &t, &te);
      ah = t;
      al += te + e;
      prod2<RES>(v, r, xi.x, xi.y, &p, &e);
      atomicAdd(&yfix[j], static_cast<unsigned long long>(f2fix(p, s) + f2fix(e, s)));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const float bh = __shfl_xor_sync(kFull, ah, o), bl = __shfl_xor_sync(kFull, al, o);
      float t, te;
      two_sum(ah, bh, &t, &te);
      ah = t;
      al = al + bl + te;
    }
    if (lane == 0)
      atomicAdd(&yfix[i], static_cast<unsigned long long>(f2fix(ah, s) + f2fix(al, s)));
  }
}

// y = yfix * 2^-s + diag * x
__global__ void k_fix_out(const unsigned long long* __restrict__ yfix,
                          const double* __restrict__ diag, const double* __restrict__ x,
                          const double* __restrict__ scal, double* __restrict__ y, uint32_t n) {
  const int s = fix_scale(scal[0] * __longlong_as_double(static_cast<long long>(
                                        reinterpret_cast<const unsigned long long*>(scal)[1])));
  const double inv = ldexp(1.0, -s);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = static_cast<double>(static_cast<long long>(yfix[i])) * inv + diag[i] * x[i];
}

}  // namespace

// H.scal[0] = bound on max_i sum_j |H_ij| from the off-diagonal sums in H.rowabs and the
// diagonal; H.rowabs stays (an incremental update adds to it).
void finish_mixed_bound(shci_ctx* c) {
  auto& H = c->H;
  cudaStream_t s = c->stream;
  const uint32_t n = static_cast<uint32_t>(H.n);
  H.scal.resize(4);
  SHCI_CUDA(cudaMemsetAsync(H.scal.p, 0, 4 * 8, s));
  unsigned* mb = reinterpret_cast<unsigned*>(H.scal.p + 2);
  k_max_bound<<<grid_for(n, 256), 256, 0, s>>>(H.rowabs.p, H.diag.p, n, mb);
  SHCI_LAUNCH_CHECK();
  unsigned bits = 0;
  SHCI_CUDA(cudaMemcpyAsync(&bits, mb, 4, cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  float fm;
  std::memcpy(&fm, &bits, 4);
  // float sums of positive terms are within n_terms * 2^-24 relative; 5% covers that
  const double bound = 1.05 * static_cast<double>(fm) + 1e-300;
  SHCI_CUDA(cudaMemcpyAsync(H.scal.p, &bound, 8, cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  H.bound_valid = true;
  c->launches += 1;
}

namespace {

// Row abs-sum bound of a mixed store that was not built with one (a pass over the store).
void mixed_bound(shci_ctx* c, unsigned grid) {
  auto& H = c->H;
  cudaStream_t s = c->stream;
  const uint32_t n = static_cast<uint32_t>(H.n);
  H.rowabs.resize(n, 1.1);
  H.rowabs_hb = false;
  SHCI_CUDA(cudaMemsetAsync(H.rowabs.p, 0, (size_t)n * 4, s));
  for (const SegView& g : segments(H)) {
    k_rowabs<true><<<grid, 256, 0, s>>>(g.row_ptr, g.row_cnt, g.col, g.val32, g.res32, H.diag.p,
                                        H.rowabs.p, static_cast<uint32_t>(g.n));
    SHCI_LAUNCH_CHECK();
    c->launches += 1;
  }
  finish_mixed_bound(c);
}

// t_i += sum over row i's stored elements of residual_ij * w_j (no atomics: the FP64 energy
// correction needs only w^T R w = 2 sum_i w_i t_i of the residual store R).  w comes split
// into float pairs and the products and sums are float pairs, as in the mixed H*v (about
// 2^-44 relative): the FP64 form spent two FP64 operations per element (conversion and FMA),
// more than the gathers cost on GB300.
__global__ void __launch_bounds__(256)
    k_res_rows(const uint64_t* __restrict__ row_ptr, const uint32_t* __restrict__ row_len,
               const uint32_t* __restrict__ col, const float* __restrict__ r32,
               const float2* __restrict__ ws, double* __restrict__ t, uint32_t n) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const uint64_t rs = row_ptr[i], re = rs + row_len[i];
    float ah = 0.0f, al = 0.0f;
    for (uint64_t k = rs + lane; k < re; k += 32) {
      const float2 wj = ws[col[k]];
      float p, e, s2, se;
      prod2<false>(r32[k], 0.0f, wj.x, wj.y, &p, &e);
      two_sum(ah, p, &s2, &se);
      ah = s2;
      al += se + e;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const float bh = __shfl_xor_sync(kFull, ah, o), bl = __shfl_xor_sync(kFull, al, o);
      float s2, se;
      two_sum(ah, bh, &s2, &se);
      ah = s2;
      al = al + bl + se;
    }
    if (lane == 0) t[i] += static_cast<double>(ah) + static_cast<double>(al);
  }
}

}  // namespace

void residual_rows(shci_ctx* c, const double* w, double* t) {
  auto& H = c->H;
  if (!H.valid || H.precision == SHCI_PREC_FP64) throw ArgError("no mixed Hamiltonian built");
  const uint32_t n = static_cast<uint32_t>(H.n);
  int sms = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const unsigned grid = grid_for((size_t)n * 32, 256, (unsigned)sms * 8u);
  cudaStream_t s = c->stream;
  ProfScope ps(c->prof, s, "spmv_res_rows");
  H.xs.resize(2 * (size_t)n, 1.1);
  float2* ws = reinterpret_cast<float2*>(H.xs.p);
  SHCI_CUDA(cudaMemsetAsync(H.scal.p + 1, 0, 8, s));
  k_split_x<<<grid_for(n, 256), 256, 0, s>>>(w, n, ws,
                                             reinterpret_cast<unsigned long long*>(H.scal.p + 1));
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaMemsetAsync(t, 0, (size_t)n * 8, s));
  for (const SegView& g : segments(H)) {
    k_res_rows<<<grid, 256, 0, s>>>(g.row_ptr, g.row_cnt, g.col, g.res32, ws, t,
                                    static_cast<uint32_t>(g.n));
    SHCI_LAUNCH_CHECK();
    c->launches += 1;
  }
  c->launches += 1;
}

void spmv(shci_ctx* c, const double* x, double* y, bool residual) {
  auto& H = c->H;
  if (!H.valid) throw ArgError("no Hamiltonian built");
  cudaStream_t s = c->stream;
  const uint32_t n = static_cast<uint32_t>(H.n);
  int sms = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const unsigned grid = grid_for((size_t)n * 32, 256, (unsigned)sms * 8u);
  if (H.precision == SHCI_PREC_FP64) {
    ProfScope ps(c->prof, s, "spmv");
    SHCI_CUDA(cudaMemsetAsync(y, 0, H.n * sizeof(double), s));
    const auto segs = segments(H);
    for (size_t k = 0; k < segs.size(); k++) {
      const SegView& g = segs[k];
      // the diagonal goes in with the current segment, which covers every row
      k_spmv<<<grid, 256, 0, s>>>(g.row_ptr, g.row_cnt, g.col, g.val64,
                                  k + 1 == segs.size() ? H.diag.p : nullptr, x, y,
                                  static_cast<uint32_t>(g.n));
      SHCI_LAUNCH_CHECK();
      c->launches += 1;
    }
    return;
  }
  if (!H.bound_valid) mixed_bound(c, grid);
  H.xs.resize(2 * (size_t)n, 1.1);
  H.yfix.resize(n, 1.1);
  ProfScope ps(c->prof, s, "spmv");
  SHCI_CUDA(cudaMemsetAsync(H.yfix.p, 0, (size_t)n * 8, s));
  SHCI_CUDA(cudaMemsetAsync(H.scal.p + 1, 0, 8, s));
  float2* xs = reinterpret_cast<float2*>(H.xs.p);
  k_split_x<<<grid_for(n, 256), 256, 0, s>>>(
      x, n, xs, reinterpret_cast<unsigned long long*>(H.scal.p + 1));
  SHCI_LAUNCH_CHECK();
  for (const SegView& g : segments(H)) {
    const uint32_t gn = static_cast<uint32_t>(g.n);
    if (residual)
      k_spmv_fix<true><<<grid, 256, 0, s>>>(g.row_ptr, g.row_cnt, g.col, g.val32, g.res32, xs,
                                             H.scal.p, H.yfix.p, gn);
    else
      k_spmv_fix<false><<<grid, 256, 0, s>>>(g.row_ptr, g.row_cnt, g.col, g.val32, nullptr, xs,
                                              H.scal.p, H.yfix.p, gn);
    SHCI_LAUNCH_CHECK();
    c->launches += 1;
  }
  k_fix_out<<<grid_for(n, 256), 256, 0, s>>>(H.yfix.p, H.diag.p, x, H.scal.p, y, n);
  SHCI_LAUNCH_CHECK();
  c->launches += 2;
}

}  // namespace shci

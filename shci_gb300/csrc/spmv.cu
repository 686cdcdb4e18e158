// Symmetric sparse H*v over the upper-triangle store (K4).
//
// Replaces SparseMatrix::mul (src/solver/sparse_matrix.cc:28-56): y = H x with H stored as
// its strict upper triangle plus an FP64 diagonal.  One warp per row i streams the row's
// (col, val) pairs once: the row part y_i += H_ij x_j is reduced in registers and the
// transpose part y_j += H_ij x_i goes out as FP64 atomics (y is L2 resident for the sizes
// of interest).  Values are FP64 or FP32 (optionally + FP32 residual); products and sums
// are FP64.
#include "ctx.h"
#include "kernels.h"

namespace shci {

namespace {

template <int MODE>  // 0: FP64 values, 1: FP32 values, 2: FP32 value + FP32 residual
__global__ void __launch_bounds__(256)
    k_spmv(const uint64_t* __restrict__ row_ptr, const uint32_t* __restrict__ col,
           const double* __restrict__ v64, const float* __restrict__ v32,
           const float* __restrict__ r32, const double* __restrict__ diag,
           const double* __restrict__ x, double* __restrict__ y, uint32_t n) {
  const unsigned lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const uint64_t rs = row_ptr[i], re = row_ptr[i + 1];
    const double xi = x[i];
    double acc = 0.0;
    for (uint64_t k = rs + lane; k < re; k += 32) {
      const uint32_t j = col[k];
      double v;
      if (MODE == 0) v = v64[k];
      else if (MODE == 1) v = static_cast<double>(v32[k]);
      else v = static_cast<double>(v32[k]) + static_cast<double>(r32[k]);
      acc += v * x[j];
      atomicAdd(&y[j], v * xi);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if (lane == 0) atomicAdd(&y[i], acc + diag[i] * xi);
  }
}

}  // namespace

void spmv(shci_ctx* c, const double* x, double* y, bool residual) {
  auto& H = c->H;
  if (!H.valid) throw ArgError("no Hamiltonian built");
  cudaStream_t s = c->stream;
  const uint32_t n = static_cast<uint32_t>(H.n);
  ProfScope ps(c->prof, s, "spmv");
  SHCI_CUDA(cudaMemsetAsync(y, 0, H.n * sizeof(double), s));
  int sms = 0;
  SHCI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const unsigned grid = grid_for((size_t)n * 32, 256, (unsigned)sms * 8u);
  if (H.precision == SHCI_PREC_FP64) {
    k_spmv<0><<<grid, 256, 0, s>>>(H.row_ptr.p, H.col.p, H.val64.p, nullptr, nullptr, H.diag.p,
                                   x, y, n);
  } else if (!residual) {
    k_spmv<1><<<grid, 256, 0, s>>>(H.row_ptr.p, H.col.p, nullptr, H.val32.p, nullptr, H.diag.p,
                                   x, y, n);
  } else {
    k_spmv<2><<<grid, 256, 0, s>>>(H.row_ptr.p, H.col.p, nullptr, H.val32.p, H.res32.p,
                                   H.diag.p, x, y, n);
  }
  SHCI_LAUNCH_CHECK();
  c->launches += 1;
}

}  // namespace shci

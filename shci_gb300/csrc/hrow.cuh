// Row assembly shared by the Hamiltonian build kernels (scan and join traversals).
//
// A warp owns one row i.  The traversal hands it candidate columns j (with their spin
// strings) that passed an excitation-degree test; RowSink queues them per warp in two ring
// buffers, one for single and one for double excitations, and evaluates them 32 at a time.
// A traversal finds a connected column for a minority of lanes, and GB300 issues an FP64 warp
// instruction at 1/16 per SM cycle however many lanes are active, so evaluating in place
// would run the matrix-element arithmetic with few useful lanes; separate queues keep the
// long single-excitation sums apart from the short double-excitation ones.
//
// MODE 0 counts the kept elements (|H_ij| >= 1e-12, src/util.h:50), MODE 1 writes FP64
// values, MODE 2 writes FP32 value + FP32 residual.  Count and fill runs of the same traversal
// drain the queues at the same points, so a row's columns land in the same order every time.
#pragma once

#include "common.cuh"

namespace shci {

constexpr uint32_t kRowQ = 64;  // ring size: < 32 waiting + 32 pushed always fit

struct RowQueues {
  uint32_t j[2][kRowQ];
  uint64_t u[2][kRowQ];
  uint64_t d[2][kRowQ];
};

__device__ __forceinline__ unsigned lanemask_lt_u() { return (1u << (threadIdx.x & 31)) - 1u; }

template <int MODE>
struct RowSink {
  RowQueues& q;
  const DevIntegrals& I;
  const uint64_t ui, di;
  const uint64_t base;  // row offset in the CSR arrays (fill modes)
  uint32_t* col;
  double* v64;
  float* v32;
  float* r32;
  const unsigned lane, lt;
  uint32_t cnt = 0;                            // elements kept so far in this row
  float* absacc = nullptr;                     // optional sums of |H| per det
  uint32_t row = 0;
  float rowabs = 0.0f;
  uint32_t qh[2] = {0u, 0u}, qn[2] = {0u, 0u};  // ring heads and lengths (warp-uniform)

  __device__ __forceinline__ RowSink(RowQueues& q_, const DevIntegrals& I_, uint64_t ui_,
                                     uint64_t di_, uint64_t base_, uint32_t* col_, double* v64_,
                                     float* v32_, float* r32_)
      : q(q_), I(I_), ui(ui_), di(di_), base(base_), col(col_), v64(v64_), v32(v32_), r32(r32_),
        lane(threadIdx.x & 31), lt(lanemask_lt_u()) {}

  // Evaluate the m <= 32 oldest entries of queue t; write the kept ones.
  __device__ __forceinline__ void drain(int t, uint32_t m) {
    __syncwarp();
    bool keep = false;
    uint32_t j = 0;
    double H = 0.0;
    if (lane < m) {
      const uint32_t s = (qh[t] + lane) & (kRowQ - 1);
      j = q.j[t][s];
      const uint64_t uj = q.u[t][s], dj = q.d[t][s];
      // counting needs |H| only: skip the permutation sign (a sign flip is exact)
      H = t == 0 ? h_one<MODE != 0>(I, ui, di, uj, dj) : h_two<MODE != 0>(I, ui, di, uj, dj);
      keep = keep_elem(H);
      if (absacc && keep) {
        // |H| rounded up, summed into both dets' totals (the row abs-sum bound of H*v)
        const float a = __double2float_ru(fabs(H));
        atomicAdd(&absacc[j], a);
        rowabs += a;
      }
    }
    __syncwarp();
    qh[t] += m;
    qn[t] -= m;
    const unsigned bal = __ballot_sync(kFull, keep);
    if (MODE && keep) {
      const uint64_t pos = base + cnt + __popc(bal & lt);
      col[pos] = j;
      if (MODE == 1) {
        v64[pos] = H;
      } else {
        const float hi = static_cast<float>(H);
        v32[pos] = hi;
        r32[pos] = static_cast<float>(H - static_cast<double>(hi));
      }
    }
    cnt += __popc(bal);
  }

  // Queue the lanes' candidates (cand) as singles or doubles; drain full queues.
  __device__ __forceinline__ void push(bool cand, bool single, uint32_t j, uint64_t uj,
                                       uint64_t dj) {
    if (I.no_mixed_doubles && !single && uj != ui && dj != di) cand = false;
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const bool mine = cand && (single == (t == 0));
      const unsigned bal = __ballot_sync(kFull, mine);
      if (!bal) continue;
      if (mine) {
        const uint32_t s = (qh[t] + qn[t] + __popc(bal & lt)) & (kRowQ - 1);
        q.j[t][s] = j;
        q.u[t][s] = uj;
        q.d[t][s] = dj;
      }
      qn[t] += __popc(bal);
      if (qn[t] >= 32u) drain(t, 32u);
    }
  }

  // Drain what is left at the end of the row; returns the row's kept count.
  __device__ __forceinline__ uint32_t finish() {
    if (qn[0]) drain(0, qn[0]);
    if (qn[1]) drain(1, qn[1]);
    if (absacc) {
#pragma unroll
      for (int o = 16; o; o >>= 1) rowabs += __shfl_xor_sync(kFull, rowabs, o);
      if (lane == 0) atomicAdd(&absacc[row], rowabs);
    }
    __syncwarp();
    return cnt;
  }

  // Also accumulate sum_j |H_ij| of row i and of each column j into acc.
  __device__ __forceinline__ void track_abs(float* acc, uint32_t i) {
    absacc = acc;
    row = i;
  }
};

// Inclusive warp prefix sum.
__device__ __forceinline__ uint32_t warp_inclusive_u32(uint32_t v) {
  const unsigned lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, v, o);
    if (lane >= (unsigned)o) v += t;
  }
  return v;
}

// Owner lane of flattened item t: the number of lanes whose inclusive prefix is <= t
// (prefixes are non-decreasing).  A fixed 5-step search, so every lane runs the same shuffles.
__device__ __forceinline__ uint32_t owner_lane(uint32_t inc, uint32_t t) {
  uint32_t lo = 0;
#pragma unroll
  for (uint32_t step = 16; step; step >>= 1) {
    const uint32_t v = __shfl_sync(kFull, inc, lo + step - 1);
    if (v <= t) lo += step;
  }
  return lo;
}

}  // namespace shci

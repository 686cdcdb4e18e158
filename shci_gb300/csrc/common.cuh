// Shared device-side definitions for the SHCI GB300 path.
//
// Determinants are two 64-bit spin strings (alpha = "up", beta = "dn"), n_orbs <= 64.  Integrals
// live in HBM as dense FP64 tables (the 8-fold packed FCIDUMP set expanded on the host), plus
// per-(i,j) contiguous slices used by the single-excitation rule.
//
// The Slater-Condon functions below follow src/chem/chem_system.cc:409-609 of the reference
// term by term and in the same summation order, so FP64 matrix elements agree bit for bit
// with a CPU evaluation of the same rules (the only multiplications are by +-1 and 2, which
// are exact, so FMA contraction cannot change a result).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace shci {

constexpr double kEps = 1.0e-12;  // src/util.h:50: |H| below this is not stored
constexpr unsigned kFull = 0xffffffffu;

struct DevIntegrals {
  int n;                 // spatial orbitals
  double e_core;
  const double* h1;      // [n*n]      h(p,q)
  const double* g2;      // [n^4]      (pq|rs) at ((p*n+q)*n+r)*n+s
  const double* dtab;    // [n^3]      (ij|oo) at (i*n+j)*n+o       (direct)
  const double* xtab;    // [n^3]      (io|oj) at (i*n+j)*n+o       (exchange)
  const double* jtab;    // [n^2]      (aa|bb) at a*n+b
  const double* ktab;    // [n^2]      (ab|ba) at a*n+b
  // the Hamiltonian leaves out opposite-spin double excitations (has_double_excitation
  // false without time_sym, hamiltonian.h:487); 0 keeps them
  int no_mixed_doubles;
};

__device__ __forceinline__ int popc64(uint64_t x) { return __popcll(x); }
__device__ __forceinline__ int ctz64(uint64_t x) { return __ffsll((long long)x) - 1; }
__device__ __forceinline__ uint64_t below(int b) { return (1ull << b) - 1ull; }

__device__ __forceinline__ double g2at(const DevIntegrals& I, int p, int q, int r, int s) {
  const int n = I.n;
  return I.g2[((size_t)(p * n + q) * n + r) * n + s];
}

// Diagonal element (chem_system.cc:426-432, 444-457, 495-542 without the cache).
__device__ __forceinline__ double h_diag(const DevIntegrals& I, uint64_t up, uint64_t dn) {
  const int n = I.n;
  double ob = 0.0;
  for (uint64_t m = up; m; m &= m - 1) {
    const int o = ctz64(m);
    ob += I.h1[o * n + o];
  }
  if (up == dn) {
    ob *= 2;
  } else {
    for (uint64_t m = dn; m; m &= m - 1) {
      const int o = ctz64(m);
      ob += I.h1[o * n + o];
    }
  }
  double direct = 0.0, exch = 0.0;
  for (uint64_t m = up; m; m &= m - 1) {
    const int a = ctz64(m);
    for (uint64_t m2 = m & (m - 1); m2; m2 &= m2 - 1) {
      const int b = ctz64(m2);
      direct += I.jtab[a * n + b];
      exch -= I.ktab[a * n + b];
    }
  }
  if (up == dn) {
    direct *= 2;
    exch *= 2;
  } else {
    for (uint64_t m = dn; m; m &= m - 1) {
      const int a = ctz64(m);
      for (uint64_t m2 = m & (m - 1); m2; m2 &= m2 - 1) {
        const int b = ctz64(m2);
        direct += I.jtab[a * n + b];
        exch -= I.ktab[a * n + b];
      }
    }
  }
  for (uint64_t m = up; m; m &= m - 1) {
    const int a = ctz64(m);
    for (uint64_t m2 = dn; m2; m2 &= m2 - 1) {
      const int b = ctz64(m2);
      direct += I.jtab[a * n + b];
    }
  }
  return ob + (direct + exch) + I.e_core;
}

// x * (-1)^odd.  Multiplying by +-1 only sets the sign bit, so the flip is done on the bits:
// the same value as the multiplication, without an FP64 instruction (GB300's FP64 pipe runs a
// warp instruction in 16 SM cycles, so every FP64 op saved in an element matters).
__device__ __forceinline__ double flip_sign(double x, int odd) {
  return __longlong_as_double(__double_as_longlong(x) ^
                              (static_cast<long long>(odd & 1) << 63));
}

// |h| >= 1e-12 (src/util.h:50) decided on the bit pattern (IEEE order of non-negative doubles
// is the integer order of their bits); equal to the FP64 comparison for every non-NaN h.
constexpr unsigned long long kEpsBits = 0x3d719799812dea11ull;  // bits of 1.0e-12
__device__ __forceinline__ bool keep_elem(double h) {
  return (static_cast<unsigned long long>(__double_as_longlong(h)) & 0x7fffffffffffffffull) >=
         kEpsBits;
}

// Single excitation oi -> oj within the spin string `same` (the other string is `oppo`);
// `same` is the spin string of the ket-side det i; the permutation sign is (-1)^odd.
// chem_system.cc:544-577, same terms in the same order; 2 * direct is exact, so
// fma(2, direct, e) rounds exactly like e + 2 * direct.
__device__ __forceinline__ double h_single(const DevIntegrals& I, uint64_t same, uint64_t oppo,
                                           int oi, int oj, int odd) {
  const int n = I.n;
  const double ob = flip_sign(I.h1[oi * n + oj], odd);
  const double* D = I.dtab + (size_t)(oi * n + oj) * n;
  const double* X = I.xtab + (size_t)(oi * n + oj) * n;
  double e = 0.0;
  for (uint64_t m = same & ~(1ull << oi) & ~(1ull << oj); m; m &= m - 1) {
    const int o = ctz64(m);
    e -= X[o];
    const double direct = D[o];
    if (oppo >> o & 1) {
      oppo &= ~(1ull << o);
      e = fma(2.0, direct, e);
    } else {
      e += direct;
    }
  }
  for (uint64_t m = oppo; m; m &= m - 1) e += D[ctz64(m)];
  return ob + flip_sign(e, odd);
}

// Parity helper of src/det/half_det.cc:120-206 for one moved orbital: electrons of `s` below b.
__device__ __forceinline__ int below_count(uint64_t s, int b) { return popc64(s & below(b)); }

// Bits strictly between orbitals a != b.
__device__ __forceinline__ uint64_t between(int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return ((1ull << hi) - 1ull) & ~((2ull << lo) - 1ull);
}

// Parity of moving one electron from orbital a of string s to orbital b (b not in s):
// below_count(s, a) + below_count(s ^ a ^ b, b) has the parity of the electrons strictly
// between a and b (the electrons below min(a, b) are counted twice).
__device__ __forceinline__ int move_parity(uint64_t s, int a, int b) {
  return popc64(s & between(a, b));
}

// H_ij for a single excitation: exactly one of ui^uj, di^dj is non-zero, with two bits set.
// SIGNED = false returns the value up to its sign (enough for the |H| >= 1e-12 test).
template <bool SIGNED = true>
__device__ __forceinline__ double h_one(const DevIntegrals& I, uint64_t ui, uint64_t di,
                                        uint64_t uj, uint64_t dj) {
  const uint64_t xu = ui ^ uj;
  const bool alpha = xu != 0;
  const uint64_t si = alpha ? ui : di, sj = alpha ? uj : dj, oi_str = alpha ? di : ui;
  const uint64_t x = si ^ sj;
  const int oi = ctz64(si & x), oj = ctz64(sj & x);
  return h_single(I, si, oi_str, oi, oj, SIGNED ? move_parity(si, oi, oj) : 0);
}

// H_ij for a double excitation (one alpha + one beta electron, or two of the same spin).
template <bool SIGNED = true>
__device__ __forceinline__ double h_two(const DevIntegrals& I, uint64_t ui, uint64_t di,
                                        uint64_t uj, uint64_t dj) {
  const uint64_t xu = ui ^ uj, xd = di ^ dj;
  if (xu && xd) {
    const int ai = ctz64(ui & xu), aj = ctz64(uj & xu);
    const int bi = ctz64(di & xd), bj = ctz64(dj & xd);
    const double g = g2at(I, ai, aj, bi, bj);
    if (!SIGNED) return g;
    return flip_sign(g, move_parity(ui, ai, aj) + move_parity(di, bi, bj));
  }
  // same-spin double
  const bool alpha = xu != 0;
  const uint64_t si = alpha ? ui : di, sj = alpha ? uj : dj, x = alpha ? xu : xd;
  const uint64_t li = si & x, rj = sj & x;
  const int l0 = ctz64(li), l1 = ctz64(li & (li - 1));
  const int r0 = ctz64(rj), r1 = ctz64(rj & (rj - 1));
  const double e = g2at(I, l0, r0, l1, r1) - g2at(I, l0, r1, l1, r0);
  if (!SIGNED) return e;
  const int par = below_count(si, l0) + below_count(si, l1) + below_count(sj, r0) +
                  below_count(sj, r1);
  return flip_sign(e, par);
}

// H_ij for dets whose excitation degree is known to be 1 or 2 (or 0: diagonal).  up/dn
// differences are given; returns 0 for degree > 2.  Equivalent to get_hamiltonian_elem(i,j,-1).
__device__ __forceinline__ double h_offdiag(const DevIntegrals& I, uint64_t ui, uint64_t di,
                                            uint64_t uj, uint64_t dj) {
  const int deg = (popc64(ui ^ uj) + popc64(di ^ dj)) >> 1;
  if (deg > 2 || deg == 0) return 0.0;
  return deg == 1 ? h_one(I, ui, di, uj, dj) : h_two(I, ui, di, uj, dj);
}

// ---------------------------------------------------------------- hashing (C21, a16)
// src/det/half_det.cc:71-89 (two chunks, the second always zero) and src/det/det.h:42-49.
__host__ __device__ __forceinline__ uint64_t half_hash(uint64_t c0) {
  uint64_t h = 0;
  h += c0;
  h += (h << 10);
  h ^= (h >> 6);
  h += (h << 10);
  h ^= (h >> 6);
  h += (h << 3);
  h ^= (h >> 11);
  h += (h << 15);
  return h;
}
__host__ __device__ __forceinline__ uint64_t det_hash(uint64_t up, uint64_t dn) {
  uint64_t seed = half_hash(up);
  seed ^= half_hash(dn) + 0x9e3779b9ull + (seed << 6) + (seed >> 2);
  return seed;
}
// src/util.cc:111-122
__host__ __device__ __forceinline__ uint64_t rehash(uint64_t a) {
  uint64_t h = a;
  h += (h << 10);
  h ^= (h >> 6);
  h += 982451653ull;
  h += (h << 10);
  h ^= (h >> 6);
  h += (h << 3);
  h ^= (h >> 11);
  h += (h << 15);
  return h;
}

// ---------------------------------------------------------------- compensated sums
// Double-double accumulator: hi + lo carries the running sum with about 2^-106 relative
// rounding per step (Knuth's branch-free two-sum, then a renormalising fast two-sum), so a
// sum of m terms is accurate to about cond * m * 2^-106 instead of m * 2^-53.  No
// multiplications, so FMA contraction cannot change a result.
struct Dd {
  double hi = 0.0, lo = 0.0;
};
__host__ __device__ __forceinline__ void two_sum64(double a, double b, double* s, double* e) {
  const double t = a + b;
  const double z = t - a;
  *e = (a - (t - z)) + (b - z);
  *s = t;
}
__host__ __device__ __forceinline__ Dd dd_add(Dd a, Dd b) {
  double s, e;
  two_sum64(a.hi, b.hi, &s, &e);
  e += a.lo + b.lo;
  Dd r;
  r.hi = s + e;
  r.lo = e - (r.hi - s);
  return r;
}
__host__ __device__ __forceinline__ Dd dd_add(Dd a, double b) {
  Dd t;
  t.hi = b;
  return dd_add(a, t);
}
__device__ __forceinline__ Dd dd_shfl_xor(Dd a, int o) {
  Dd r;
  r.hi = __shfl_xor_sync(kFull, a.hi, o);
  r.lo = __shfl_xor_sync(kFull, a.lo, o);
  return r;
}

// Error word written by kernels (never __trap): host checks it after each launch group.
enum DevError : unsigned { kDevOk = 0, kDevOverflow = 1, kDevCheck = 2 };

}  // namespace shci

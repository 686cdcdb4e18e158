// The library context: every device buffer of one SHCI instance, on one stream.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "../../include/shci_gpu.h"
#include "common.cuh"
#include "devbuf.h"
#include "host_system.h"
#include "prof.h"
#include "solver.h"
#include "sort.cuh"

namespace shci {

// Determinant index used by the Hamiltonian build (rebuilt from the det list each update).
struct DetIndex {
  size_t n = 0;
  size_t n_alpha = 0, n_beta = 0;
  DevBuf<uint32_t> det_aid, det_bid;      // [n] unique alpha / beta id of each det
  DevBuf<uint32_t> a_start, b_start;      // [n_alpha+1], [n_beta+1] group offsets
  DevBuf<uint32_t> am_idx;                // [n] det ids, alpha groups, by beta string
  DevBuf<uint64_t> am_dn;                 // [n] beta strings in that order
  DevBuf<uint32_t> ad_idx, bd_idx;        // [n] det ids, alpha / beta groups, by det id
  DevBuf<uint64_t> ad_dn, bd_up;          // [n] the other spin string in that order
  DevBuf<uint64_t> ua, ub;                // sorted unique alpha / beta strings
  DevBuf<uint32_t> as_off;                // [n_alpha+1] alpha-singles CSR
  DevBuf<uint32_t> as_list;               // alpha ids one single excitation away
  DevBuf<uint32_t> bs_off;                // [n_beta+1] beta-singles CSR
  DevBuf<uint32_t> bs_list;               // beta ids one single excitation away
  DevBuf<uint64_t> bs_str;                // their beta strings
};

// Two-hole core join of the det list (hjoin.cu): every det contributes one entry per pair of
// its electrons; entries are sorted by a hash of the det minus that pair.
struct JoinIndex {
  uint32_t K = 0;               // entries per det = C(n_up + n_dn, 2)
  int n_up = 0, n_dn = 0;
  size_t m = 0;                 // n * K entries
  DevBuf<uint32_t> pairs;       // [K] electron ranks r1 | r2 << 16 (r1 < r2)
  int bits = 0, key_bytes = 0;  // hash bits kept; key width used by the last index
  DevBuf<uint64_t> keys;        // [m] core hashes (sort keys; released after bucketing)
  DevBuf<uint32_t> keys32;      //     the same when at most 32 hash bits are kept
  DevBuf<uint32_t> scan;        // [m] bucket index of each sorted position (while bucketing)
  DevBuf<uint32_t> bstart;      // [buckets + 1] bucket start positions (while bucketing)
  DevBuf<uint32_t> jdet;        // [m] det id of each sorted entry
  DevBuf<uint64_t> span;        // [m] per entry (in det order): sorted position | bucket end << 32
};

// Segments an incremental update may leave before the next update rebuilds the whole matrix.
constexpr size_t kMaxSegments = 12;

// A store segment kept from an earlier build: rows [0, n) of the strict upper part, row i at
// [row_ptr[i], row_ptr[i] + row_cnt[i]).
struct HSeg {
  size_t n = 0, nnz = 0;
  bool packed = true;
  DevBuf<uint64_t> row_ptr;
  DevBuf<uint32_t> row_cnt, col;
  DevBuf<double> val64;
  DevBuf<float> val32, res32;
};

// Read-only view of one segment (older segments first, then the current build's).
struct SegView {
  size_t n, nnz;
  size_t len;  // entries allocated in col / values (row_ptr indexes into them)
  bool packed;
  const uint64_t* row_ptr;
  const uint32_t* row_cnt;
  const uint32_t* col;
  const double* val64;
  const float* val32;
  const float* res32;
};

// Upper-triangle Hamiltonian (strict upper part in CSR; FP64 diagonal kept apart).  An
// incremental update (Hamiltonian<S>::update with n_dets_prev > 0, hamiltonian.h:421-428)
// moves the current store into `older` and builds a new segment with the new rows and the
// new columns of the old rows; every consumer walks all segments.
struct DevHamiltonian {
  size_t n = 0;
  size_t nnz = 0;
  bool join = false;      // built by the core join (else by the group scan)
  size_t candidates = 0;  // (row, candidate) pairs examined by the last build
  size_t cand_parts[3] = {0, 0, 0};  // scan: same beta, same alpha, alpha single x beta single;
                                     // join: core entries, 0, 0
  int precision = SHCI_PREC_FP64;
  bool packed = true;     // rows contiguous (row_ptr[i+1] = row_ptr[i] + row_cnt[i])
  uint64_t build_id = 0;  // changes whenever the stored matrix does
  DevBuf<uint64_t> row_ptr;   // [n+1] row i = [row_ptr[i], row_ptr[i] + row_cnt[i])
  DevBuf<uint32_t> col;       // [nnz]
  DevBuf<double> val64;       // [nnz]   FP64 storage
  DevBuf<float> val32;        // [nnz]   mixed storage: FP32 value
  DevBuf<float> res32;        // [nnz]   mixed storage: FP32 residual (value - (double)val32)
  DevBuf<double> diag;        // [n]
  DevBuf<uint32_t> row_cnt;   // [n+1] elements of each row
  bool valid = false;
  // the stored matrix is that of the first n dets of the current list (dets were only
  // appended since the build): an update can be incremental
  bool prefix_ok = false;
  std::vector<std::unique_ptr<HSeg>> older;  // segments of earlier (incremental) builds
  size_t nnz_current = 0;                    // elements of the current segment
  size_t n_prev = 0;                         // rows built before the last update (0: full)
  // mixed-storage H*v (spmv.cu): row abs-sum bound and fixed-point scratch
  bool bound_valid = false;
  DevBuf<double> scal;        // [0] max row abs sum, [1] max |x| (bits), [2] spare
  DevBuf<float> xs;           // [2n] x split into float pairs
  DevBuf<unsigned long long> yfix;  // [n] y in 64-bit fixed point
  DevBuf<float> rowabs;       // [n] scratch for the bound
  bool rowabs_hb = false;     // rowabs holds the heat-bath bounds of the dets (not store sums)
};

// All segments of H: older ones, then the current build's.
inline std::vector<SegView> segments(const DevHamiltonian& H) {
  std::vector<SegView> v;
  for (const auto& s : H.older)
    v.push_back(SegView{s->n, s->nnz, s->col.n, s->packed, s->row_ptr.p, s->row_cnt.p,
                        s->col.p, s->val64.p, s->val32.p, s->res32.p});
  v.push_back(SegView{H.n, H.nnz_current, H.col.n, H.packed, H.row_ptr.p, H.row_cnt.p, H.col.p,
                      H.val64.p, H.val32.p, H.res32.p});
  return v;
}

struct DevQueues {
  size_t n_pairs = 0;
  DevBuf<uint64_t> d_off;
  DevBuf<double> d_H;
  DevBuf<uint32_t> d_rs;
  DevBuf<uint32_t> s_off;
  DevBuf<double> s_S;
  DevBuf<uint32_t> s_r;
  // sums of the queue values: per orbital over its singles queue, per pair over its doubles
  // queue (bounds of sum_j |H_ij| over all excitations of a det)
  DevBuf<double> s_tot, d_tot;
  double max_hci = 0.0, max_singles = 0.0;
  size_t n_hci = 0, n_singles = 0;
  bool built = false;
};

// Largest n_states of a several-state run (the subspace holds 5 vectors per state).
constexpr unsigned kMaxStates = 8;

struct Davidson {
  DevBuf<double> v[5], Hv[5], w, Hw;
  // several states (davidson_states): 5 * n_states stored vectors, a Ritz vector per state
  DevBuf<double> sv[5 * kMaxStates], sHv[5 * kMaxStates], sw[kMaxStates], sHw[kMaxStates];
  DevBuf<double> scal;     // device scalars
  DevBuf<double> partial;  // dot partial sums
  DevBuf<double> rt;       // residual-store row sums of the FP64 energy correction
  // w and Hw hold the last Ritz vector and its image under the Hamiltonian of build ritz_h
  bool ritz = false;
  uint64_t ritz_h = 0;
};

}  // namespace shci

struct shci_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  shci::MemTracker mem;

  bool have_integrals = false;
  shci::HostIntegrals I;
  shci::DevBuf<double> h1, g2, dtab, xtab, jtab, ktab;
  // PT2 diagonals in 64-bit fixed point (pt2.cu): h_oo, J - K (same spin), J (opposite spin)
  shci::DevBuf<long long> dfix;
  int dfix_scale = 0;
  bool dfix_valid = false;
  // PT2 single-excitation elements in 64-bit fixed point (pt2.cu): h_pq, (pq|oo), (po|oq)
  shci::DevBuf<long long> sfix;
  int sfix_scale = 0;
  double sfix_margin = 0.0;
  shci::DevIntegrals dI{};
  double energy_hf = 0.0;

  shci::DevQueues Q;

  // determinants (host mirror + device) in the canonical order
  std::vector<uint64_t> up, dn;
  std::vector<double> coefs;
  shci::DevBuf<uint64_t> d_up, d_dn;
  shci::DevBuf<double> d_coef;
  bool dets_dirty = true;  // device copy out of date
  // n_states > 1 (config "n_states"): d_coef is state 0, d_xcoef[s - 1] state s; energies of
  // every state from the last variational run (FP64-corrected in mixed mode)
  unsigned n_states = 1;
  shci::DevBuf<double> d_xcoef[shci::kMaxStates - 1];
  std::vector<double> state_energy;

  // sorted membership keys of the current det list (for selection / PT2)
  shci::DevBuf<uint64_t> set_up, set_dn;
  shci::DevBuf<unsigned long long> set_hash;  // hash set of the det list (in_set)
  uint64_t set_hash_mask = 0;

  std::vector<double> eps_tried;
  // second rejection of the selection (solver.h:426-428: config "second_rejection",
  // "second_rejection_factor"; off and 0.2 by default)
  bool second_rejection = false;
  double second_rejection_factor = 0.2;
  // time-reversal symmetry (config "time_sym"): the det list holds up <= dn, an open det
  // stands for (|up,dn> + |dn,up>) / sqrt(2); the Hamiltonian is the packed one
  bool time_sym = false;
  // find_connected_dets options (chem_system.cc:29-30, 327-329, 345, 383-387): doubles off
  // ("has_double_excitation": false; the Hamiltonian then also drops opposite-spin doubles
  // unless time_sym, hamiltonian.h:97-104, 487) and the active space ("chem/active_space":
  // targets above the highest active orbital of their irrep are skipped)
  bool has_doubles = true;
  uint64_t inactive_orbs = 0;  // orbitals that may not be excitation targets
  // selection from the HF det with eps_min = 0 ("var_sd", solver.h:424, 446)
  bool var_sd = false;
  // HF det construction options (integrals.cc:155-226), used by the FCIDUMP loads that follow
  shci::HfOptions hf_opts;

  shci::DetIndex idx;
  shci::JoinIndex join;
  shci::DevHamiltonian H;
  shci::Davidson dav;
  shci::SortScratch sort;

  // generic scratch
  shci::DevBuf<uint64_t> k0, k1, k2;
  shci::DevBuf<uint32_t> u0, u1, u2;
  shci::DevBuf<double> f0, f1;
  shci::DevBuf<unsigned> err_word;

  // per-iteration record of the last variational run
  std::vector<shci::VarIter> var_trace;

  // counters for the bench: kernels launched by this context
  size_t launches = 0;
  shci::Profiler prof;
};

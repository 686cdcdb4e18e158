// Host-callable entry points of the device kernels (one translation unit per stage).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "devbuf.h"

struct shci_ctx;

namespace shci {

// misc.cu
void widen_u32_u64(const uint32_t* in, uint64_t* out, size_t n, cudaStream_t s);
// Packed CSR copy of the element store (FP64 values) on the device.
void pack_hamiltonian(shci_ctx* c, DevBuf<uint64_t>& ptr, DevBuf<uint32_t>& col,
                      DevBuf<double>& val);
// Rows rows[0..m) of the current Hamiltonian: offsets[m+1] always; cols / vals (FP64; value +
// residual for mixed storage) when non-null, each row in increasing column order.
void get_rows(shci_ctx* c, const uint64_t* rows, size_t m, uint64_t* offsets, uint32_t* cols,
              double* vals);
void upload_integrals(shci_ctx* c);
void upload_queues(shci_ctx* c);
void sync_dets(shci_ctx* c);          // host det list -> device (if dirty)
void hamiltonian_elems(shci_ctx* c, const uint64_t* ui, const uint64_t* di, const uint64_t* uj,
                       const uint64_t* dj, size_t n, double* out);

// noalloc.cu: hamiltonian_elems with staging in a fixed device array (no allocation)
void hamiltonian_elems_noalloc(shci_ctx* c, const uint64_t* ui, const uint64_t* di,
                               const uint64_t* uj, const uint64_t* dj, size_t n, double* out);

// hbuild.cu: group index + scan traversal, and the build driver (join when possible, else
// scan; the SHCI_HBUILD environment variable set to "scan" forces the scan)
void build_index(shci_ctx* c);
size_t build_hamiltonian(shci_ctx* c, int precision);
// timesym.cu: the packed time-reversal-symmetric Hamiltonian (c->time_sym)
size_t build_time_sym(shci_ctx* c, int precision);

// hjoin.cu: two-hole core join.  join_prepare returns false (nothing held) when the join
// cannot be used for the current dets; join_rows runs one pass (mode as the row kernels;
// every mode writes each row's kept count to row_cnt when given).
bool join_prepare(shci_ctx* c);
// n_prev > 0 (incremental update): rows < n_prev take only columns >= n_prev.
void join_rows(shci_ctx* c, int mode, uint32_t* row_cnt, const uint64_t* row_ptr,
               uint32_t* col, double* v64, float* v32, float* r32, unsigned* work,
               unsigned grid, float* absacc, uint32_t n_prev);
void join_release(shci_ctx* c);
// Row starts of a single-pass build: row_start[i] = sum of the candidate counts of rows < i
// (row_start has n + 1 entries); returns the total capacity.
uint64_t join_row_caps(shci_ctx* c, uint64_t* row_start, uint32_t n_prev);

// rowsort.cu: sorts each row of the element store by column (tiles of 2048 elements), so
// that H*v's scattered accesses share sectors; SHCI_ROW_SORT=0 turns the pass off.
bool row_sort_enabled();
void sort_rows(shci_ctx* c);

// spmv.cu: y = H x (FP64 vectors on the device); residual adds the FP32 residual store.
void spmv(shci_ctx* c, const double* x, double* y, bool residual);
// t_i = sum_j R_ij w_j over the stored (upper) elements of the residual store R (mixed H).
void residual_rows(shci_ctx* c, const double* w, double* t);
// Mixed H*v needs a bound on the row abs sums: a mixed build sums |H_ij| into H.rowabs
// (off-diagonal) during its count or single fill pass, and this turns the sums into the bound.
void finish_mixed_bound(shci_ctx* c);

// davidson.cu
struct DavidsonOut {
  double eval = 0.0;
  bool converged = false;
  std::vector<double> trace;
  int n_matvec = 0;
};
// Runs on c->H with the initial vector c->d_coef (length H.n); Ritz vector left in d_coef.
DavidsonOut davidson(shci_ctx* c, double tol);
// Several states (c->n_states > 1): initial vectors d_coef and d_xcoef[0 .. n_states - 2],
// Ritz vectors left there; eigenvalues per state in evals.
struct DavidsonStatesOut {
  std::vector<double> evals;
  bool converged = false;
  int n_matvec = 0;
};
DavidsonStatesOut davidson_states(shci_ctx* c, double tol);
double rayleigh_fp64(shci_ctx* c);
// FP64 Rayleigh quotient x^T H x / x^T x with value + residual (any device vector x).
double rayleigh_fp64_of(shci_ctx* c, const double* x);
// Pointer to the device coefficients of state s (0 = d_coef).
double* state_coef(shci_ctx* c, unsigned s);
void jacobi_eig(int k, const double* lower, int ld, double* evals, double* evecs);

// select.cu
size_t select_dets(shci_ctx* c, double eps_var, bool var_sd);
void rebuild_det_set(shci_ctx* c);
size_t sort_unique_pairs(shci_ctx* c, DevBuf<uint64_t>& a, DevBuf<uint64_t>& b, size_t m,
                         DevBuf<double>* vals = nullptr, int n_vals = 1, int a_bits = 0);
void compact_valid(shci_ctx* c, const uint64_t* a, const uint64_t* b, const double* const* v,
                   int n_vals, size_t m, DevBuf<uint64_t>& oa, DevBuf<uint64_t>& ob,
                   DevBuf<double>* ov, size_t* n_out);

// pt2.cu
struct Pt2Out {
  double value = 0.0, uncert = 0.0;
  size_t n_pt_dets = 0;
  size_t n_batches_done = 0;  // batches (dtm / psto) or iterations (sto) computed
};
Pt2Out pt2_dtm(shci_ctx* c, double energy_var, double eps_pt_dtm, size_t n_batches);
Pt2Out pt2_psto(shci_ctx* c, double energy_var, double eps_pt_dtm, double eps_pt_psto,
                size_t n_batches, double target_error, double eps_pt);
// pt2.cu: the pseudo-stochastic stage's automatic batch count (solver.h:772-814)
size_t psto_auto_batches(shci_ctx* c, double eps_pt_psto, double pt_mem_avail, double mem_usage,
                         size_t* n_pilot);
Pt2Out pt2_sto(shci_ctx* c, double energy_var, double eps_pt_psto, double eps_pt,
               size_t n_batches, size_t n_dets_in_sample, bool semisto, unsigned random_seed,
               size_t max_iterations, double target_error, double psto_uncert,
               double pt_mem_avail, double mem_usage, std::vector<double>* loops,
               size_t* info);

// pt2.cu: out[2g], out[2g+1] = sum and sum of squares of x over segment g = [starts[g],
// starts[g+1]) (device arrays; m = total length), compensated and in a fixed order.
void seg_reduce2(shci_ctx* c, const double* x, const uint64_t* starts, uint32_t nseg, size_t m,
                 double* out);

// connected.cu: BaseSystem::find_connected_dets for host det lists (see the C ABI); without
// out_up, fills offsets[0..n] from the counts; with it, writes the lists at those offsets.
void find_connected(shci_ctx* c, const uint64_t* up, const uint64_t* dn, const double* eps_max,
                    const double* eps_min, size_t n, uint64_t* offsets, uint64_t* out_up,
                    uint64_t* out_dn, uint8_t* n_excite);

// rdm.cu
void rdm1(shci_ctx* c, double* out);       // host [n*n]
void rdm2(shci_ctx* c, double* out_half);  // host [n^2 (n^2+1) / 2]
void rdm1_dev(shci_ctx* c, double* res_dev);    // device [n*n] (state 0 coefficients)
void rdm2_dev(shci_ctx* c, double* half_dev);   // device [n^2 (n^2+1) / 2]

// orbopt.cu: generalized Fock matrix F[n*n] (host) from the RDMs of every state
void generalized_fock(shci_ctx* c, double* F);
// orbopt.cu: natural orbitals of a 1-RDM g1 (n x n) per irrep, and the rotation of the
// context's integrals by an orthogonal rot (n x n, rot[i * n + p] = U_ip)
void natural_orbitals(shci_ctx* c, const double* g1, double* rot, double* occ);
void rotate_integrals(shci_ctx* c, const double* rot);
// orbopt.cu: the diagonal of the orbital Hessian for the pairs (p, q), and rot = exp(X(kappa))
void orbital_hessian_diagonal(shci_ctx* c, const unsigned* p, const unsigned* q, size_t n_param,
                              double* hdiag);
void rotation_from_parameters(int n, const unsigned* p, const unsigned* q, const double* kappa,
                              size_t n_param, double* rot);

// spin.cu: <S^2> of the first state over the current det list (ChemSystem::get_s2).
double get_s2(shci_ctx* c);

}  // namespace shci

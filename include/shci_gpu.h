/*
 * shci_gpu.h - C ABI of the GB300 SHCI hot path (libshci_gpu.so).
 *
 * Replaces, for one process on one GPU, the reference's in-process C++ interfaces on the
 * SHCI hot path (QMC-Cornell/shci):
 *   - the system plugin API, class BaseSystem (src/base_system.h:43-136), as implemented by
 *     ChemSystem (src/chem/chem_system.{h,cc});
 *   - the solver-level operators Hamiltonian<S>::update (src/solver/hamiltonian.h:87-112),
 *     SparseMatrix::mul (src/solver/sparse_matrix.cc:28-56), Davidson::diagonalize
 *     (src/solver/davidson.cc:8-196) and the selection / PT2 / RDM stages of
 *     Solver<S> (src/solver/solver.h) and RDM (src/chem/rdm.cc).
 *
 * Conventions.  Plain pointers and sizes only.  Pointers are HOST pointers unless the name
 * ends in _dev (device pointers on the context's device).  The caller owns host buffers;
 * the context owns all device memory it allocates.  Every call returns a status and never
 * throws across the ABI; shci_last_error() gives the message of the last failure.  Calls on
 * one context are not thread safe; separate contexts are independent.  Determinants are two
 * 64-bit spin strings (bit k = spatial orbital k occupied), so n_orbs <= 64.
 */
#ifndef SHCI_GPU_H
#define SHCI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct shci_ctx shci_ctx;

typedef enum {
  SHCI_OK = 0,
  SHCI_ERR_OOM = 1,      /* device allocation failed or budget exceeded */
  SHCI_ERR_ARG = 2,      /* invalid argument / state (message says which) */
  SHCI_ERR_CUDA = 3,     /* CUDA runtime error */
  SHCI_ERR_TIMEOUT = 4,  /* a bounded device-side wait gave up */
  SHCI_ERR_OVERFLOW = 5, /* a device buffer bound was exceeded (host splits and retries) */
  SHCI_ERR_CHECK = 6,    /* a device-side consistency check failed */
  SHCI_ERR_IO = 7        /* file could not be read / parsed */
} shci_status;

/* Matrix-element storage precision for shci_update_hamiltonian. */
typedef enum {
  SHCI_PREC_FP64 = 0,  /* off-diagonal elements stored as FP64 */
  SHCI_PREC_MIXED = 1  /* off-diagonal elements stored as FP32 (+ FP32 residual for the
                          final FP64 correction); accumulation always FP64 */
} shci_precision;

/* ---- lifecycle --------------------------------------------------------------------- */

/* Create a context on `device`.  hbm_budget_bytes = 0: no explicit budget. */
shci_status shci_create(shci_ctx** out, int device, size_t hbm_budget_bytes);
shci_status shci_destroy(shci_ctx* ctx);
const char* shci_last_error(const shci_ctx* ctx);
/* The CUDA stream all work of this context is issued on (a cudaStream_t). */
void* shci_stream(shci_ctx* ctx);

/* ---- integrals (ChemSystem::setup / Integrals::load) --------------------------------- */

/* Read FCIDUMP at `path` and prepare integrals exactly as Integrals::load does
 * (src/chem/integrals.cc:17-35, 37-114, 155-384): |v| < 1e-9 dropped, duplicates keep the
 * larger |v|, HF det filled lowest (or from occs_up/occs_dn when both non-NULL), orbitals
 * reordered by HF orbital energy when reorder = -1 (default: unless occs given) or 1.
 * point_group: "C1", "C2", "Cs", "Ci", "C2v", "C2h", "D2", "D2h", or a linear group "Dooh" /
 * "Dih" / "Coov" / "Civ" (case-insensitive; chem_system.cc:198-221).  ORBSYM labels with
 * negative entries are converted to the reference's linear-group labels (integrals.cc:
 * 116-153).  For a linear group every (pq|rs) with lz_p + lz_r != lz_q + lz_s is zero, as
 * Integrals::get_2b returns it (integrals.cc:394-406), and the heat-bath queues pair r with
 * the conjugate irrep (chem_system.cc:133-135). */
shci_status shci_load_fcidump(shci_ctx* ctx, const char* path, unsigned n_up, unsigned n_dn,
                              const char* point_group, int reorder, const unsigned* occs_up,
                              const unsigned* occs_dn);

/* Integrals cache (Integrals::save_to_cache / load_from_cache, src/chem/integrals.cc:17-35,
 * 424-440): the prepared integrals (reordered h1, g2, orbital symmetries, orbital order, HF
 * det, E_core) in this build's own little-endian layout (magic "SHCIGIC1"; the reference's hps
 * byte format is not available).  Save writes `path` unless a file not in this layout is there
 * (*written = 0: it is not overwritten).  Load reads `path` when it is in this layout
 * (*loaded = 1) and leaves the context unchanged otherwise (*loaded = 0: missing or foreign
 * file); the point group is passed again, as the reference takes it from the config.  A file
 * in this layout that is truncated or inconsistent gives SHCI_ERR_IO, one written for other
 * n_up / n_dn gives SHCI_ERR_ARG. */
shci_status shci_save_integrals_cache(shci_ctx* ctx, const char* path, int* written);
shci_status shci_load_integrals_cache(shci_ctx* ctx, const char* path, unsigned n_up,
                                      unsigned n_dn, const char* point_group, int* loaded);

/* Set already-prepared integrals: h1[n*n] (h_pq), g2[n^4] (chemists' (pq|rs) at
 * ((p*n+q)*n+r)*n+s), orb_sym[n] (irreps 1..8, or linear-group labels; NULL = all 1).  The
 * HF det is given.  Linear groups screen g2 by Lz as shci_load_fcidump does. */
shci_status shci_set_integrals(shci_ctx* ctx, int n_orbs, unsigned n_up, unsigned n_dn,
                               double e_core, const double* h1, const double* g2,
                               const unsigned* orb_sym, const char* point_group,
                               uint64_t hf_up, uint64_t hf_dn);

/* Reordered dense integrals as used on the device (any pointer may be NULL). */
shci_status shci_get_integrals(shci_ctx* ctx, int* n_orbs, double* e_core, double* h1,
                               double* g2, unsigned* orb_sym, unsigned* orb_order);

/* HF det and its energy (ChemSystem::setup, chem_system.cc:50-60). */
shci_status shci_get_hf(shci_ctx* ctx, uint64_t* up, uint64_t* dn, double* energy_hf);

/* Heat-bath queues (ChemSystem::setup_hci_queue / setup_singles_queue,
 * chem_system.cc:74-196); built on the host, uploaded to HBM.  info[4] =
 * {max hci elem, n hci entries, max singles elem, n singles entries}. */
shci_status shci_build_queues(shci_ctx* ctx, double* info);

/* ---- determinants and coefficients (BaseSystem::dets / coefs) ------------------------ */

shci_status shci_set_dets(shci_ctx* ctx, const uint64_t* up, const uint64_t* dn,
                          const double* coefs, size_t n);
shci_status shci_get_n_dets(shci_ctx* ctx, size_t* n);
shci_status shci_get_dets(shci_ctx* ctx, uint64_t* up, uint64_t* dn, double* coefs, size_t cap);
shci_status shci_set_coefs(shci_ctx* ctx, const double* coefs, size_t n);
/* Same from a device buffer (no host round trip). */
shci_status shci_set_coefs_dev(shci_ctx* ctx, const double* coefs_dev, size_t n);

/* ---- matrix elements (BaseSystem::get_hamiltonian_elem, base_system.h:94-95) --------- */

/* out[k] = H(det_i[k], det_j[k]) for k < n (n_excite = -1 semantics: degree computed,
 * 0 for degree > 2; equal dets give the diagonal). */
shci_status shci_hamiltonian_elems(shci_ctx* ctx, const uint64_t* up_i, const uint64_t* dn_i,
                                   const uint64_t* up_j, const uint64_t* dn_j, size_t n,
                                   double* out);

/* Same results as shci_hamiltonian_elems for callers that cannot allocate device memory
 * (for example a process whose device memory is held by another framework's caching
 * allocator, or one that forbids device allocation after start-up).  It has no counterpart
 * in the reference: it exists only for such callers.  It allocates nothing: inputs and
 * results are staged in one fixed 2.5 MiB device array built into the library (resident on
 * every GPU that loads it until the process exits).  At most 65,536 pairs per call (larger
 * n: SHCI_ERR_ARG).  All calls share the array, so calls that overlap on the GPU race; each
 * call looks up the array's address in the current context, and the first call on a device
 * (which can load the library's device code) should come before any stream capture. */
shci_status shci_hamiltonian_elems_noalloc(shci_ctx* ctx, const uint64_t* up_i,
                                           const uint64_t* dn_i, const uint64_t* up_j,
                                           const uint64_t* dn_j, size_t n, double* out);

/* ---- connected dets (BaseSystem::find_connected_dets, base_system.h:57-62) ----------- */

/* ChemSystem::find_connected_dets (src/chem/chem_system.cc:289-402) with second rejection off,
 * for n dets at once.  Det k receives the dets its handler would be called with for the
 * window [eps_min[k], eps_max[k]), in the handler's order: single excitations whose
 * heat-bath bound S >= eps_min[k] (the upper end does not apply to singles, as in the
 * reference), then double excitations with eps_min[k] <= |H| < eps_max[k], both with
 * unoccupied targets; n_excite[] is 1 or 2.  A det with eps_max < eps_min has none (the
 * reference's early return).  Two calls: with out_up == NULL, offsets[0..n] receive the
 * running counts (det k's list is [offsets[k], offsets[k+1])); then, with those offsets,
 * out_up / out_dn / n_excite (offsets[n] entries each) receive the lists.  The reference's
 * return value (the largest rejected |H|) is eps_min[k] without second rejection. */
shci_status shci_find_connected_dets(shci_ctx* ctx, const uint64_t* up, const uint64_t* dn,
                                     const double* eps_max, const double* eps_min, size_t n,
                                     uint64_t* offsets, uint64_t* out_up, uint64_t* out_dn,
                                     uint8_t* n_excite);

/* ---- Hamiltonian build (Hamiltonian<S>::update, hamiltonian.h:87-112, 415-598) -------- */

/* Build the upper-triangle sparse Hamiltonian of the current dets on the device.
 * nnz_out[0] = stored strict-upper elements, nnz_out[1] = the reference's symmetric count
 * (2 * (strict + n) - n, sparse_matrix.cc:13-26).  Elements with |H| < 1e-12 are dropped. */
shci_status shci_update_hamiltonian(shci_ctx* ctx, int precision, size_t* nnz_out);

/* Sizes of the last build: stats[0..9] = {n dets, strict-upper nnz, unique alpha strings,
 * unique beta strings, alpha-single pairs, (row, candidate) pairs examined, three counts,
 * path}.  path (stats[9]) is 1 when the two-hole core join built the matrix: then
 * stats[2..4] are 0 and stats[6] is the number of core entries (dets x electron pairs).
 * path 0 is the group scan: stats[6..8] split the candidates into same-beta, same-alpha and
 * alpha-single x beta-single parts.  For the core join, stats[7] is 1 when the single-pass
 * build (rows sized by their candidate counts) ran and 0 for the two-pass build (counted,
 * then filled); the build takes the single pass when its store fits the free memory and the
 * context's budget, else the two-pass join, else the group scan. */
shci_status shci_hamiltonian_stats(shci_ctx* ctx, uint64_t* stats);

/* Device bytes held by the context now, the most it has held, its budget (0: none), of the
 * bytes held those in its cache of released blocks (returned to the driver before an
 * allocation would fail; at most a quarter of the device), and the most held by live buffers
 * (out[5]).  With a budget, an allocation past it fails with SHCI_ERR_OOM and leaves the
 * context usable. */
shci_status shci_memory_stats(shci_ctx* ctx, size_t* out);

/* Copy the Hamiltonian to the host: row_ptr[n+1] (strict upper), cols[nnz], vals[nnz]
 * (as FP64), diag[n].  Rows list their columns in the device traversal order. */
shci_status shci_get_hamiltonian(shci_ctx* ctx, uint64_t* row_ptr, uint32_t* cols,
                                 double* vals, double* diag);

/* Selected rows of the Hamiltonian (the strict upper part of SparseMatrix rows,
 * sparse_matrix.h): offsets[0..n_rows] receive the running element counts of rows[k]; cols and
 * vals (offsets[n_rows] entries, may be NULL for a size query) the elements of each row in
 * increasing column order, vals as FP64 (value + residual for mixed storage). */
shci_status shci_get_hamiltonian_rows(shci_ctx* ctx, const uint64_t* rows, size_t n_rows,
                                      uint64_t* offsets, uint32_t* cols, double* vals);

/* ---- H*v and Davidson (SparseMatrix::mul, Davidson::diagonalize) --------------------- */

/* y_dev = H x_dev on the context stream (n = number of dets, FP64 vectors).
 * use_residual = 1 adds the FP32 residual of mixed storage (FP64-accurate product). */
shci_status shci_hv(shci_ctx* ctx, const double* x_dev, double* y_dev, int use_residual);

/* Host-buffer variant of shci_hv (copies in and out). */
shci_status shci_hv_host(shci_ctx* ctx, const double* x, double* y, int use_residual);

/* One Davidson::diagonalize call (n_states = 1) on the current Hamiltonian, starting from the
 * context's coefficients; on return they hold the Ritz vector.  eval = lowest eigenvalue,
 * converged as in davidson.cc:174-185.  trace (may be NULL) receives the eigenvalue estimate
 * after each step (up to trace_cap); n_trace its count. */
shci_status shci_davidson(shci_ctx* ctx, double tol, double* eval, int* converged,
                          double* trace, size_t trace_cap, size_t* n_trace);

/* Rayleigh quotient <c|H|c>/<c|c> of the context's coefficients with the FP64-accurate
 * product (mixed storage: FP32 value + FP32 residual) - the final FP64 correction. */
shci_status shci_energy_fp64(shci_ctx* ctx, double* energy);

/* Davidson on a caller-supplied upper-triangle CSR (strict upper + diag), e.g. the Hilbert
 * matrix of src/solver/davidson_test.cc.  init/evec are host vectors of length n. */
shci_status shci_davidson_csr(shci_ctx* ctx, size_t n, const uint64_t* row_ptr,
                              const uint32_t* cols, const double* vals, const double* diag,
                              const double* init, double tol, double* eval, double* evec,
                              int* converged);

/* Several-state Davidson (davidson.cc:8-196 with n_states initial vectors, as a Solver with
 * n_states > 1 calls it) on a caller-supplied CSR: init[n_states * n] in, evecs[n_states * n]
 * and evals[n_states] out.  1 <= n_states <= 8. */
shci_status shci_davidson_csr_states(shci_ctx* ctx, size_t n, const uint64_t* row_ptr,
                                     const uint32_t* cols, const double* vals,
                                     const double* diag, unsigned n_states, const double* init,
                                     double tol, double* evals, double* evecs, int* converged);

/* ---- several states (config "n_states", chem_system.cc:24, 52-56) ------------------------ */

/* Number of states of the variational stage (1 <= n_states <= 8).  States 1.. start at 1e-16
 * on every current det.  With n_states > 1 the selection uses the coefficient of largest
 * magnitude over the states (solver.h:440-444); while the det list is small (<= 50 dets when a
 * step begins) new det k starts as state k's unit vector (solver.h:479-486); Davidson runs
 * with all states (davidson.cc); the RDMs sum over the states (rdm.cc:222-231, 648-657).  The
 * coefficients of state 0 are the context's coefficients (shci_get_dets / shci_set_coefs).
 * PT2 of state s: shci_set_coefs with state s's coefficients, then the PT2 calls with state
 * s's energy (solver.h:620-632). */
shci_status shci_set_n_states(shci_ctx* ctx, unsigned n_states);
shci_status shci_get_state_coefs(shci_ctx* ctx, unsigned state, double* coefs, size_t cap);
shci_status shci_set_state_coefs(shci_ctx* ctx, unsigned state, const double* coefs, size_t n);
/* ---- time-reversal symmetry (config "time_sym", needs n_up == n_dn) -------------------- */

/* With on != 0 the det list holds one det of each time-reversal pair, the one with up <= dn
 * (every current det must be in that form); an open det stands for (|up,dn> + |dn,up>)/sqrt(2).
 * Selection multiplies an open source's eps_min by sqrt(2) and stores candidates in that form
 * (solver.h:447-455); the Hamiltonian is the packed one of Hamiltonian<S>::update_matrix with
 * time_sym (hamiltonian.h:415-598; elements get_hamiltonian_elem_time_sym, base_system.h:
 * 86-101); updates rebuild it whole. */
shci_status shci_set_time_sym(shci_ctx* ctx, int on);
/* unpack_time_sym (base_system.h:108-123), as Solver::run_perturbation does before PT2: every
 * det with up < dn gets its reverse appended, both coefficients (all states) times 1/sqrt(2);
 * the context leaves time_sym mode. */
shci_status shci_unpack_time_sym(shci_ctx* ctx);

/* Energies of the states after the last variational iteration (FP64-corrected in mixed mode). */
shci_status shci_get_state_energies(shci_ctx* ctx, double* energies, size_t cap);
/* Per-iteration energies of every state of the last shci_run_variation:
 * energies[iteration * n_states + state]; *n = number of iterations. */
shci_status shci_get_var_trace_states(shci_ctx* ctx, double* energies, size_t cap, size_t* n);

/* ---- heat-bath selection (Solver<S>::run_variation, solver.h:435-495) ---------------- */

/* One selection step with the context's coefficients: five passes over var dets i = j mod 5,
 * each pass's new dets appended in ascending Det order with coefficient 1e-16.  Keeps the
 * eps_tried_prev memo (solver.h:445-448, 465-468) across calls.  n_new = dets added. */
shci_status shci_select(shci_ctx* ctx, double eps_var, int var_sd, size_t* n_new);

/* Second rejection of the selection (config "second_rejection" / "second_rejection_factor",
 * solver.h:426-428, 461-465; chem_system.cc:300-308, 318-324, 364-370): when enabled, window
 * entries with |H|^2 / (one-body energy difference to HF) < factor * eps_min^2 are dropped and
 * eps_tried_prev becomes 1.000000001 * max(largest dropped |H|, eps_min).  Off by default
 * (factor 0.2).  Applies to shci_select and shci_run_variation of this context. */
shci_status shci_set_second_rejection(shci_ctx* ctx, int enable, double factor);

/* Double excitations on or off (config "has_double_excitation", default on;
 * chem_system.cc:29, 345; hamiltonian.h:97-104, 487).  Off: find_connected_dets yields single
 * excitations only (selection, PT2, shci_find_connected_dets) and returns eps_min (what the
 * singles' second rejection dropped is not kept), and the Hamiltonian leaves out the
 * opposite-spin doubles (same-spin doubles stay; with time_sym every double stays). */
shci_status shci_set_has_double_excitation(shci_ctx* ctx, int on);

/* Active space (config "chem/active_space" with "chem/irrep_active_space",
 * integrals.cc:295-326, chem_system.cc:327-329, 383-387): irrep_active_space[k] orbitals of
 * irrep k + 1, the lowest in the current orbital order, are active; find_connected_dets skips
 * excitations whose target orbital lies above the highest active orbital of its irrep (after
 * the second-rejection test, before the occupancy tests).  n = 0 turns it off; n must cover
 * every irrep of the orbitals (SHCI_ERR_ARG otherwise).  The reference requires
 * "reorder_orbs": false with it (the orbital order is the FCIDUMP's).  Reset by loading
 * integrals. */
shci_status shci_set_active_space(shci_ctx* ctx, const unsigned* irrep_active_space, size_t n);
/* Bit r set: orbital r may not be an excitation target. */
shci_status shci_get_inactive_orbitals(shci_ctx* ctx, uint64_t* mask);

/* Selection of shci_run_variation starts the HF det with eps_min = 0 (config "var_sd",
 * default "get_pair_contrib", solver.h:423-424, 446).  Off by default. */
shci_status shci_set_var_sd(shci_ctx* ctx, int on);

/* HF det options of the following shci_load_fcidump calls (Integrals::generate_det_hf,
 * integrals.cc:155-226): without occs_up / occs_dn, n_irreps > 0 fills irreps[k] (orbital
 * symmetry labels as in ORBSYM, linear groups in the reference's labels) with
 * irrep_occs_up[k] / irrep_occs_dn[k] electrons in orbital order (config "chem/irreps",
 * "chem/irrep_occs_up", "chem/irrep_occs_dn"; such an HF det counts as explicit, so the
 * orbitals are not reordered by default); otherwise the lowest orbitals, with the beta
 * electrons placed above the alpha ones when allow_doubly_occupy = 0 (config
 * "allow_doubly_occupy_hf", default 1).  An impossible filling gives SHCI_ERR_IO from the
 * load. */
shci_status shci_set_hf_options(shci_ctx* ctx, int allow_doubly_occupy, const unsigned* irreps,
                                const unsigned* irrep_occs_up, const unsigned* irrep_occs_dn,
                                size_t n_irreps);

/* eps_tried_prev memo (length = n dets at the last selection). */
shci_status shci_get_eps_tried(shci_ctx* ctx, double* out, size_t cap);

/* Whole variational stage (solver.h:338-397, 413-539): eps_vars[n_eps] with the
 * eps_vars_schedule; energies[n_eps] out.  precision as for shci_update_hamiltonian. */
shci_status shci_run_variation(shci_ctx* ctx, const double* eps_vars, size_t n_eps,
                               const double* schedule, size_t n_sched, double target_error,
                               int precision, double* energies);

/* Per-iteration record of the last shci_run_variation (the reference's "Iteration N ...
 * ndets= ... energy=" log lines and "Number of nonzero elems"): n_dets, symmetric nnz and
 * energy of each iteration; *n = number of iterations (entries beyond cap not written). */
shci_status shci_get_var_trace(shci_ctx* ctx, uint64_t* n_dets, uint64_t* nnz, double* energy,
                               size_t cap, size_t* n);

/* Number of kernel launches issued by this context so far (for launch accounting). */
shci_status shci_get_launch_count(shci_ctx* ctx, uint64_t* n);

/* Per-stage device timing with CUDA events on the context stream (replaces the reference's
 * barriered Timer sections, src/timer.cc:25-63).  enable = 1 starts (and clears) the
 * record, 0 stops it.  shci_profile_get returns, for up to cap stages, the stage name
 * (NUL-terminated, 32 bytes each in names[]), total milliseconds and launch count. */
shci_status shci_profile(shci_ctx* ctx, int enable);
shci_status shci_profile_get(shci_ctx* ctx, char* names, double* total_ms, uint64_t* count,
                             size_t cap, size_t* n);

/* ---- PT2 (Solver<S>::get_energy_pt_dtm, solver.h:636-764) ---------------------------- */

/* Deterministic Epstein-Nesbet PT2 over n_batches hash batches (rehash(DetHasher(a)) %
 * n_batches); n_batches = 0 picks the count from the candidate total and free HBM (the
 * result does not depend on it).  energy_var = E_var of the context's wavefunction.  out:
 * correction, its uncertainty (0 when all batches ran), number of unique PT dets. */
shci_status shci_pt2_dtm(shci_ctx* ctx, double energy_var, double eps_pt_dtm, size_t n_batches,
                         double* correction, double* uncert, size_t* n_pt_dets);

/* The PT2 stages' map-reduce (Solver<S>::mapreduce_sum, solver.h:1155-1177): out[0] = sum of
 * x[k], out[1] = sum of x[k]^2 over k < n (host x), in the fixed-order, compensated
 * (double-double) reduction the PT2 stages use for their per-det contributions. */
shci_status shci_mapreduce_sum(shci_ctx* ctx, const double* x, size_t n, double* out);

/* Pseudo-stochastic stage (Solver<S>::get_energy_pt_psto, solver.h:766-896): batches of the
 * PT space between eps_pt_psto and eps_pt_dtm with the reference's batch extrapolation,
 * uncertainty and early stop (uncert <= target_error / 2, or eps_pt_psto <= eps_pt and
 * uncert <= target_error).  out: correction (excluding the dtm part), uncertainty, PT dets,
 * batches computed. */
shci_status shci_pt2_psto(shci_ctx* ctx, double energy_var, double eps_pt_dtm,
                          double eps_pt_psto, size_t n_batches, double target_error,
                          double eps_pt, double* correction, double* uncert, size_t* n_pt_dets,
                          size_t* n_batches_done);

/* Automatic batch count of the pseudo-stochastic stage ("n_batches_pt_psto" 0 or unset,
 * solver.h:772-814): the unique PT dets of hash batch 0 of 128 from every 100th variational
 * det starting at 50 (single excitations below eps_pt_psto dropped), then
 * n = ceil(2.5 * 128 * 100 * n_pilot * 48 / (pt_mem_avail * mem_usage)), at least 16
 * (mem_usage = config "pt_psto_mem_usage", default 1; pt_mem_avail from shci_pt_mem_avail).
 * Needs n_orbs <= 57. */
shci_status shci_pt2_psto_auto_batches(shci_ctx* ctx, double eps_pt_psto, double pt_mem_avail,
                                       double mem_usage, size_t* n_batches, size_t* n_pilot_dets);

/* Stochastic stage (Solver<S>::get_energy_pt_sto, solver.h:898-1153): |c_i|-weighted
 * samples drawn on the host with the reference's generator
 * (std::default_random_engine(random_seed)) and alias tables, a random hash batch per
 * iteration, the reference's estimator and stopping rules (at most max_iterations).
 * n_dets_in_sample = 0 sizes the sample as the reference does when n_dets_in_sample_pt_sto is
 * unset (solver.h:942-1006): a 1,000-draw pilot counts the PT dets of one hash batch of 128,
 * and the unique-sample target follows from pt_mem_avail (bytes, shci_pt_mem_avail) and
 * mem_usage (pt_sto_mem_usage, the reference's default 0.4).  semisto = 1 (the reference's
 * default semisto_sto) makes the dets above the quantile of the top quarter of that target
 * deterministic and samples the rest with renormalised weights (solver.h:1009-1036); it needs
 * n_dets_in_sample = 0 (with a given sample size the reference's quantile heap is empty: the
 * call returns SHCI_ERR_ARG).  psto_uncert = uncertainty of the preceding psto stage.
 * loops (may be NULL, cap entries) receives each iteration's estimate; sample_info (may be
 * NULL) = {n_dets_in_sample used, deterministic dets, unique-sample target}; out: correction,
 * uncertainty, iterations run. */
shci_status shci_pt2_sto(shci_ctx* ctx, double energy_var, double eps_pt_psto, double eps_pt,
                         size_t n_batches, size_t n_dets_in_sample, int semisto,
                         unsigned random_seed, size_t max_iterations, double target_error,
                         double psto_uncert, double pt_mem_avail, double mem_usage,
                         double* correction, double* uncert, size_t* n_iterations,
                         size_t* sample_info, double* loops, size_t cap);

/* PT memory of the reference's run_all_perturbations (solver.h:601-611, one process):
 * mem_total * 0.7 - n_dets * 104 - 32 * (heat-bath queue entries), in bytes (mem_total is the
 * config's "mem_total", else the machine's memory).  Needs the queues built. */
shci_status shci_pt_mem_avail(shci_ctx* ctx, double mem_total, double* out);

/* ---- batched small instances ------------------------------------------------------------ */

/* One instance of a batch: the reference's whole run (setup, variation with its schedule,
 * PT2) for one FCIDUMP.  eps_pt_dtm <= 0 skips PT2; the psto stage runs (16 batches) when
 * 0 < eps_pt_psto < eps_pt_dtm. */
typedef struct {
  const char* fcidump;
  unsigned n_up, n_dn;
  const char* point_group;
  const double* eps_vars;
  size_t n_eps;
  const double* schedule;
  size_t n_sched;
  double target_error;
  double eps_pt_dtm, eps_pt_psto, eps_pt;
  int precision;
} shci_batch_item;

typedef struct {
  int status;             /* shci_status of this instance */
  double energy_hf, energy_var;
  double correction_pt;   /* PT2 correction (E_total = energy_var + correction_pt) */
  double uncert_pt;
  uint64_t n_dets, n_pt_dets;
  double seconds;         /* wall time of this instance's solve */
} shci_batch_result;

/* Solves n instances on `device` concurrently (n_workers contexts and streams, largest
 * instances first); n_workers <= 0 lets the autotuner choose from measured throughput
 * (*workers_used reports the choice).  No counterpart object in the reference, which runs
 * one instance per process; each instance follows Solver<S>::run (solver.h:100-160). */
shci_status shci_batch_solve(int device, const shci_batch_item* items, size_t n, int n_workers,
                             shci_batch_result* results, int* workers_used);

/* ---- RDMs: the adjoint of E_var (RDM::get_1rdm / get_2rdm, src/chem/rdm.cc) ---------- */

/* Natural orbitals (Optimization::get_natorb_rotation_matrix, optimization.cc:6-79): the
 * context's 1-RDM (summed over the states) diagonalised within each irrep; rot[i * n + p] is
 * the rotation (column p of an irrep's block = the eigenvector of its p-th largest
 * occupation, in that irrep's orbital order), occ[p] the occupation numbers. */
shci_status shci_natural_orbitals(shci_ctx* ctx, double* rot, double* occ);

/* Rotates the context's integrals by the orthogonal rot (rot[i * n + p] = U_ip, mixing only
 * orbitals of the same irrep): (pq|rs) -> sum_ijkl U_ip U_jq U_kr U_ls (ij|kl) on the device,
 * one index at a time, and h -> U^T h U (Optimization::rotate_integrals / rewrite_integrals,
 * optimization.cc:81-240; each class of symmetry-equal integrals keeps its first value of
 * largest magnitude, as the reference's tables do).  The det list returns to the HF det and
 * the heat-bath queues are rebuilt on the next use, as after a new FCIDUMP. */
shci_status shci_rotate_integrals(shci_ctx* ctx, const double* rot);

/* Diagonal of the orbital Hessian for the pairs (p[k], q[k]) (Optimization::hessian_diagonal,
 * optimization.cc:605-618, with hessian_part and Y_matrix, :652-676, Helgaker 10.8.50-53), from
 * the device RDMs summed over the states (the direct 1-RDM; the reference's Newton step uses
 * the one contracted from the 2-RDM, equal to rounding).  With shci_orbital_gradient it gives
 * the approximate Newton step kappa_k = -grad_k / max(hdiag_k, 1e-5) (:315-328). */
shci_status shci_orbital_hessian_diagonal(shci_ctx* ctx, const uint32_t* p, const uint32_t* q,
                                          size_t n_param, double* hdiag);

/* rot = exp(X) with X[p_k][q_k] = -kappa_k, X[q_k][p_k] = kappa_k
 * (Optimization::fill_rot_matrix_with_parameters, optimization.cc:524-563); rot[i * n + j],
 * ready for shci_rotate_integrals. */
shci_status shci_orbital_rotation(shci_ctx* ctx, const uint32_t* p, const uint32_t* q,
                                  const double* kappa, size_t n_param, double* rot);

/* <S^2> of the first state of the context's wavefunction (ChemSystem::get_s2,
 * chem_system.cc:745-798; config "s2", post_variation :627-634).  A time_sym wavefunction must
 * be unpacked first (SHCI_ERR_ARG). */
shci_status shci_get_s2(shci_ctx* ctx, double* s2);

/* 1-RDM of the context's wavefunction: rdm1[p*n + r] = sum_ij c_i c_j <D_i| a+_r a_p |D_j>
 * summed over spin (rdm.cc:12-131), in the reordered orbital basis. */
shci_status shci_rdm1(shci_ctx* ctx, double* rdm1);

/* Spatial 2-RDM over the connections of the current Hamiltonian (rdm.cc:333-642), half
 * stored as the reference does: Gamma(p,q,r,s) = <a+_p a+_q a_r a_s> at index
 * A(A+1)/2 + B with A = max(p n + s, q n + r), B = min(...) (rdm.cc:233-241, 644-657);
 * rdm2_half has n^2 (n^2 + 1) / 2 entries.  E_var = E_core + sum_pq h_pq g1_pq +
 * 1/2 sum_pqrs Gamma(p,q,r,s) (ps|qr), with g1 the 2-RDM contraction (rdm.cc:707-753). */
shci_status shci_rdm2(shci_ctx* ctx, double* rdm2_half);

/* ---- orbital optimisation inputs (src/chem/optimization.cc) -------------------------- */

/* Generalized Fock matrix F[n*n] (row m, column n) of Optimization::get_generalized_Fock /
 * generalized_Fock_element (optimization.cc:620-650, Helgaker 10.8.24) from the device RDMs of
 * the current wavefunction (all states summed when n_states > 1):
 * F(m,n) = sum_q gamma(m,q) h(n,q) + sum_qrs Gamma(m,r,s,q) (nq|rs) for orbitals of equal irrep,
 * 0 otherwise.  Builds the Hamiltonian (FP64) if it is not current (the 2-RDM walks its
 * connections). */
shci_status shci_generalized_fock(shci_ctx* ctx, double* F);
/* Optimization::parameter_indices (optimization.cc:500-522, no active space): the pairs
 * p < q of equal irrep; *n = their count, up to cap written. */
shci_status shci_orbital_parameters(shci_ctx* ctx, uint32_t* p, uint32_t* q, size_t cap,
                                    size_t* n);
/* Optimization::gradient (optimization.cc:565-578): grad[k] = 2 (F(p_k,q_k) - F(q_k,p_k)). */
shci_status shci_orbital_gradient(shci_ctx* ctx, const uint32_t* p, const uint32_t* q,
                                  size_t n_param, double* grad);

#ifdef __cplusplus
}
#endif

#endif /* SHCI_GPU_H */

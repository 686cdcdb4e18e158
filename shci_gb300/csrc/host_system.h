// Host-side chemistry system of the product library: FCIDUMP reading, orbital reordering,
// dense integral tables and the heat-bath queues that are uploaded to HBM.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace shci {

struct HostIntegrals {
  unsigned n = 0;            // spatial orbitals
  unsigned n_up = 0, n_dn = 0;
  double e_core = 0.0;
  std::vector<unsigned> orb_sym;    // 1-based irreps, reordered
  std::vector<unsigned> orb_order;  // new index -> FCIDUMP index (0-based)
  std::vector<double> h1;           // [n*n]
  std::vector<double> g2;           // [n^4]
  uint64_t hf_up = 0, hf_dn = 0;
  unsigned n_syms = 1;
  // Linear molecules (D-infinity-h / C-infinity-v): irreps are (Lz, g/u) labels in the
  // reference's "Adam's notation" and products add Lz (src/chem/dooh_util.cc).
  bool linear = false;

  double h(unsigned p, unsigned q) const { return h1[p * n + q]; }
  double g(unsigned p, unsigned q, unsigned r, unsigned s) const {
    return g2[((size_t)(p * n + q) * n + r) * n + s];
  }
};

// HF det options of Integrals::generate_det_hf (src/chem/integrals.cc:155-226): without
// explicit occupations, the HF det fills each listed irrep ("chem/irreps") with its
// "chem/irrep_occs_up" / "chem/irrep_occs_dn" electrons in orbital order (and then counts as
// explicit: no reordering by default), or else the lowest orbitals, the beta electrons on
// top of the alpha ones when "allow_doubly_occupy_hf" is false.
struct HfOptions {
  bool allow_doubly_occupy = true;
  std::vector<unsigned> irreps, irrep_occs_up, irrep_occs_dn;
};

// Reads FCIDUMP and prepares the integrals like Integrals::load (src/chem/integrals.cc:17-384).
// Throws std::runtime_error with a message on failure.
void load_fcidump(HostIntegrals& I, const std::string& path, unsigned n_up, unsigned n_dn,
                  const std::string& point_group, int reorder, const unsigned* occs_up,
                  const unsigned* occs_dn, const HfOptions& hf = HfOptions());

// Orbitals outside the active space (Integrals::reorder_orbs, src/chem/integrals.cc:295-326):
// per irrep k the first irrep_active_space[k] orbitals of irrep k + 1, in orbital order, are
// active, and an orbital above the highest active orbital of its irrep may not be an
// excitation target (chem_system.cc:327-329, 383-387).  An irrep with no active orbital
// allows none of its orbitals as targets (the reference reads past an empty list there).
// Throws std::invalid_argument when fewer entries than irreps are given.
uint64_t inactive_orbitals(const HostIntegrals& I, const std::vector<unsigned>& irrep_active_space);

// Integrals cache: Integrals::save_to_cache / load_from_cache (src/chem/integrals.cc:17-35,
// 424-440) keep the prepared integrals (after orbital reordering) in "integrals_cache.dat" so
// that a later run skips FCIDUMP parsing.  The reference writes its Integrals fields with hps,
// an un-vendored library whose byte format is not available; this build stores the same fields
// in its own little-endian layout:
//
//   8 bytes   magic "SHCIGIC1"
//   u32       n_orbs, n_up, n_dn
//   f64       energy_core
//   u32       orb_sym[n_orbs]     (irreps after reordering; linear groups: Adam's labels)
//   u32       orb_order[n_orbs]   (new index -> FCIDUMP index)
//   u64       det_hf up, dn
//   f64       h1[n*n], g2[n^4]    (dense, reordered basis; g2 at ((p*n+q)*n+r)*n+s)
//
// The point group is not stored (the reference's cache does not hold it either): the caller
// passes it again.  Load returns kCacheMissing or kCacheForeign (a file not in this layout,
// for instance one the reference wrote) without touching I; save does not overwrite a foreign
// file.  A file in this layout that is truncated or inconsistent throws std::runtime_error.
enum CacheStatus { kCacheMissing = 0, kCacheOk = 1, kCacheForeign = 2 };
CacheStatus load_integrals_cache(HostIntegrals& I, const std::string& path,
                                 const std::string& point_group);
CacheStatus save_integrals_cache(const HostIntegrals& I, const std::string& path);

// Number of irreps of a point group name as ProductTable::get_n_syms counts them
// (src/chem/product_table.cc:37-47; 128 for the linear groups); *linear tells whether the name
// is one of the linear groups ("Dooh", "Dih", "Coov", "Civ": ChemSystem::get_point_group,
// src/chem/chem_system.cc:198-221, maps all four to D-infinity-h).
unsigned point_group_order(const std::string& pg, bool* linear = nullptr);

// Lz and g/u of a linear-group irrep label (DoohUtil::get_lz, src/chem/dooh_util.cc:5-15).
int linear_lz(int label, int* gu);
// Product of two irreps (ProductTable::get_product, product_table.cc:31-36 and
// DoohUtil::get_product, dooh_util.cc:27-33).
unsigned irrep_product(bool linear, unsigned a, unsigned b);
// Zeroes every (pq|rs) whose orbitals do not conserve Lz, lz_p + lz_r != lz_q + lz_s: the
// test Integrals::get_2b applies to every two-body lookup once the system's point group is
// linear (src/chem/integrals.cc:394-406).  No-op unless I.linear.
void screen_linear(HostIntegrals& I);

// Heat-bath queues in CSR form (src/chem/chem_system.cc:74-196).
struct HostQueues {
  // doubles: pair index pq = combine2(p, q) over spin-orbitals (q may be >= n)
  std::vector<uint64_t> d_off;   // [n_pairs + 1]
  std::vector<double> d_H;       // |H|, descending within a pair
  std::vector<uint32_t> d_rs;    // r | s << 16 (spin-orbital indices as the reference stores)
  // singles: per spatial orbital p
  std::vector<uint32_t> s_off;   // [n + 1]
  std::vector<double> s_S;       // upper bound S, descending
  std::vector<uint32_t> s_r;
  double max_hci = 0.0, max_singles = 0.0;
};

void build_queues(const HostIntegrals& I, HostQueues& Q);

double host_diag(const HostIntegrals& I, uint64_t up, uint64_t dn);

// Host threads a host-side loop of the calling thread may use: the machine's hardware threads
// unless the calling thread set a cap (the batch runner's workers each take their share).
unsigned host_threads();
void set_host_threads(unsigned n);  // 0 = no cap

inline size_t combine2(size_t a, size_t b) {
  return a > b ? (a * (a + 1)) / 2 + b : (b * (b + 1)) / 2 + a;
}

}  // namespace shci

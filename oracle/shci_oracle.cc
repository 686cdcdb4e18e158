// SHCI oracle: a plain C++17 + OpenMP restatement of the reference's (QMC-Cornell/shci,
// "Arrow") CPU algorithm for the hot path.  TEST INFRASTRUCTURE ONLY: the product library
// never links, loads or calls this file.  Only tests/, the smoke check and the bench's CPU
// baseline leg use it, and there only as the checker / the timed CPU restatement.
//
// Each function cites the reference file:line it follows.  Half-determinants are one 64-bit
// word (n_orbs <= 64); the reference's second chunk (N_CHUNKS=2, src/det/half_det.h:10) is
// always zero for such sizes and is carried explicitly where it changes a result (the hash).
//
// Determinant order: the reference appends each selection pass's new dets in the iteration
// order of an un-vendored distributed hash set (src/solver/solver.h:475-487), which is not
// reproducible.  This restatement appends them sorted by Det::operator< (src/det/det.h:16-18)
// instead (the "canonical order").  Everything else follows the reference line by line.
//
// Floating point: compiled with -ffp-contract=off so x86 and Arm builds agree bit for bit.

#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <numeric>
#include <queue>
#include <random>
#include <regex>
#include <stack>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#include <omp.h>

namespace orc {

constexpr double EPS = 1.0e-12;   // src/util.h:50
constexpr double INF = 1.0e100;   // src/util.h:52

static inline int popc(uint64_t x) { return __builtin_popcountll(x); }

constexpr double kSqrt2 = 1.4142135623730951;     // src/util.h:58
constexpr double kSqrt2Inv = 0.7071067811865475;  // src/util.h:60
static inline int ctz(uint64_t x) { return __builtin_ctzll(x); }

// ---------------------------------------------------------------- determinants (C1)
struct Det {
  uint64_t up, dn;
  bool operator==(const Det& o) const { return up == o.up && dn == o.dn; }
  bool operator!=(const Det& o) const { return !(*this == o); }
  // src/det/det.h:16-18 (HalfDet order compares the high chunk first; one chunk here)
  bool operator<(const Det& o) const { return up < o.up || (up == o.up && dn < o.dn); }
};

// src/det/half_det.cc:71-89 with N_CHUNKS=2: the second chunk (always 0) still runs a round.
static inline uint64_t half_hash(uint64_t c0) {
  uint64_t h = 0;
  h += c0;
  h += (h << 10);
  h ^= (h >> 6);
  h += 0;
  h += (h << 10);
  h ^= (h >> 6);
  h += (h << 3);
  h ^= (h >> 11);
  h += (h << 15);
  return h;
}

// src/det/det.h:42-49
static inline uint64_t det_hash(const Det& d) {
  uint64_t seed = half_hash(d.up);
  seed ^= half_hash(d.dn) + 0x9e3779b9ull + (seed << 6) + (seed >> 2);
  return seed;
}

// src/util.cc:111-122
static inline uint64_t rehash(uint64_t a) {
  uint64_t hash = a;
  hash += (hash << 10);
  hash ^= (hash >> 6);
  hash += 982451653ull;
  hash += (hash << 10);
  hash ^= (hash >> 6);
  hash += (hash << 3);
  hash ^= (hash >> 11);
  hash += (hash << 15);
  return hash;
}

struct DetHasher {
  size_t operator()(const Det& d) const { return det_hash(d); }
};
struct HalfHasher {
  size_t operator()(uint64_t h) const { return half_hash(h); }
};

// src/det/diff_result.h
struct Diff {
  unsigned left[2] = {0, 0};
  unsigned right[2] = {0, 0};
  unsigned n = 0;
  int perm = 1;
};

// src/det/half_det.cc:120-206 (one chunk).  left = orbitals only in a, right = only in b.
static Diff diff(uint64_t a, uint64_t b) {
  Diff res;
  if (a == b) return res;
  unsigned nl = 0, nr = 0, helper = 0;
  uint64_t lo = a & ~b;
  while (lo) {
    if (nl >= 2) {
      res.n = 3;
      return res;
    }
    const int tz = ctz(lo);
    const uint64_t bit = 1ull << tz;
    lo &= ~bit;
    res.left[nl++] = tz;
    helper += popc(a & (bit - 1));
  }
  uint64_t ro = b & ~a;
  while (ro) {
    if (nr >= 2) {
      res.n = 3;
      return res;
    }
    const int tz = ctz(ro);
    const uint64_t bit = 1ull << tz;
    ro &= ~bit;
    res.right[nr++] = tz;
    helper += popc(b & (bit - 1));
  }
  res.n = nl;
  if (helper & 1) res.perm = -1;
  return res;
}

static std::vector<unsigned> occ(uint64_t h) {  // src/det/half_det.cc:55-69
  std::vector<unsigned> r;
  while (h) {
    const int tz = ctz(h);
    h &= ~(1ull << tz);
    r.push_back(tz);
  }
  return r;
}

// ---------------------------------------------------------------- integrals (C2)
static size_t combine2(size_t a, size_t b) {  // src/chem/integrals.cc:410-416
  return a > b ? (a * (a + 1)) / 2 + b : (b * (b + 1)) / 2 + a;
}
static size_t combine4(size_t a, size_t b, size_t c, size_t d) {  // :418-422
  return combine2(combine2(a, b), combine2(c, d));
}

struct Hpqrs {
  double H;
  unsigned p, q, r, s;
};

struct Integrals {
  unsigned n_orbs = 0, n_elecs = 0, n_up = 0, n_dn = 0;
  double energy_core = 0.0;
  std::vector<unsigned> orb_sym, orb_order, orb_order_inv;
  std::vector<double> h1, g2;  // packed by combine2 / combine4, 0.0 = absent
  std::vector<Hpqrs> raw;
  Det det_hf{0, 0};
  bool explicit_orbs = false;

  // Linear point groups: Lz of each (reordered) orbital, and whether lookups screen by it
  // (set once the system's point group is known, after loading: chem_system.cc:33-34).
  bool lz_screen = false;
  std::vector<int> lz;

  double get_1b(unsigned p, unsigned q) const { return h1[combine2(p, q)]; }
  // src/chem/integrals.cc:394-406
  double get_2b(unsigned p, unsigned q, unsigned r, unsigned s) const {
    if (lz_screen && lz[p] + lz[r] != lz[q] + lz[s]) return 0.;
    return g2[combine4(p, q, r, s)];
  }
  // Reducer used on duplicate keys: the larger |v| wins (src/chem/integrals.cc:104-111).
  static void set(std::vector<double>& v, size_t key, double x) {
    if (v[key] == 0.0 || std::abs(v[key]) < std::abs(x)) v[key] = x;
  }
};

// src/chem/integrals.cc:116-153
static std::vector<unsigned> adams_syms(const std::vector<int>& raw) {
  bool neg = false;
  for (int o : raw)
    if (o < 0) neg = true;
  std::vector<unsigned> res(raw.size());
  if (!neg) {
    for (size_t i = 0; i < raw.size(); i++) res[i] = raw[i];
    return res;
  }
  for (size_t i = 0; i < raw.size(); i++) {
    const int s = raw[i];
    if (s == 1 || s == 2) {
      res[i] = s;
      continue;
    }
    const unsigned a = std::abs(s) >> 1;
    const unsigned b = (std::abs(s) + 1) >> 1;
    unsigned v = a + 3 * b - 8;
    if (s < 0) v += 2;
    res[i] = v;
  }
  return res;
}

// src/chem/integrals.cc:37-114 (read_fcidump)
static void read_fcidump(Integrals& I, const std::string& path) {
  std::ifstream f(path);
  if (!f.good()) throw std::runtime_error("cannot open FCIDUMP");
  std::regex words("([\\-]?[^\\s,=\\-]+)");
  std::string line;
  enum class State { NONE, ORBSYM, END };
  State state = State::NONE;
  std::vector<int> raw_syms;
  while (!f.eof()) {
    std::getline(f, line);
    auto wb = std::sregex_iterator(line.begin(), line.end(), words);
    auto we = std::sregex_iterator();
    for (auto it = wb; it != we; it++) {
      const std::string m = it->str();
      if (m == "NORB" || m == "NORBS") {
        it++;
        I.n_orbs = std::stoul(it->str());
      } else if (m == "NELEC") {
        it++;
        I.n_elecs = std::stoul(it->str());
      } else if (m == "ORBSYM") {
        state = State::ORBSYM;
      } else if (state == State::ORBSYM) {
        raw_syms.push_back(std::stoi(m));
        if (raw_syms.size() == I.n_orbs) state = State::NONE;
      } else if (m == "&END" || m == "/") {
        state = State::END;
      }
    }
    if (state == State::END) break;
  }
  I.orb_sym = adams_syms(raw_syms);
  double v;
  unsigned p, q, r, s;
  while (true) {
    f >> v >> p >> q >> r >> s;
    if (f.eof()) break;
    if (std::abs(v) < 1.0e-9) continue;
    I.raw.push_back(Hpqrs{v, p, q, r, s});
  }
}

static void fill_tables(Integrals& I, const std::vector<unsigned>& inv) {
  const size_t n = I.n_orbs;
  const size_t n2 = combine2(n - 1, n - 1) + 1;
  I.h1.assign(n2, 0.0);
  I.g2.assign(combine2(n2 - 1, n2 - 1) + 1, 0.0);
  for (const auto& it : I.raw) {
    if (it.p == 0 && it.q == 0 && it.r == 0 && it.s == 0) {
      I.energy_core = it.H;
    } else if (it.r == 0 && it.s == 0) {
      Integrals::set(I.h1, combine2(inv[it.p - 1], inv[it.q - 1]), it.H);
    } else {
      Integrals::set(
          I.g2, combine4(inv[it.p - 1], inv[it.q - 1], inv[it.r - 1], inv[it.s - 1]), it.H);
    }
  }
}

struct LoadOptions {
  int reorder = -1;  // -1: default (!explicit_orbs), 0/1 forced
  std::vector<unsigned> occs_up, occs_dn;
  // integrals.cc:163-164, 179-185: "chem/irreps" with "chem/irrep_occs_up/dn", and
  // "allow_doubly_occupy_hf"
  std::vector<unsigned> irreps, irrep_occs_up, irrep_occs_dn;
  bool allow_doubly_occupy = true;
};

// src/chem/integrals.cc:17-35, 155-226 (fill-lowest / explicit occs), 228-384 (reorder)
static void load_integrals(Integrals& I, const std::string& path, unsigned n_up, unsigned n_dn,
                           const LoadOptions& opt) {
  read_fcidump(I, path);
  if (I.n_orbs > 64) throw std::runtime_error("oracle supports n_orbs <= 64");
  std::vector<unsigned> ident(I.n_orbs);
  std::iota(ident.begin(), ident.end(), 0);
  I.energy_core = 0.0;
  fill_tables(I, ident);
  // generate_det_hf
  I.n_up = n_up;
  I.n_dn = n_dn;
  I.n_elecs = n_up + n_dn;
  I.det_hf = Det{0, 0};
  I.explicit_orbs = false;
  if (!opt.occs_up.empty() || !opt.occs_dn.empty()) {
    if (opt.occs_up.size() != n_up || opt.occs_dn.size() != n_dn)
      throw std::invalid_argument("occs do not match n_up/n_dn");
    for (unsigned o : opt.occs_up) I.det_hf.up |= 1ull << o;
    for (unsigned o : opt.occs_dn) I.det_hf.dn |= 1ull << o;
    I.explicit_orbs = true;
  } else if (opt.irreps.empty()) {
    // fill lowest (:176-185)
    for (unsigned i = 0; i < n_up; i++) I.det_hf.up |= 1ull << i;
    if (opt.allow_doubly_occupy) {
      for (unsigned i = 0; i < n_dn; i++) I.det_hf.dn |= 1ull << i;
    } else {
      for (unsigned i = 0; i < n_dn; i++) I.det_hf.dn |= 1ull << (i + n_up);
    }
  } else {
    // fill according to irreps (:186-215)
    for (size_t i = 0; i < opt.irreps.size(); i++) {
      const unsigned irrep = opt.irreps[i];
      unsigned occ_up = opt.irrep_occs_up.at(i), occ_dn = opt.irrep_occs_dn.at(i);
      for (unsigned j = 0; j < I.n_orbs; j++) {
        if (I.orb_sym[j] != irrep) continue;
        if (occ_up > 0) {
          I.det_hf.up |= 1ull << j;
          occ_up--;
        } else {
          I.det_hf.up &= ~(1ull << j);
        }
        if (occ_dn > 0) {
          I.det_hf.dn |= 1ull << j;
          occ_dn--;
        } else {
          I.det_hf.dn &= ~(1ull << j);
        }
        if (occ_up == 0 && occ_dn == 0 && j >= n_up && j >= n_dn) break;
      }
      if (occ_up > 0 || occ_dn > 0) throw std::runtime_error("unable to construct hf with given irrep");
    }
    I.explicit_orbs = true;
  }
  // get_orb_energies (:228-255), with the un-reordered tables
  const unsigned n = I.n_orbs;
  std::vector<double> e(n);
  const auto ou = occ(I.det_hf.up), od = occ(I.det_hf.dn);
  for (unsigned i = 0; i < n; i++) {
    e[i] = I.get_1b(i, i);
    double direct = 0, exch = 0;
    for (unsigned o : ou) {
      if (o == i) {
        direct += I.get_2b(i, i, o, o);
      } else {
        direct += 2 * I.get_2b(i, i, o, o);
        exch -= I.get_2b(i, o, o, i);
      }
    }
    for (unsigned o : od) {
      if (o == i) {
        direct += I.get_2b(i, i, o, o);
      } else {
        direct += 2 * I.get_2b(i, i, o, o);
        exch -= I.get_2b(i, o, o, i);
      }
    }
    e[i] += 0.5 * (direct + exch);
  }
  // reorder_orbs (:257-384)
  I.orb_order.resize(n);
  I.orb_order_inv.resize(n);
  std::iota(I.orb_order.begin(), I.orb_order.end(), 0);
  const bool do_reorder = opt.reorder < 0 ? !I.explicit_orbs : opt.reorder != 0;
  if (do_reorder) {
    std::stable_sort(I.orb_order.begin(), I.orb_order.end(),
                     [&](unsigned a, unsigned b) { return e[a] < e[b] - EPS; });
  }
  std::vector<unsigned> sym_new(n);
  for (unsigned i = 0; i < n; i++) sym_new[i] = I.orb_sym[I.orb_order[i]];
  I.orb_sym = sym_new;
  for (unsigned i = 0; i < n; i++) I.orb_order_inv[I.orb_order[i]] = i;
  Det hf{0, 0};
  for (unsigned i = 0; i < n; i++) {
    if (I.det_hf.up >> I.orb_order[i] & 1) hf.up |= 1ull << i;
    if (I.det_hf.dn >> I.orb_order[i] & 1) hf.dn |= 1ull << i;
  }
  I.det_hf = hf;
  fill_tables(I, I.orb_order_inv);
  I.raw.clear();
}

// ---------------------------------------------------------------- symmetry (C3)
// src/chem/dooh_util.cc:5-45: linear-group labels.  1, 2: Lz = 0 (g, u); label >= 3:
// |Lz| = 1 + (label - 3) / 4, the sign from bit 1 of (label - 1), g/u from the parity.
static int dooh_lz(int ind, int& gu) {
  if (ind <= 2) {
    gu = ind - 1;
    return 0;
  }
  int lz = 1 + ((ind - 3) >> 2);
  if ((((ind - 1) >> 1) & 1) == 0) lz = -lz;
  gu = (ind + 1) & 1;
  return lz;
}
static int dooh_ind(int lz, int gu) {
  if (lz == 0) return gu + 1;
  int ind = (std::abs(lz) << 2) - 1 + gu;
  if (lz < 0) ind += 2;
  return ind;
}
static unsigned dooh_inverse(unsigned i) {
  int gu;
  const int lz = dooh_lz(static_cast<int>(i), gu);
  return lz > 0 ? i + 2 : lz < 0 ? i - 2 : i;
}

// src/chem/product_table.cc:5-47: the C1..D2h tables are the XOR group on (irrep-1); the
// linear groups add Lz and combine g/u.
static unsigned sym_product(bool dooh, unsigned a, unsigned b) {
  if (!dooh) return ((a - 1) ^ (b - 1)) + 1;
  int ga, gb;
  const int la = dooh_lz(static_cast<int>(a), ga), lb = dooh_lz(static_cast<int>(b), gb);
  return static_cast<unsigned>(dooh_ind(la + lb, (ga + gb) & 1));
}

// src/chem/chem_system.cc:198-221 and product_table.cc:43-47 (128 irreps for Dooh)
static unsigned point_group_order(const std::string& pg, bool& dooh) {
  std::string s;
  for (char c : pg) s.push_back(std::tolower(c));
  dooh = false;
  if (s == "c1") return 1;
  if (s == "c2" || s == "cs" || s == "ci") return 2;
  if (s == "c2v" || s == "c2h" || s == "d2") return 4;
  if (s == "d2h") return 8;
  if (s == "coov" || s == "civ" || s == "dooh" || s == "dih") {
    dooh = true;
    return 128;
  }
  throw std::invalid_argument("point group not supported by the oracle: " + pg);
}

// ---------------------------------------------------------------- the chemistry system
struct Hrs {
  double H;
  unsigned r, s;
};
struct Sr {
  double S;
  unsigned r;
};

struct System {
  Integrals I;
  unsigned n_orbs = 0, n_up = 0, n_dn = 0, n_elecs = 0;
  unsigned n_syms = 1;
  bool dooh = false;
  std::vector<std::vector<unsigned>> sym_orbs;
  std::vector<std::vector<Hrs>> hci_queue;
  std::vector<std::vector<Sr>> singles_queue;
  double max_hci = 0.0, max_singles = 0.0;
  size_t n_hci_entries = 0, n_singles_entries = 0;
  double energy_hf = 0.0;
  double energy_hf_1b = 0.0;
  double second_rejection_factor = 0.2;
  bool has_double_excitation = true;
  // "chem/active_space" (chem_system.cc:30, integrals.cc:295-326): the highest active orbital
  // of each irrep; empty = no active space
  bool enforce_active_space = false;
  std::vector<int> highest_occ_orb_in_irrep;

  std::vector<Det> dets;
  std::vector<double> coefs;  // state 0
  double energy_var = 0.0;    // state 0
  // n_states > 1 (config "n_states", chem_system.cc:24, 52-56): the coefficients and
  // variational energies of states 1 .. n_states - 1
  unsigned n_states = 1;
  std::vector<std::vector<double>> xcoefs;
  std::vector<double> xenergy_var;
  // time-reversal symmetry (config "time_sym"): a det with up != dn stands for
  // (|up,dn> + |dn,up>) / sqrt(2); the list holds the form with up <= dn
  bool time_sym = false;

  // ------------------------------------------------ Slater-Condon (C6)
  // src/chem/chem_system.cc:444-457
  double one_body_diag(const Det& d) const {
    double e = 0.0;
    for (unsigned o : occ(d.up)) e += I.get_1b(o, o);
    if (d.up == d.dn) {
      e *= 2;
    } else {
      for (unsigned o : occ(d.dn)) e += I.get_1b(o, o);
    }
    return e;
  }
  // src/chem/chem_system.cc:495-542 without the diag_helper cache
  double two_body_diag(const Det& d) const {
    const auto ou = occ(d.up), od = occ(d.dn);
    double direct = 0.0, exch = 0.0;
    for (size_t i = 0; i < ou.size(); i++)
      for (size_t j = i + 1; j < ou.size(); j++) {
        direct += I.get_2b(ou[i], ou[i], ou[j], ou[j]);
        exch -= I.get_2b(ou[i], ou[j], ou[j], ou[i]);
      }
    if (d.up == d.dn) {
      direct *= 2;
      exch *= 2;
    } else {
      for (size_t i = 0; i < od.size(); i++)
        for (size_t j = i + 1; j < od.size(); j++) {
          direct += I.get_2b(od[i], od[i], od[j], od[j]);
          exch -= I.get_2b(od[i], od[j], od[j], od[i]);
        }
    }
    for (size_t i = 0; i < ou.size(); i++)
      for (size_t j = 0; j < od.size(); j++) direct += I.get_2b(ou[i], ou[i], od[j], od[j]);
    return direct + exch;
  }
  // src/chem/chem_system.cc:544-550
  double one_body_single(const Diff& du, const Diff& dd) const {
    const Diff& df = du.n == 1 ? du : dd;
    return df.perm * I.get_1b(df.left[0], df.right[0]);
  }
  // src/chem/chem_system.cc:552-577
  double two_body_single(const Det& di, const Diff& du, const Diff& dd) const {
    const bool is_up = du.n == 1;
    const Diff& df = is_up ? du : dd;
    const unsigned oi = df.left[0], oj = df.right[0];
    const uint64_t same = is_up ? di.up : di.dn;
    uint64_t oppo = is_up ? di.dn : di.up;
    double e = 0.0;
    for (unsigned o : occ(same)) {
      if (o == oi || o == oj) continue;
      e -= I.get_2b(oi, o, o, oj);
      const double direct = I.get_2b(oi, oj, o, o);
      if (oppo >> o & 1) {
        oppo &= ~(1ull << o);
        e += 2 * direct;
      } else {
        e += direct;
      }
    }
    for (unsigned o : occ(oppo)) e += I.get_2b(oi, oj, o, o);
    e *= df.perm;
    return e;
  }
  // src/chem/chem_system.cc:579-609
  double two_body_double(const Diff& du, const Diff& dd) const {
    double e = 0.0;
    if (du.n == 0) {
      if (dd.n != 2) return 0.0;
      e = I.get_2b(dd.left[0], dd.right[0], dd.left[1], dd.right[1]) -
          I.get_2b(dd.left[0], dd.right[1], dd.left[1], dd.right[0]);
      e *= dd.perm;
    } else if (dd.n == 0) {
      if (du.n != 2) return 0.0;
      e = I.get_2b(du.left[0], du.right[0], du.left[1], du.right[1]) -
          I.get_2b(du.left[0], du.right[1], du.left[1], du.right[0]);
      e *= du.perm;
    } else {
      if (du.n != 1 || dd.n != 1) return 0.0;
      e = I.get_2b(du.left[0], du.right[0], dd.left[0], dd.right[0]);
      e *= du.perm * dd.perm;
    }
    return e;
  }
  // src/chem/chem_system.cc:409-442
  // src/base_system.h:86-101 (SQRT2 = src/util.h:58)
  double hamiltonian_elem_time_sym(const Det& di, const Det& dj, int n_excite) const {
    double h = hamiltonian_elem(di, dj, n_excite);
    if (di.up == di.dn) {
      if (dj.up != dj.dn) h *= kSqrt2;
    } else {
      if (dj.up == dj.dn) {
        h *= kSqrt2;
      } else {
        const Det r{di.dn, di.up};
        h += hamiltonian_elem(r, dj, -1);
      }
    }
    return h;
  }

  // src/base_system.h:108-123: every det with up < dn gets its reverse appended, both
  // coefficients divided by sqrt(2) (SQRT2_INV = src/util.h:60)
  // <S^2> of a state: src/chem/chem_system.cc:745-798 (serial here, same terms)
  double get_s2(const std::vector<double>& state_coefs) const {
    std::unordered_map<Det, double, DetHasher> det2coef;
    for (size_t i = 0; i < dets.size(); i++) det2coef[dets[i]] = state_coefs[i];
    double s2 = 0.;
    const double nu = n_up, nd = n_dn;
    for (size_t i_det = 0; i_det < dets.size(); i_det++) {
      const Det this_det = dets[i_det];
      unsigned num_db_occ = 0;
      for (unsigned o : occ(this_det.up))
        if (this_det.dn >> o & 1) num_db_occ++;
      double diag = 0.5 * nu - num_db_occ + 0.5 * nd;
      diag += 0.25 * (std::pow(nu, 2) + std::pow(nd, 2)) - 0.5 * nu * nd;
      diag *= std::pow(state_coefs[i_det], 2);
      s2 += diag;
      for (unsigned i_orb = 0; i_orb < n_orbs; i_orb++) {
        if (!(this_det.dn >> i_orb & 1)) continue;
        if (this_det.up >> i_orb & 1) continue;
        for (unsigned j_orb = i_orb + 1; j_orb < n_orbs; j_orb++) {
          if (!(this_det.up >> j_orb & 1)) continue;
          if (this_det.dn >> j_orb & 1) continue;
          Det new_det = this_det;
          new_det.up &= ~(1ull << j_orb);
          new_det.up |= 1ull << i_orb;
          new_det.dn &= ~(1ull << i_orb);
          new_det.dn |= 1ull << j_orb;
          const auto it = det2coef.find(new_det);
          if (it == det2coef.end()) continue;
          const double perm_up = diff(this_det.up, new_det.up).perm;
          const double perm_dn = diff(this_det.dn, new_det.dn).perm;
          s2 += -2 * it->second * state_coefs[i_det] * perm_up * perm_dn;
        }
      }
    }
    return s2;
  }

  void unpack_time_sym() {
    const size_t n_old = dets.size();
    for (size_t i = 0; i < n_old; i++) {
      const Det det = dets[i];
      if (det.up < det.dn) {
        auto half = [&](std::vector<double>& c) {
          const double v = c[i] * kSqrt2Inv;
          c[i] = v;
          c.push_back(v);
        };
        half(coefs);
        for (auto& xc : xcoefs) half(xc);
        dets.push_back(Det{det.dn, det.up});
      }
    }
  }

  double hamiltonian_elem(const Det& di, const Det& dj, int n_excite) const {
    Diff du, dd;
    if (n_excite < 0) {
      du = diff(di.up, dj.up);
      if (du.n > 2) return 0.0;
      dd = diff(di.dn, dj.dn);
      n_excite = du.n + dd.n;
      if (n_excite > 2) return 0.0;
    } else if (n_excite > 0) {
      du = diff(di.up, dj.up);
      if (du.n < static_cast<unsigned>(n_excite)) dd = diff(di.dn, dj.dn);
    }
    if (n_excite == 0) {
      return one_body_diag(di) + two_body_diag(di) + I.energy_core;
    } else if (n_excite == 1) {
      const double ob = one_body_single(du, dd);
      const double tb = two_body_single(di, du, dd);
      return ob + tb;
    } else if (n_excite == 2) {
      return two_body_double(du, dd);
    }
    throw std::runtime_error("hamiltonian with >2 excitation");
  }

  // ------------------------------------------------ heat-bath queues (C4)
  // src/chem/chem_system.cc:237-259
  double singles_queue_elem(unsigned i, unsigned j) const {
    if (i == j) return 0.0;
    std::vector<double> el;
    el.reserve(2 * n_orbs - 2);
    for (unsigned o = 0; o < n_orbs; o++) {
      const double ex = I.get_2b(i, o, o, j);
      const double direct = I.get_2b(i, j, o, o);
      if (o == i || o == j) {
        el.push_back(direct);
      } else {
        el.push_back(direct);
        el.push_back(direct - ex);
      }
    }
    std::sort(el.begin(), el.end());
    double smin = I.get_1b(i, j), smax = smin;
    for (unsigned k = 0; k < std::min(n_elecs - 1, 2 * n_orbs - 2); k++) {
      smin += el[k];
      smax += el[2 * n_orbs - 3 - k];
    }
    return std::max(std::abs(smin), std::abs(smax));
  }
  // src/chem/chem_system.cc:261-287
  double hci_queue_elem(unsigned p, unsigned q, unsigned r, unsigned s) const {
    if (p == q || r == s || p == r || q == s || p == s || q == r) return 0.0;
    Diff du, dd;
    if (p < n_orbs && q < n_orbs) {
      du.left[0] = p;
      du.left[1] = q;
      du.right[0] = r;
      du.right[1] = s;
      du.n = 2;
    } else {
      du.left[0] = p;
      dd.left[0] = q - n_orbs;
      du.right[0] = r;
      dd.right[0] = s - n_orbs;
      du.n = 1;
      dd.n = 1;
    }
    return std::abs(two_body_double(du, dd));
  }

  void setup(const std::string& fcidump, unsigned nu, unsigned nd, const std::string& pg,
             const LoadOptions& opt) {
    load_integrals(I, fcidump, nu, nd, opt);
    n_orbs = I.n_orbs;
    n_up = nu;
    n_dn = nd;
    n_elecs = nu + nd;
    n_syms = point_group_order(pg, dooh);
    if (dooh) {  // Integrals::set_point_group after load (chem_system.cc:33-34)
      I.lz.resize(n_orbs);
      for (unsigned o = 0; o < n_orbs; o++) {
        int gu;
        I.lz[o] = dooh_lz(static_cast<int>(I.orb_sym[o]), gu);
      }
      I.lz_screen = true;
    }
    // src/chem/chem_system.cc:65-72
    sym_orbs.assign(n_syms + 1, {});
    for (unsigned o = 0; o < n_orbs; o++) {
      const unsigned s = I.orb_sym[o];
      if (s >= sym_orbs.size()) sym_orbs.resize(s + 1);
      sym_orbs[s].push_back(o);
    }
    setup_hci_queue();
    setup_singles_queue();
    dets.assign(1, I.det_hf);
    coefs.assign(1, 1.0);
    energy_hf = hamiltonian_elem(I.det_hf, I.det_hf, 0);
    energy_var = 0.0;
  }

  // src/chem/chem_system.cc:74-113
  void setup_singles_queue() {
    singles_queue.assign(n_orbs, {});
    max_singles = 0.0;
    n_singles_entries = 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (unsigned p = 0; p < n_orbs; p++) {
      for (unsigned r : sym_orbs[I.orb_sym[p]]) {
        const double S = singles_queue_elem(p, r);
        if (S == 0.0) continue;
        singles_queue[p].push_back(Sr{S, r});
      }
      std::sort(singles_queue[p].begin(), singles_queue[p].end(),
                [](const Sr& a, const Sr& b) { return a.S > b.S; });
    }
    for (unsigned p = 0; p < n_orbs; p++) {
      n_singles_entries += singles_queue[p].size();
      if (!singles_queue[p].empty()) max_singles = std::max(max_singles, singles_queue[p][0].S);
    }
  }

  // src/chem/chem_system.cc:115-196
  void setup_hci_queue() {
    hci_queue.assign(combine2(n_orbs, 2 * n_orbs), {});
    max_hci = 0.0;
    n_hci_entries = 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (unsigned p = 0; p < n_orbs; p++) {
      const unsigned sp = I.orb_sym[p];
      for (unsigned q = p + 1; q < n_orbs; q++) {
        const size_t pq = combine2(p, q);
        const unsigned sq = sym_product(dooh, sp, I.orb_sym[q]);
        for (unsigned r = 0; r < n_orbs; r++) {
          unsigned sr = I.orb_sym[r];
          if (dooh) sr = dooh_inverse(sr);
          sr = sym_product(dooh, sq, sr);
          if (sr >= sym_orbs.size()) continue;
          for (unsigned s : sym_orbs[sr]) {
            if (s < r) continue;
            const double H = hci_queue_elem(p, q, r, s);
            if (H == 0.0) continue;
            hci_queue[pq].push_back(Hrs{H, r, s});
          }
        }
        std::sort(hci_queue[pq].begin(), hci_queue[pq].end(),
                  [](const Hrs& a, const Hrs& b) { return a.H > b.H; });
      }
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (unsigned p = 0; p < n_orbs; p++) {
      const unsigned sp = I.orb_sym[p];
      for (unsigned q = n_orbs + p; q < 2 * n_orbs; q++) {
        const size_t pq = combine2(p, q);
        const unsigned sq = sym_product(dooh, sp, I.orb_sym[q - n_orbs]);
        for (unsigned r = 0; r < n_orbs; r++) {
          unsigned sr = I.orb_sym[r];
          if (dooh) sr = dooh_inverse(sr);
          sr = sym_product(dooh, sq, sr);
          if (sr >= sym_orbs.size()) continue;
          for (unsigned s : sym_orbs[sr]) {
            const double H = hci_queue_elem(p, q, r, s + n_orbs);
            if (H == 0.0) continue;
            hci_queue[pq].push_back(Hrs{H, r, s + n_orbs});
          }
        }
        std::sort(hci_queue[pq].begin(), hci_queue[pq].end(),
                  [](const Hrs& a, const Hrs& b) { return a.H > b.H; });
      }
    }
    for (const auto& qv : hci_queue) {
      n_hci_entries += qv.size();
      if (!qv.empty()) max_hci = std::max(max_hci, qv[0].H);
    }
  }

  // ------------------------------------------------ connected dets (C5)
  // src/chem/chem_system.cc:289-402
  double find_connected_dets(const Det& det, double eps_max, double eps_min,
                             const std::function<void(const Det&, int)>& handler,
                             bool second_rejection = false) const {
    if (eps_max < eps_min) return eps_min;
    const auto ou = occ(det.up), od = occ(det.dn);
    double diff_from_hf = -energy_hf_1b;
    if (second_rejection) {
      for (unsigned p : ou) diff_from_hf += I.get_1b(p, p);
      for (unsigned p : od) diff_from_hf += I.get_1b(p, p);
    }
    double max_rejection = 0.0;
    if (eps_min <= max_singles) {
      for (unsigned p_id = 0; p_id < n_elecs; p_id++) {
        const unsigned p = p_id < n_up ? ou[p_id] : od[p_id - n_up];
        for (const auto& sr : singles_queue[p]) {
          const double S = sr.S;
          if (S < eps_min) break;
          const unsigned r = sr.r;
          if (second_rejection) {
            const double den = diff_from_hf - I.get_1b(p, p) + I.get_1b(r, r);
            if (den > 0. && S * S / den < second_rejection_factor * eps_min * eps_min) {
              max_rejection = std::max(max_rejection, S);
              continue;
            }
          }
          if (enforce_active_space) {
            if (static_cast<int>(r) > highest_occ_orb_in_irrep[I.orb_sym[r] - 1]) continue;
          }
          Det c = det;
          if (p_id < n_up) {
            if (det.up >> r & 1) continue;
            c.up = (c.up & ~(1ull << p)) | (1ull << r);
          } else {
            if (det.dn >> r & 1) continue;
            c.dn = (c.dn & ~(1ull << p)) | (1ull << r);
          }
          handler(c, 1);
        }
      }
    }
    if (!has_double_excitation) return eps_min;
    if (eps_min > max_hci) return eps_min;
    const unsigned n = n_orbs;
    for (unsigned p_id = 0; p_id < n_elecs; p_id++) {
      for (unsigned q_id = p_id + 1; q_id < n_elecs; q_id++) {
        const unsigned p = p_id < n_up ? ou[p_id] : od[p_id - n_up] + n;
        const unsigned q = q_id < n_up ? ou[q_id] : od[q_id - n_up] + n;
        unsigned p2 = p, q2 = q;
        const bool both_dn = p >= n && q >= n;
        const bool swapped = p < n && q >= n && p > q - n;
        if (both_dn) {
          p2 -= n;
          q2 -= n;
        } else if (swapped) {
          p2 = q - n;
          q2 = p + n;
        }
        const size_t pq = combine2(p2, q2);
        for (const auto& hrs : hci_queue[pq]) {
          const double H = hrs.H;
          if (H < eps_min) break;
          if (H >= eps_max) continue;
          unsigned r = hrs.r, s = hrs.s;
          if (both_dn) {
            r += n;
            s += n;
          } else if (swapped) {
            const unsigned tmp = s - n;
            s = r + n;
            r = tmp;
          }
          if (second_rejection) {
            const double den = diff_from_hf - I.get_1b(p % n, p % n) - I.get_1b(q % n, q % n) +
                               I.get_1b(r % n, r % n) + I.get_1b(s % n, s % n);
            if (den > 0. && H * H / den < second_rejection_factor * eps_min * eps_min) {
              max_rejection = std::max(max_rejection, H);
              continue;
            }
          }
          if (enforce_active_space) {
            const unsigned rr = r % n, ss = s % n;
            if (static_cast<int>(rr) > highest_occ_orb_in_irrep[I.orb_sym[rr] - 1]) continue;
            if (static_cast<int>(ss) > highest_occ_orb_in_irrep[I.orb_sym[ss] - 1]) continue;
          }
          const bool occ_r = r < n ? (det.up >> r & 1) : (det.dn >> (r - n) & 1);
          if (occ_r) continue;
          const bool occ_s = s < n ? (det.up >> s & 1) : (det.dn >> (s - n) & 1);
          if (occ_s) continue;
          Det c = det;
          if (p < n) c.up &= ~(1ull << p); else c.dn &= ~(1ull << (p - n));
          if (q < n) c.up &= ~(1ull << q); else c.dn &= ~(1ull << (q - n));
          if (r < n) c.up |= 1ull << r; else c.dn |= 1ull << (r - n);
          if (s < n) c.up |= 1ull << s; else c.dn |= 1ull << (s - n);
          handler(c, 2);
        }
      }
    }
    return std::max(max_rejection, eps_min);
  }
};

// ---------------------------------------------------------------- sparse matrix (C8)
struct SparseMatrix {
  std::vector<std::vector<std::pair<uint32_t, double>>> rows;  // upper triangle incl. diag
  std::vector<double> diag;
  void set_dim(size_t n) {
    rows.resize(n);
    diag.resize(n, 0.0);
  }
  void append(size_t i, size_t j, double v) {  // src/solver/sparse_matrix.cc:8-11
    rows[i].emplace_back(static_cast<uint32_t>(j), v);
    if (i == j) diag[i] = v;
  }
  size_t n_upper() const {
    size_t c = 0;
    for (const auto& r : rows) c += r.size();
    return c;
  }
  // src/solver/sparse_matrix.cc:13-26
  size_t count_n_elems() const { return n_upper() * 2 - rows.size(); }
  // src/solver/sparse_matrix.cc:28-56, with per-thread partial vectors summed in thread order
  // instead of atomics (deterministic for a fixed thread count).
  std::vector<double> mul(const std::vector<double>& x) const {
    const size_t dim = rows.size();
    const int nt = omp_get_max_threads();
    std::vector<std::vector<double>> part(nt, std::vector<double>(dim, 0.0));
#pragma omp parallel
    {
      auto& y = part[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 64)
      for (size_t i = 0; i < dim; i++) {
        const auto& row = rows[i];
        double acc = 0.0;
        for (const auto& e : row) {
          const size_t j = e.first;
          acc += e.second * x[j];
          if (i != j) y[j] += e.second * x[i];
        }
        y[i] += acc;
      }
    }
    std::vector<double> y(dim, 0.0);
    for (int t = 0; t < nt; t++)
      for (size_t i = 0; i < dim; i++) y[i] += part[t][i];
    return y;
  }
};

// ---------------------------------------------------------------- Hamiltonian (C7)
// src/solver/hamiltonian.h, time_sym = false.
struct Hamiltonian {
  SparseMatrix matrix;
  size_t n_dets = 0, n_dets_prev = 0;
  bool sort_by_det_id = false;
  std::vector<uint64_t> unique_alphas, unique_betas;
  std::unordered_map<uint64_t, size_t, HalfHasher> alpha_to_id, beta_to_id;
  std::unordered_map<uint64_t, std::pair<std::vector<size_t>, std::vector<size_t>>, HalfHasher>
      abm1;
  std::vector<std::vector<size_t>> alpha_singles, beta_singles;
  std::vector<std::vector<size_t>> a2b, a2d, b2a, b2d;

  void clear() { *this = Hamiltonian(); }

  static void sort_by_first(std::vector<size_t>& v1, std::vector<size_t>& v2) {
    std::vector<std::pair<size_t, size_t>> v(v1.size());
    for (size_t i = 0; i < v1.size(); i++) v[i] = {v1[i], v2[i]};
    std::sort(v.begin(), v.end(),
              [](const std::pair<size_t, size_t>& a, const std::pair<size_t, size_t>& b) {
                return a.first < b.first;
              });
    for (size_t i = 0; i < v1.size(); i++) {
      v1[i] = v[i].first;
      v2[i] = v[i].second;
    }
  }

  // src/solver/hamiltonian.h:87-112
  void update(const System& sys) {
    n_dets_prev = n_dets;
    n_dets = sys.dets.size();
    if (n_dets_prev == n_dets) return;
    sort_by_det_id = (n_dets < n_dets_prev * 1.15);
    update_abdet(sys);
    if (sys.has_double_excitation) {
      update_abm1(sys);
      update_absingles(sys);
      abm1.clear();
    }
    update_matrix(sys);
    alpha_singles.clear();
    beta_singles.clear();
  }

  // src/solver/hamiltonian.h:157-254
  void update_abdet(const System& sys) {
    const bool ts = sys.time_sym;
    std::unordered_set<size_t> ua, ub;
    for (size_t i = n_dets_prev; i < n_dets; i++) {
      const Det& d = sys.dets[i];
      size_t aid, bid;
      auto ita = alpha_to_id.find(d.up);
      if (ita == alpha_to_id.end()) {
        aid = alpha_to_id.size();
        alpha_to_id[d.up] = aid;
        unique_alphas.push_back(d.up);
        a2b.resize(aid + 1);
        a2d.resize(aid + 1);
      } else {
        aid = ita->second;
      }
      ua.insert(aid);
      if (ts) {  // time_sym: beta strings take ids in the alpha id space (:182-198, 219-228)
        auto itb2 = alpha_to_id.find(d.dn);
        if (itb2 == alpha_to_id.end()) {
          bid = alpha_to_id.size();
          alpha_to_id[d.dn] = bid;
          unique_alphas.push_back(d.dn);
        } else {
          bid = itb2->second;
        }
        const size_t m = alpha_to_id.size();
        if (a2b.size() < m) {
          a2b.resize(m);
          a2d.resize(m);
        }
        if (b2a.size() < m) {
          b2a.resize(m);
          b2d.resize(m);
        }
        ub.insert(bid);
      } else {
        auto itb = beta_to_id.find(d.dn);
        if (itb == beta_to_id.end()) {
          bid = beta_to_id.size();
          beta_to_id[d.dn] = bid;
          unique_betas.push_back(d.dn);
          b2a.resize(bid + 1);
          b2d.resize(bid + 1);
        } else {
          bid = itb->second;
        }
        ub.insert(bid);
      }
      a2b[aid].push_back(bid);
      a2d[aid].push_back(i);
      b2a[bid].push_back(aid);
      b2d[bid].push_back(i);
    }
    if (sort_by_det_id) {
      for (size_t a : ua) sort_by_first(a2d[a], a2b[a]);
      for (size_t b : ub) sort_by_first(b2d[b], b2a[b]);
    } else {
      for (size_t a : ua) sort_by_first(a2b[a], a2d[a]);
      for (size_t b : ub) sort_by_first(b2a[b], b2d[b]);
    }
  }

  // src/solver/hamiltonian.h:256-305
  void update_abm1(const System& sys) {
    std::unordered_set<size_t> ua, ub;
    for (size_t i = n_dets_prev; i < n_dets; i++) {
      const Det& d = sys.dets[i];
      const size_t aid = alpha_to_id[d.up];
      if (!ua.count(aid)) {
        for (unsigned o : occ(d.up)) abm1[d.up & ~(1ull << o)].first.push_back(aid);
        ua.insert(aid);
      }
      if (sys.time_sym) {  // beta strings join the alpha lists (:277-287)
        const size_t bid = alpha_to_id[d.dn];
        if (!ua.count(bid)) {
          for (unsigned o : occ(d.dn)) abm1[d.dn & ~(1ull << o)].first.push_back(bid);
          ua.insert(bid);
        }
        continue;
      }
      const size_t bid = beta_to_id[d.dn];
      if (!ub.count(bid)) {
        for (unsigned o : occ(d.dn)) abm1[d.dn & ~(1ull << o)].second.push_back(bid);
        ub.insert(bid);
      }
    }
  }

  // src/solver/hamiltonian.h:307-413 (serial; the pair set is order independent)
  void update_absingles(const System& sys) {
    std::unordered_set<size_t> ua, ub;
    alpha_singles.resize(alpha_to_id.size());
    beta_singles.resize(beta_to_id.size());
    for (size_t i = n_dets_prev; i < n_dets; i++) {
      ua.insert(alpha_to_id[sys.dets[i].up]);
      if (sys.time_sym) ua.insert(alpha_to_id[sys.dets[i].dn]);  // (:316-325)
      else ub.insert(beta_to_id[sys.dets[i].dn]);
    }
    for (size_t aid = 0; aid < unique_alphas.size(); aid++) {
      const uint64_t a = unique_alphas[aid];
      for (unsigned o : occ(a)) {
        auto it = abm1.find(a & ~(1ull << o));
        if (it == abm1.end()) continue;
        for (size_t as : it->second.first) {
          if (as == aid) continue;
          if (aid > as && ua.count(aid) && ua.count(as)) continue;
          alpha_singles[aid].push_back(as);
          alpha_singles[as].push_back(aid);
        }
      }
    }
    for (size_t bid = 0; bid < unique_betas.size(); bid++) {
      const uint64_t b = unique_betas[bid];
      for (unsigned o : occ(b)) {
        auto it = abm1.find(b & ~(1ull << o));
        if (it == abm1.end()) continue;
        for (size_t bs : it->second.second) {
          if (bs == bid) continue;
          if (bid > bs && ub.count(bid) && ub.count(bs)) continue;
          beta_singles[bid].push_back(bs);
          beta_singles[bs].push_back(bid);
        }
      }
    }
    for (auto& v : alpha_singles) std::sort(v.begin(), v.end());
    for (auto& v : beta_singles) std::sort(v.begin(), v.end());
  }

  // src/solver/hamiltonian.h:415-598.  With time_sym the elements are
  // get_hamiltonian_elem_time_sym and each open det also meets the dets connected to its
  // reverse: same-string partners of the reversed strings (:448-459, 473-484) and mixed
  // doubles of the reverse (:535-590).
  void update_matrix(const System& sys) {
    matrix.set_dim(n_dets);
    const auto& dets = sys.dets;
    const bool ts = sys.time_sym;
    auto elem = [&](const Det& a, const Det& b, int nx) {
      return ts ? sys.hamiltonian_elem_time_sym(a, b, nx) : sys.hamiltonian_elem(a, b, nx);
    };
#pragma omp parallel for schedule(dynamic, 16)
    for (size_t det_id = 0; det_id < n_dets; det_id++) {
      const Det& det = dets[det_id];
      auto& row = matrix.rows[det_id];
      const bool is_new = det_id >= n_dets_prev;
      if (is_new) {
        const double H = elem(det, det, 0);
        row.emplace_back(static_cast<uint32_t>(det_id), H);
        matrix.diag[det_id] = H;
      }
      const size_t start_id = is_new ? det_id + 1 : n_dets_prev;
      const bool open = det.up != det.dn;
      auto take = [&](size_t j, double H) {
        if (std::abs(H) < EPS) return;
        row.emplace_back(static_cast<uint32_t>(j), H);
      };
      // alpha excitations: same beta string (:436-447), then the reverse's (:448-459)
      const size_t bid = ts ? alpha_to_id.at(det.dn) : beta_to_id.at(det.dn);
      for (size_t j : b2d[bid]) {
        if (j < start_id) continue;
        take(j, elem(det, dets[j], -1));
      }
      if (ts && open && a2d.size() > bid) {
        for (size_t j : a2d[bid]) {
          if (j < start_id) continue;
          const Det& c = dets[j];
          if (c.up == c.dn) continue;
          take(j, sys.hamiltonian_elem_time_sym(det, c, -1));
        }
      }
      // beta excitations: same alpha string (:461-472), then the reverse's (:473-484)
      const size_t aid = alpha_to_id.at(det.up);
      for (size_t j : a2d[aid]) {
        if (j < start_id) continue;
        take(j, elem(det, dets[j], -1));
      }
      if (ts && open && b2d.size() > aid) {
        for (size_t j : b2d[aid]) {
          if (j < start_id) continue;
          const Det& c = dets[j];
          if (c.up == c.dn) continue;
          take(j, sys.hamiltonian_elem_time_sym(det, c, -1));
        }
      }
      if (!sys.has_double_excitation && !ts) continue;
      // mixed doubles (:487-533)
      const auto& as_list = alpha_singles[aid];
      const auto& bs_list = ts ? alpha_singles[bid] : beta_singles[bid];
      for (size_t as : as_list) {
        if (a2b.size() <= as) continue;
        if (ts && as == bid) continue;
        const auto& rel_b = a2b[as];
        const auto& rel_d = a2d[as];
        const size_t nrel = rel_b.size();
        if (sort_by_det_id) {
          const size_t st =
              std::lower_bound(rel_d.begin(), rel_d.end(), start_id) - rel_d.begin();
          for (size_t k = st; k < nrel; k++) {
            if (ts && rel_b[k] == aid) continue;
            if (std::binary_search(bs_list.begin(), bs_list.end(), rel_b[k])) {
              const size_t j = rel_d[k];
              take(j, elem(det, dets[j], 2));
            }
          }
        } else {
          size_t ptr = 0;
          for (size_t bs : bs_list) {
            if (ts && bs == aid) continue;
            while (ptr < nrel && rel_b[ptr] < bs) ptr++;
            if (ptr == nrel) break;
            if (rel_b[ptr] == bs) {
              const size_t j = rel_d[ptr];
              ptr++;
              if (j < start_id) continue;
              take(j, elem(det, dets[j], 2));
            }
          }
        }
      }
      if (!(ts && open)) continue;
      // mixed doubles of the reverse (:535-590)
      const Det rev{det.dn, det.up};
      for (size_t as : as_list) {
        if (as == bid) continue;
        if (b2a.size() <= as) continue;
        const auto& rel_b = b2a[as];
        const auto& rel_d = b2d[as];
        const size_t nrel = rel_b.size();
        auto visit = [&](size_t j) {
          const Det& c = dets[j];
          if (c.up == c.dn) return;
          if (popc(c.up ^ det.up) == 2 && popc(c.dn ^ det.dn) == 2) return;
          take(j, sys.hamiltonian_elem_time_sym(rev, c, 2));
        };
        if (sort_by_det_id) {
          const size_t st =
              std::lower_bound(rel_d.begin(), rel_d.end(), start_id) - rel_d.begin();
          for (size_t k = st; k < nrel; k++) {
            if (rel_b[k] == aid) continue;
            if (std::binary_search(bs_list.begin(), bs_list.end(), rel_b[k])) visit(rel_d[k]);
          }
        } else {
          size_t ptr = 0;
          for (size_t bs : bs_list) {
            if (bs == aid) continue;
            while (ptr < nrel && rel_b[ptr] < bs) ptr++;
            if (ptr == nrel) break;
            if (rel_b[ptr] == bs) {
              const size_t j = rel_d[ptr];
              ptr++;
              if (j < start_id) continue;
              visit(j);
            }
          }
        }
      }
    }
  }
};

// ---------------------------------------------------------------- small symmetric eigensolver
// Cyclic Jacobi on the lower triangle of a k x k matrix (k <= 64).  Eigenvalues ascending,
// eigenvectors in columns.  Stands in for Eigen::SelfAdjointEigenSolver used at
// src/solver/davidson.cc:144-147.
static void jacobi_eig(int k, const std::vector<double>& lower, std::vector<double>& evals,
                       std::vector<double>& evecs) {
  std::vector<double> a(k * k), v(k * k, 0.0);
  for (int i = 0; i < k; i++)
    for (int j = 0; j <= i; j++) a[i * k + j] = a[j * k + i] = lower[i * k + j];
  for (int i = 0; i < k; i++) v[i * k + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < k; i++)
      for (int j = 0; j < k; j++) {
        tot += a[i * k + j] * a[i * k + j];
        if (i != j) off += a[i * k + j] * a[i * k + j];
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < k; p++)
      for (int q = p + 1; q < k; q++) {
        const double apq = a[p * k + q];
        if (apq == 0.0) continue;
        const double theta = (a[q * k + q] - a[p * k + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::abs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < k; r++) {
          const double arp = a[r * k + p], arq = a[r * k + q];
          a[r * k + p] = c * arp - s * arq;
          a[r * k + q] = s * arp + c * arq;
        }
        for (int r = 0; r < k; r++) {
          const double apr = a[p * k + r], aqr = a[q * k + r];
          a[p * k + r] = c * apr - s * aqr;
          a[q * k + r] = s * apr + c * aqr;
        }
        for (int r = 0; r < k; r++) {
          const double vrp = v[r * k + p], vrq = v[r * k + q];
          v[r * k + p] = c * vrp - s * vrq;
          v[r * k + q] = s * vrp + c * vrq;
        }
      }
  }
  std::vector<int> idx(k);
  std::iota(idx.begin(), idx.end(), 0);
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return a[x * k + x] < a[y * k + y]; });
  evals.resize(k);
  evecs.assign(k * k, 0.0);
  for (int c = 0; c < k; c++) {
    evals[c] = a[idx[c] * k + idx[c]];
    for (int r = 0; r < k; r++) evecs[r * k + c] = v[r * k + idx[c]];
  }
}

static double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
  return s;
}

// ---------------------------------------------------------------- Davidson (C9), one state
// src/solver/davidson.cc:8-196 with n_states = 1.
struct DavidsonResult {
  double eval = 0.0;
  std::vector<double> evec;
  bool converged = false;
  int n_matvec = 0;
};

static DavidsonResult davidson(const SparseMatrix& H, const std::vector<double>& init, double tol,
                               std::vector<double>* trace = nullptr) {
  DavidsonResult res;
  const size_t dim = init.size();
  if (dim == 1) {
    res.eval = H.diag[0];
    res.evec = {1.0};
    res.converged = true;
    return res;
  }
  const size_t store = std::min<size_t>(dim, 5);
  std::vector<std::vector<double>> v(store, std::vector<double>(dim)), Hv(store);
  std::vector<double> w(dim), Hw(dim);
  double norm = std::sqrt(dot(init, init));
  for (size_t j = 0; j < dim; j++) v[0][j] = init[j] / norm;
  std::vector<double> hk(store * store, 0.0);
  Hv[0] = H.mul(v[0]);
  res.n_matvec++;
  double lambda = dot(v[0], Hv[0]);
  hk[0] = lambda;
  w = v[0];
  Hw = Hv[0];
  if (trace) trace->push_back(lambda);
  double lambda_prev = lambda;
  bool converged = false;
  for (size_t it = 1; it < store * 2; it++) {
    const size_t ic = it % store;
    if (it >= store && ic == 0) {
      // restart: collapse onto the current Ritz vector (:115-131)
      v[0] = w;
      Hv[0] = Hw;
      lambda = dot(v[0], Hv[0]);
      hk[0] = lambda;
      continue;
    }
    for (size_t j = 0; j < dim; j++) {  // preconditioner (:135-143)
      const double d = lambda - H.diag[j];
      v[ic][j] = std::abs(d) < 1.0e-8 ? 0.0 : (Hw[j] - lambda * w[j]) / d;
    }
    for (size_t i = 0; i < ic; i++) {  // Gram-Schmidt (:146-152)
      const double nrm = dot(v[ic], v[i]);
      for (size_t j = 0; j < dim; j++) v[ic][j] -= nrm * v[i][j];
    }
    norm = std::sqrt(dot(v[ic], v[ic]));
    if (norm < 1e-12) {
      converged = true;
      break;
    }
    for (size_t j = 0; j < dim; j++) v[ic][j] /= norm;
    Hv[ic] = H.mul(v[ic]);
    res.n_matvec++;
    for (size_t i = 0; i <= ic; i++) hk[ic * store + i] = dot(v[i], Hv[ic]);
    const int k = static_cast<int>(ic + 1);
    std::vector<double> lower(k * k, 0.0), ev, evec;
    for (int i = 0; i < k; i++)
      for (int j = 0; j <= i; j++) lower[i * k + j] = hk[i * store + j];
    jacobi_eig(k, lower, ev, evec);
    lambda = ev[0];
    const double factor = evec[0] < 0 ? -1.0 : 1.0;
    std::vector<double> ek(k);
    for (int i = 0; i < k; i++) ek[i] = evec[i * k + 0] * factor;
    for (size_t j = 0; j < dim; j++) {
      double wj = 0.0, hwj = 0.0;
      for (int i = 0; i < k; i++) {
        wj += v[i][j] * ek[i];
        hwj += Hv[i][j] * ek[i];
      }
      w[j] = wj;
      Hw[j] = hwj;
    }
    if (trace) trace->push_back(lambda);
    if (std::abs(lambda - lambda_prev) <= tol) converged = true;  // (:174-185)
    if (!converged) lambda_prev = lambda;
    if (converged) break;
  }
  res.eval = lambda;
  res.evec = w;
  res.converged = converged;
  return res;
}

// ---------------------------------------------------------------- Davidson, several states
// src/solver/davidson.cc:8-196 for any n_states: n_states * 5 stored vectors, the initial
// vectors normalised and orthogonalised in order, a subspace matrix that starts with only its
// diagonal set (:62-77), one preconditioned vector per step for state i_state_precond (cycling
// over the unconverged states), a subspace solve after the last state's vector, restarts that
// collapse onto the Ritz vectors (:86-103), and convergence state by state (:174-186).
struct DavidsonStates {
  std::vector<double> evals;
  std::vector<std::vector<double>> evecs;
  bool converged = false;
};

static DavidsonStates davidson_states(const SparseMatrix& H,
                                      const std::vector<std::vector<double>>& init, double tol,
                                      std::vector<std::vector<double>>* trace = nullptr) {
  DavidsonStates res;
  const size_t dim = init[0].size();
  const unsigned ns = static_cast<unsigned>(std::min(dim, init.size()));
  res.evals.assign(init.size(), 0.0);
  res.evecs.assign(init.size(), std::vector<double>(dim, 0.0));
  if (dim == 1) {
    res.evals[0] = H.diag[0];
    res.evecs[0] = {1.0};
    res.converged = true;
    return res;
  }
  const size_t nis = std::min<size_t>(dim, 5);
  const size_t m = ns * nis;
  std::vector<std::vector<double>> v(m, std::vector<double>(dim)), Hv(m), w(ns), Hw(ns);
  for (unsigned i = 0; i < ns; i++) {
    double norm = std::sqrt(dot(init[i], init[i]));
    for (size_t j = 0; j < dim; j++) v[i][j] = init[i][j] / norm;
    if (i > 0) {
      for (unsigned k = 0; k < i; k++) {
        const double ip = dot(v[i], v[k]);
        for (size_t j = 0; j < dim; j++) v[i][j] -= ip * v[k][j];
      }
      norm = std::sqrt(dot(v[i], v[i]));
      for (size_t j = 0; j < dim; j++) v[i][j] /= norm;
    }
  }
  std::vector<double> hk(m * m, 0.0);
  std::vector<double> lam(ns), lam_prev(ns);
  for (unsigned i = 0; i < ns; i++) {
    Hv[i] = H.mul(v[i]);
    lam[i] = dot(v[i], Hv[i]);
    hk[i * m + i] = lam[i];
    w[i] = v[i];
    Hw[i] = Hv[i];
  }
  if (trace) trace->push_back(lam);
  lam_prev = lam;
  bool converged = false;
  size_t n_conv = 0, precond = 0;
  for (size_t it = ns; it < m * 2; it++) {
    const size_t ic = it % m;
    if (it >= m) {
      if (ic < ns - 1) continue;
      if (ic == ns - 1) {
        for (unsigned i = 0; i < ns; i++) {
          v[i] = w[i];
          Hv[i] = Hw[i];
        }
        for (unsigned i = 0; i < ns; i++) {
          lam[i] = dot(v[i], Hv[i]);
          hk[i * m + i] = lam[i];
          for (unsigned k = i + 1; k < ns; k++) {
            const double e = dot(v[i], Hv[k]);
            hk[i * m + k] = e;
            hk[k * m + i] = e;
          }
        }
        continue;
      }
    }
    const double l = lam[precond];
    for (size_t j = 0; j < dim; j++) {
      const double d = l - H.diag[j];
      v[ic][j] = std::abs(d) < 1.0e-8 ? 0.0 : (Hw[precond][j] - l * w[precond][j]) / d;
    }
    for (size_t i = 0; i < ic; i++) {
      const double nrm = dot(v[ic], v[i]);
      for (size_t j = 0; j < dim; j++) v[ic][j] -= nrm * v[i][j];
    }
    const double norm = std::sqrt(dot(v[ic], v[ic]));
    if (norm < 1e-12) {
      converged = true;
      break;
    }
    for (size_t j = 0; j < dim; j++) v[ic][j] /= norm;
    Hv[ic] = H.mul(v[ic]);
    for (size_t i = 0; i <= ic; i++) hk[ic * m + i] = dot(v[i], Hv[ic]);
    if (precond + 1 == ns) {
      const int k = static_cast<int>(ic + 1);
      std::vector<double> lower(k * k, 0.0), ev, evec;
      for (int i = 0; i < k; i++)
        for (int j = 0; j <= i; j++) lower[i * k + j] = hk[i * m + j];
      jacobi_eig(k, lower, ev, evec);
      for (unsigned s = 0; s < ns; s++) {
        lam[s] = ev[s];
        const double factor = evec[0 * k + s] < 0 ? -1.0 : 1.0;
        std::vector<double> ek(k);
        for (int i = 0; i < k; i++) ek[i] = evec[i * k + s] * factor;
        w[s].assign(dim, 0.0);
        Hw[s].assign(dim, 0.0);
        for (size_t j = 0; j < dim; j++) {
          double wj = 0.0, hwj = 0.0;
          for (int i = 0; i < k; i++) {
            wj += v[i][j] * ek[i];
            hwj += Hv[i][j] * ek[i];
          }
          w[s][j] = wj;
          Hw[s][j] = hwj;
        }
      }
      if (trace) trace->push_back(lam);
      for (unsigned s = static_cast<unsigned>(n_conv); s < ns; s++) {
        if (std::abs(lam[s] - lam_prev[s]) > tol) break;
        n_conv++;
      }
      if (n_conv == ns) converged = true;
      if (!converged) lam_prev = lam;
      if (converged) break;
    }
    precond++;
    if (precond >= ns) precond = n_conv;
  }
  for (unsigned s = 0; s < ns; s++) {
    res.evals[s] = lam[s];
    res.evecs[s] = w[s];
  }
  for (size_t s = ns; s < init.size(); s++) res.evecs[s] = init[s];  // (:191-195)
  res.converged = converged;
  return res;
}

// ---------------------------------------------------------------- solver (C10, C11)
struct Solver {
  System sys;
  Hamiltonian ham;
  std::vector<double> eps_tried_prev;
  std::unordered_set<Det, DetHasher> var_dets;
  double target_error = 5.0e-5;
  bool var_sd = false;
  bool second_rejection = false;
  std::vector<size_t> iter_ndets, iter_nnz;
  std::vector<double> iter_energy;
  std::vector<std::vector<double>> iter_xenergy;  // states 1.. per iteration (n_states > 1)
  bool last_davidson_converged = false;

  // One selection step (src/solver/solver.h:435-495): five passes over i = j mod 5, each
  // pass's new dets appended in canonical (sorted) order.  Returns the number of new dets.
  size_t select(double eps_var) {
    const size_t n_dets = sys.dets.size();
    eps_tried_prev.resize(n_dets, INF);
    size_t n_new_total = 0;
    for (size_t j = 0; j < 5; j++) {
      const int nt = omp_get_max_threads();
      std::vector<std::vector<Det>> found(nt);
#pragma omp parallel for schedule(dynamic, 16)
      for (size_t i = j; i < n_dets; i += 5) {
        auto& out = found[omp_get_thread_num()];
        const Det& det = sys.dets[i];
        double max_coef = sys.coefs[i];  // the largest |c| over the states (solver.h:440-444)
        for (const auto& xc : sys.xcoefs)
          if (std::abs(xc[i]) > std::abs(max_coef)) max_coef = xc[i];
        double eps_min = eps_var / std::abs(max_coef);
        if (i == 0 && var_sd) eps_min = 0.0;
        if (sys.time_sym && det.up != det.dn) eps_min *= kSqrt2;  // (:451)
        if (eps_min >= eps_tried_prev[i]) continue;
        auto handler = [&](const Det& c, int n_excite) {
          Det reg = c;  // the stored form up <= dn (:453-455)
          if (sys.time_sym && c.up > c.dn) reg = Det{c.dn, c.up};
          if (var_dets.count(reg)) return;
          if (n_excite == 1) {
            const double h_ai = sys.hamiltonian_elem(det, c, 1);
            if (std::abs(h_ai) < eps_min) return;
          }
          out.push_back(reg);
        };
        if (second_rejection) {
          const double mr = sys.find_connected_dets(det, eps_tried_prev[i], eps_min, handler, true);
          eps_tried_prev[i] = 1.000000001 * mr;
        } else {
          sys.find_connected_dets(det, eps_tried_prev[i], eps_min, handler);
          eps_tried_prev[i] = 1.000000001 * eps_min;
        }
      }
      std::vector<Det> all;
      for (auto& f : found) all.insert(all.end(), f.begin(), f.end());
      std::sort(all.begin(), all.end());
      all.erase(std::unique(all.begin(), all.end()), all.end());
      for (const Det& d : all) {
        var_dets.insert(d);
        sys.dets.push_back(d);
        sys.coefs.push_back(1e-16);
        // solver.h:479-486: while the list is small, det k starts as state k's unit vector
        for (unsigned s = 1; s < sys.n_states; s++) {
          auto& xc = sys.xcoefs[s - 1];
          xc.push_back(n_dets <= 50 && xc.size() == s ? 1.0 : 1e-16);
        }
      }
      n_new_total += all.size();
    }
    return n_new_total;
  }

  // src/solver/solver.h:413-539 (n_states = 1)
  void run_variation(double eps_var, bool until_converged) {
    size_t n_dets = sys.dets.size();
    size_t n_dets_new = n_dets;
    double energy_prev = 0.0;
    bool converged = false, dets_converged = false;
    sys.energy_hf_1b = 0.0;
    if (second_rejection) {
      // ChemSystem::get_e_hf_1b (chem_system.cc:812-823)
      for (unsigned p : occ(sys.dets[0].up)) sys.energy_hf_1b += sys.I.get_1b(p, p);
      if (sys.time_sym) sys.energy_hf_1b *= 2.;
      else
        for (unsigned p : occ(sys.dets[0].dn)) sys.energy_hf_1b += sys.I.get_1b(p, p);
    }
    while (!converged) {
      if (!dets_converged) {
        n_dets_new = n_dets + select(eps_var);
        ham.update(sys);
      }
      const double tol = until_converged ? target_error / 500000 : target_error / 50;
      DavidsonResult dr;
      if (sys.n_states == 1) {
        dr = davidson(ham.matrix, sys.coefs, tol);
      } else {  // davidson.cc with n_states initial vectors
        std::vector<std::vector<double>> init(1, sys.coefs);
        init.insert(init.end(), sys.xcoefs.begin(), sys.xcoefs.end());
        DavidsonStates ds = davidson_states(ham.matrix, init, tol);
        dr.eval = ds.evals[0];
        dr.evec = ds.evecs[0];
        dr.converged = ds.converged;
        for (unsigned s = 1; s < sys.n_states; s++) {
          sys.xcoefs[s - 1] = ds.evecs[s];
          sys.xenergy_var[s - 1] = ds.evals[s];
        }
        iter_xenergy.push_back(std::vector<double>(ds.evals.begin() + 1, ds.evals.end()));
      }
      sys.coefs = dr.evec;
      last_davidson_converged = dr.converged;
      iter_ndets.push_back(n_dets_new);
      iter_nnz.push_back(ham.matrix.count_n_elems());
      iter_energy.push_back(dr.eval);
      if (n_dets_new < n_dets * 1.001) dets_converged = true;
      if (dets_converged && dr.converged) converged = true;
      n_dets = n_dets_new;
      energy_prev = dr.eval;
      if (!until_converged) break;
    }
    sys.energy_var = energy_prev;
  }

  // src/solver/solver.h:338-397 (no wf files: always computes)
  std::vector<double> run_all_variations(const std::vector<double>& eps_vars,
                                         const std::vector<double>& schedule) {
    std::vector<double> energies;
    double eps_var_prev = INF;
    for (const Det& d : sys.dets) var_dets.insert(d);
    size_t it_s = 0;
    for (double eps_var : eps_vars) {
      while (it_s < schedule.size() && schedule[it_s] >= eps_var_prev) it_s++;
      while (it_s < schedule.size() && schedule[it_s] > eps_var) {
        run_variation(schedule[it_s], false);
        it_s++;
      }
      run_variation(eps_var, true);
      energies.push_back(sys.energy_var);
      eps_var_prev = eps_var;
    }
    return energies;
  }

  // ------------------------------------------------ PT2 (C11): deterministic stage
  // src/solver/solver.h:636-764 with a given number of batches (>= 1).
  struct PtResult {
    double value = 0.0, uncert = 0.0;
    size_t n_pt_dets = 0;
  };
  PtResult pt_dtm(double eps_pt_dtm, size_t n_batches) {
    std::unordered_set<Det, DetHasher> vset(sys.dets.begin(), sys.dets.end());
    const size_t n_var = sys.dets.size();
    double esum = 0.0, esq = 0.0;
    size_t n_sum = 0;
    PtResult res;
    for (size_t batch = 0; batch < n_batches; batch++) {
      const int nt = omp_get_max_threads();
      std::vector<std::unordered_map<Det, double, DetHasher>> part(nt);
#pragma omp parallel for schedule(dynamic, 8)
      for (size_t i = 0; i < n_var; i++) {
        auto& m = part[omp_get_thread_num()];
        const Det& det = sys.dets[i];
        const double coef = sys.coefs[i];
        auto handler = [&](const Det& a, int n_excite) {
          if (rehash(det_hash(a)) % n_batches != batch) return;
          if (vset.count(a)) return;
          const double h_ai = sys.hamiltonian_elem(det, a, n_excite);
          const double hc = h_ai * coef;
          if (std::abs(hc) < eps_pt_dtm) return;
          m[a] += hc;
        };
        sys.find_connected_dets(det, INF / std::abs(coef), eps_pt_dtm / std::abs(coef), handler);
      }
      std::unordered_map<Det, double, DetHasher> hc;
      for (auto& m : part)
        for (auto& kv : m) hc[kv.first] += kv.second;
      std::vector<std::pair<Det, double>> items(hc.begin(), hc.end());
      double bs = 0.0, bsq = 0.0;
#pragma omp parallel for reduction(+ : bs, bsq)
      for (size_t k = 0; k < items.size(); k++) {
        const double Haa = sys.hamiltonian_elem(items[k].first, items[k].first, 0);
        const double c = items[k].second * items[k].second / (sys.energy_var - Haa);
        bs += c;
        bsq += c * c;
      }
      n_sum += items.size();
      esum += bs;
      esq += bsq;
      res.value = esum / (batch + 1) * n_batches;
      if (batch == n_batches - 1) {
        res.uncert = 0.0;
      } else {
        const double avg = esum / n_sum;
        const double sd = std::sqrt(esq / n_sum - avg * avg);
        res.uncert = sd * std::sqrt(n_sum) / (batch + 1) * (n_batches - batch - 1);
      }
    }
    res.n_pt_dets = n_sum;
    return res;
  }

  // ------------------------------------------------ PT2: pseudo-stochastic stage
  // src/solver/solver.h:766-896 with a given number of batches.
  PtResult pt_psto(double eps_dtm, double eps_psto, size_t n_batches, double target_error,
                   double eps_pt, size_t* batches_done) {
    std::unordered_set<Det, DetHasher> vset(sys.dets.begin(), sys.dets.end());
    const size_t n_var = sys.dets.size();
    double esum = 0.0, esq = 0.0;
    size_t n_sum = 0;
    PtResult res;
    *batches_done = 0;
    for (size_t batch = 0; batch < n_batches; batch++) {
      const int nt = omp_get_max_threads();
      std::vector<std::unordered_map<Det, std::array<double, 2>, DetHasher>> part(nt);
#pragma omp parallel for schedule(dynamic, 8)
      for (size_t i = 0; i < n_var; i++) {
        auto& m = part[omp_get_thread_num()];
        const Det& det = sys.dets[i];
        const double coef = sys.coefs[i];
        auto handler = [&](const Det& a, int n_excite) {
          if (rehash(det_hash(a)) % n_batches != batch) return;
          if (vset.count(a)) return;
          const double hc = sys.hamiltonian_elem(det, a, n_excite) * coef;
          if (std::abs(hc) < eps_psto) return;
          auto& v = m[a];
          v[0] += hc;
          if (std::abs(hc) >= eps_dtm) v[1] += hc;
        };
        sys.find_connected_dets(det, INF / std::abs(coef), eps_psto / std::abs(coef), handler);
      }
      std::unordered_map<Det, std::array<double, 2>, DetHasher> hc;
      for (auto& m : part)
        for (auto& kv : m) {
          auto& v = hc[kv.first];
          v[0] += kv.second[0];
          v[1] += kv.second[1];
        }
      double bs = 0.0, bsq = 0.0;
      for (auto& kv : hc) {
        const double d = kv.second[0] * kv.second[0] - kv.second[1] * kv.second[1];
        const double x = d / (sys.energy_var - sys.hamiltonian_elem(kv.first, kv.first, 0));
        bs += x;
        bsq += x * x;
      }
      n_sum += hc.size();
      esum += bs;
      esq += bsq;
      res.value = esum / (batch + 1) * n_batches;
      if (batch == n_batches - 1) {
        res.uncert = 0.0;
      } else {
        const double avg = esum / n_sum;
        const double sd = std::sqrt(esq / n_sum - avg * avg);
        res.uncert = sd / std::sqrt((double)n_sum) * n_sum / (batch + 1) * (n_batches - batch - 1);
      }
      *batches_done = batch + 1;
      if (res.uncert <= target_error * 0.5) break;
      if (eps_psto <= eps_pt && res.uncert <= target_error) break;
    }
    res.n_pt_dets = n_sum;
    return res;
  }

  // ------------------------------------------------ PT2: stochastic stage
  // src/solver/solver.h:898-1153.  n_samples == 0: the sample size comes from the 1,000-draw
  // pilot and the PT memory pt_mem_avail (solver.h:942-1006); semisto: the dets above the
  // quantile of the top quarter of the unique-sample target are deterministic
  // (solver.h:1009-1036).  info (may be null) = {n_samples, n_dtm, n_unique_target}.
  struct StoInfo {
    size_t n_samples = 0, n_dtm = 0, n_unique_target = 0;
  };
  PtResult pt_sto(double eps_psto, double eps_pt, size_t n_batches, size_t n_samples,
                  unsigned seed, size_t max_iter, double target_error, double psto_uncert,
                  std::vector<double>* loops, bool semisto = false, double pt_mem_avail = 0.0,
                  double mem_usage = 0.4, StoInfo* info = nullptr) {
    std::unordered_set<Det, DetHasher> vset(sys.dets.begin(), sys.dets.end());
    const size_t n_var = sys.dets.size();
    double sw = 0.0;
    for (size_t i = 0; i < n_var; i++) sw += std::abs(sys.coefs[i]);
    std::vector<double> probs(n_var), cum(n_var);
    for (size_t i = 0; i < n_var; i++) {
      probs[i] = std::abs(sys.coefs[i]) / sw;
      cum[i] = i > 0 ? probs[i] + cum[i - 1] : probs[i];
    }
    std::default_random_engine gen(seed);
    std::uniform_real_distribution<double> ur(0., 1.);
    size_t n_target = 0;
    if (n_samples == 0) {
      // pilot: 1,000 draws by inverse CDF, PT dets of the unique draws in hash batch 0 of 128
      std::unordered_map<size_t, unsigned> sto;
      std::vector<size_t> list;
      for (size_t k = 0; k < 1000; k++) {
        const double r = ur(gen);
        const size_t id = std::lower_bound(cum.begin(), cum.end(), r) - cum.begin();
        if (sto.count(id) == 0) list.push_back(id);
        sto[id]++;
      }
      const int nt = omp_get_max_threads();
      std::vector<std::unordered_set<Det, DetHasher>> part(nt);
#pragma omp parallel for schedule(dynamic, 1)
      for (size_t si = 0; si < list.size(); si++) {
        auto& m = part[omp_get_thread_num()];
        const Det& det = sys.dets[list[si]];
        const double coef = sys.coefs[list[si]];
        auto handler = [&](const Det& a, int n_excite) {
          if (vset.count(a)) return;
          if ((rehash(det_hash(a)) & 127) != 0) return;
          if (n_excite == 1) {
            const double hc = sys.hamiltonian_elem(det, a, n_excite) * coef;
            if (std::abs(hc) < eps_pt) return;
          }
          m.insert(a);
        };
        sys.find_connected_dets(det, INF / std::abs(coef), eps_pt / std::abs(coef), handler);
      }
      std::unordered_set<Det, DetHasher> pts;
      for (auto& m : part) pts.insert(m.begin(), m.end());
      const size_t n_pt_batch = pts.size() * 128 / n_batches;
      const size_t bytes_per_entry = 2 * 16 + 40;  // solver.h:402, 905 (two 64-bit chunks)
      const size_t cap = n_var / 8 + 1;
      // a pilot with no PT det gives the reference a division by zero; take the cap
      n_target = cap;
      if (n_pt_batch > 0) {
        const double t = static_cast<double>(static_cast<size_t>(pt_mem_avail)) * mem_usage *
                         static_cast<double>(list.size()) / static_cast<double>(bytes_per_entry) /
                         5.0 / static_cast<double>(n_pt_batch);
        n_target = static_cast<size_t>(t);
        if (n_target >= cap) n_target = cap;
      }
      sto.clear();
      size_t n_unique = 0;
      while (n_unique < n_target) {
        const double r = ur(gen);
        const size_t id = std::lower_bound(cum.begin(), cum.end(), r) - cum.begin();
        if (sto.count(id) == 0) n_unique++;
        n_samples++;
        sto[id]++;
      }
    }
    std::vector<size_t> dtm_list;
    if (semisto) {
      size_t n_heap = n_target / 4;
      if (n_heap == 0)
        throw std::runtime_error("semistochastic PT2 needs a sample-size target of at least 4 "
                                 "(the reference's quantile heap would be empty)");
      std::priority_queue<double, std::vector<double>, std::greater<double>> heap;
      for (size_t i = 0; i < n_heap; i++) heap.push(probs[i]);
      for (size_t i = n_heap; i < n_var; i++)
        if (heap.top() < probs[i]) {
          heap.pop();
          heap.push(probs[i]);
        }
      const double C = heap.top();
      double s2 = 0.0;
      for (size_t i = 0; i < n_var; i++) {
        if (probs[i] > C) {
          probs[i] = 0.;
          dtm_list.push_back(i);
        } else {
          s2 += probs[i];
        }
      }
      for (auto& p : probs) p /= s2;
    }
    const size_t n_dtm = dtm_list.size();
    if (info) {
      info->n_samples = n_samples;
      info->n_dtm = n_dtm;
      info->n_unique_target = n_target;
    }
    // Vose alias tables (src/util.cc:128-175)
    std::vector<double> ap(n_var), tp(n_var);
    std::vector<size_t> al(n_var, 0);
    {
      std::stack<size_t> sm, lg;
      for (size_t i = 0; i < n_var; i++) {
        tp[i] = probs[i] * n_var;
        if (tp[i] < 1.) sm.push(i); else lg.push(i);
      }
      while (!sm.empty() && !lg.empty()) {
        const size_t l = lg.top(), s = sm.top();
        ap[s] = tp[s];
        al[s] = l;
        tp[l] = tp[l] + tp[s] - 1.;
        if (tp[l] < 1.) {
          lg.pop();
          sm.top() = l;
        } else {
          sm.pop();
        }
      }
      while (!lg.empty()) { ap[lg.top()] = 1.; lg.pop(); }
      while (!sm.empty()) { ap[sm.top()] = 1.; sm.pop(); }
    }
    std::uniform_int_distribution<size_t> ui_var(0, n_var - 1);
    std::uniform_int_distribution<size_t> ui_batch(0, n_batches - 1);
    const double factor = 1. / (n_samples - n_dtm - 1.);
    PtResult res;
    std::vector<double> lv;
    size_t iteration = 0;
    while (iteration < max_iter) {
      std::unordered_map<size_t, unsigned> cnt;  // stochastic dets only
      std::vector<size_t> list = dtm_list;       // deterministic dets first
      for (size_t k = 0; k < n_samples - n_dtm; k++) {
        const size_t r1 = ui_var(gen);
        const double r2 = ur(gen);
        const size_t id = r2 < ap[r1] ? r1 : al[r1];
        if (cnt.count(id) == 0) list.push_back(id);
        cnt[id]++;
      }
      const size_t batch_id = ui_batch(gen);
      const int nt = omp_get_max_threads();
      std::vector<std::unordered_map<Det, std::array<double, 5>, DetHasher>> part(nt);
#pragma omp parallel for schedule(dynamic, 8)
      for (size_t si = 0; si < list.size(); si++) {
        auto& m = part[omp_get_thread_num()];
        const size_t i = list[si];
        const Det& det = sys.dets[i];
        const double coef = sys.coefs[i];
        const bool is_dtm = si < n_dtm;
        const double count = is_dtm ? 1. : static_cast<double>(cnt.at(i));
        const double weight = is_dtm ? 1. : (n_samples - n_dtm) * probs[i];
        auto handler = [&](const Det& a, int n_excite) {
          if (rehash(det_hash(a)) % n_batches != batch_id) return;
          if (vset.count(a)) return;
          const double hc = sys.hamiltonian_elem(det, a, n_excite) * coef;
          if (std::abs(hc) < eps_pt) return;
          auto& v = m[a];
          const double x = count * hc / weight;
          v[0] += x;
          if (std::abs(hc) > eps_psto) v[1] += x;
          if (!is_dtm) {
            const double x2 = count * hc / weight * std::sqrt(factor);
            if (std::abs(hc) > eps_psto) {
              v[2] += x2;
              v[3] += x2;
            } else {
              v[2] += x2;
              v[4] += std::pow(count * hc / weight, 2) * (1. - weight / count + factor);
            }
          }
        };
        sys.find_connected_dets(det, INF / std::abs(coef), eps_pt / std::abs(coef), handler);
      }
      std::unordered_map<Det, std::array<double, 5>, DetHasher> hc;
      for (auto& m : part)
        for (auto& kv : m) {
          auto& v = hc[kv.first];
          for (int k = 0; k < 5; k++) v[k] += kv.second[k];
        }
      double loop = 0.0;
      for (auto& kv : hc) {
        const auto& s = kv.second;
        const double f = static_cast<double>(n_batches) /
                         (sys.energy_var - sys.hamiltonian_elem(kv.first, kv.first, 0));
        loop += (s[0] * s[0] - s[1] * s[1] + s[2] * s[2] - s[3] * s[3] - s[4]) * f;
      }
      res.n_pt_dets += hc.size();
      lv.push_back(loop);
      const double n = static_cast<double>(lv.size());
      double sm = 0.0, sq = 0.0;
      for (double v : lv) {
        sm += v;
        sq += v * v;
      }
      res.value = sm / n;
      res.uncert = std::sqrt((sq - sm * sm / n) / (n - 1)) / std::sqrt(n);
      iteration++;
      if (iteration >= 6 && res.uncert <= target_error * 0.7) break;
      if (iteration >= 10 &&
          std::sqrt(res.uncert * res.uncert + psto_uncert * psto_uncert) <= target_error)
        break;
    }
    if (loops) *loops = lv;
    return res;
  }
};

// ---------------------------------------------------------------- RDMs (C13), time_sym = false
// src/chem/rdm.cc:12-131 (1-RDM), 233-269 (indexing / permfac), 333-371 + 435-657 (2-RDM).
static void rdm1(const System& sys, std::vector<double>& out) {
  const unsigned n = sys.n_orbs;
  out.assign(n * n, 0.0);
  std::unordered_map<Det, size_t, DetHasher> idx;
  for (size_t i = 0; i < sys.dets.size(); i++) idx[sys.dets[i]] = i;
  const auto& sym = sys.I.orb_sym;
  for (size_t i = 0; i < sys.dets.size(); i++) {
    const Det& d = sys.dets[i];
    for (int spin = 0; spin < 2; spin++) {
      const uint64_t h = spin == 0 ? d.up : d.dn;
      for (unsigned p : occ(h)) {
        for (unsigned r = 0; r < n; r++) {
          if (sym[p] != sym[r]) continue;
          if (p != r && (h >> r & 1)) continue;
          Det nd = d;
          const uint64_t nh = (h & ~(1ull << p)) | (1ull << r);
          if (spin == 0) nd.up = nh; else nd.dn = nh;
          auto it = idx.find(nd);
          if (it == idx.end()) continue;
          const double factor = diff(h, nh).perm;
          out[p * n + r] += sys.coefs[i] * sys.coefs[it->second] * factor;
        }
      }
    }
  }
}

struct Rdm2 {
  unsigned n;
  std::vector<double> half;
  const std::vector<double>* coefs;
  size_t idx(unsigned p, unsigned q, unsigned r, unsigned s) const {
    const size_t a = (size_t)p * n + s, b = (size_t)q * n + r;
    return a > b ? a * (a + 1) / 2 + b : b * (b + 1) / 2 + a;
  }
  void write(unsigned p, unsigned q, unsigned r, unsigned s, double f, size_t i, size_t j) {
    const size_t a = (size_t)p * n + s, b = (size_t)q * n + r;
    if (a >= b) half[a * (a + 1) / 2 + b] += (*coefs)[i] * (*coefs)[j] * f;
  }
  static unsigned bit_till(uint64_t h, unsigned p) { return popc(h & ((1ull << p) - 1)); }
  static int permfac_ccaa(uint64_t h, unsigned p, unsigned q, unsigned r, unsigned s) {
    unsigned c = 0;
    c += bit_till(h, s);
    h &= ~(1ull << s);
    c += bit_till(h, r);
    h &= ~(1ull << r);
    c += bit_till(h, q);
    h |= 1ull << q;
    c += bit_till(h, p);
    h |= 1ull << p;
    return c % 2 == 0 ? 1 : -1;
  }
  void elements(const Det& cd, size_t jd, const Det& td, size_t id, double tr,
                unsigned n_up, unsigned n_dn) {
    const auto ou = occ(td.up), od = occ(td.dn);
    if (td.up == cd.up) {
      if (td.dn == cd.dn) {
        for (unsigned a = 0; a < n_up; a++)
          for (unsigned b = a + 1; b < n_up; b++) {
            const unsigned s = ou[a], r = ou[b];
            write(s, r, r, s, tr, id, jd);
            write(s, r, s, r, -tr, id, jd);
            write(r, s, s, r, tr, id, jd);
            write(r, s, r, s, -tr, id, jd);
          }
        for (unsigned a = 0; a < n_dn; a++)
          for (unsigned b = a + 1; b < n_dn; b++) {
            const unsigned s = od[a], r = od[b];
            write(s, r, r, s, tr, id, jd);
            write(s, r, s, r, -tr, id, jd);
            write(r, s, s, r, tr, id, jd);
            write(r, s, r, s, -tr, id, jd);
          }
        for (unsigned a = 0; a < n_up; a++)
          for (unsigned b = 0; b < n_dn; b++) {
            const unsigned s = ou[a], r = od[b];
            write(s, r, r, s, tr, id, jd);
            write(r, s, s, r, tr, id, jd);
          }
      } else {
        const Diff dcd = diff(cd.dn, td.dn), dtd = diff(td.dn, cd.dn);
        if (dcd.n == 1) {
          const unsigned b1 = dcd.right[0], b2 = dcd.left[0];
          for (unsigned a = 0; a < n_dn; a++) {
            const unsigned p = od[a];
            if (p != b1 && p != b2) {
              double sf = tr * permfac_ccaa(td.dn, p, b2, b1, p);
              write(p, b2, b1, p, sf, id, jd);
              write(b2, p, b1, p, -sf, id, jd);
              write(p, b2, p, b1, -sf, id, jd);
              write(b2, p, p, b1, sf, id, jd);
              sf = tr * permfac_ccaa(cd.dn, p, b1, b2, p);
              write(p, b1, b2, p, sf, id, jd);
              write(b1, p, b2, p, -sf, id, jd);
              write(p, b1, p, b2, -sf, id, jd);
              write(b1, p, p, b2, sf, id, jd);
            }
          }
          for (unsigned a = 0; a < n_up; a++) {
            const unsigned p = ou[a];
            double sf = tr * dcd.perm;
            write(p, b2, b1, p, sf, id, jd);
            write(b2, p, p, b1, sf, id, jd);
            sf = tr * dtd.perm;
            write(p, b1, b2, p, sf, id, jd);
            write(b1, p, p, b2, sf, id, jd);
          }
        } else if (dcd.n == 2) {
          const unsigned b1 = dcd.right[0], b2 = dcd.right[1], b3 = dcd.left[0], b4 = dcd.left[1];
          double sf = tr * dcd.perm;
          write(b3, b4, b2, b1, sf, id, jd);
          write(b3, b4, b1, b2, -sf, id, jd);
          write(b4, b3, b2, b1, -sf, id, jd);
          write(b4, b3, b1, b2, sf, id, jd);
          sf = tr * dtd.perm;
          write(b1, b2, b4, b3, sf, id, jd);
          write(b1, b2, b3, b4, -sf, id, jd);
          write(b2, b1, b4, b3, -sf, id, jd);
          write(b2, b1, b3, b4, sf, id, jd);
        }
      }
    } else {
      const Diff cu = diff(cd.up, td.up), tu = diff(td.up, cd.up);
      if (cu.n == 1) {
        if (td.dn == cd.dn) {
          const unsigned a1 = cu.right[0], a2 = cu.left[0];
          for (unsigned a = 0; a < n_up; a++) {
            const unsigned p = ou[a];
            if (p != a1 && p != a2) {
              double sf = tr * permfac_ccaa(td.up, p, a2, a1, p);
              write(p, a2, a1, p, sf, id, jd);
              write(p, a2, p, a1, -sf, id, jd);
              write(a2, p, a1, p, -sf, id, jd);
              write(a2, p, p, a1, sf, id, jd);
              sf = tr * permfac_ccaa(cd.up, p, a1, a2, p);
              write(p, a1, a2, p, sf, id, jd);
              write(p, a1, p, a2, -sf, id, jd);
              write(a1, p, a2, p, -sf, id, jd);
              write(a1, p, p, a2, sf, id, jd);
            }
          }
          for (unsigned a = 0; a < n_dn; a++) {
            const unsigned p = od[a];
            double sf = tr * cu.perm;
            write(a2, p, p, a1, sf, id, jd);
            write(p, a2, a1, p, sf, id, jd);
            sf = tr * tu.perm;
            write(a1, p, p, a2, sf, id, jd);
            write(p, a1, a2, p, sf, id, jd);
          }
        } else {
          const Diff cdn = diff(cd.dn, td.dn), tdn = diff(td.dn, cd.dn);
          if (cdn.n == 1) {
            const unsigned a1 = cu.right[0], a2 = cu.left[0], b1 = cdn.right[0], b2 = cdn.left[0];
            double sf = tr * cu.perm * cdn.perm;
            write(a2, b2, b1, a1, sf, id, jd);
            write(b2, a2, a1, b1, sf, id, jd);
            sf = tr * tu.perm * tdn.perm;
            write(a1, b1, b2, a2, sf, id, jd);
            write(b1, a1, a2, b2, sf, id, jd);
          }
        }
      } else if (cu.n == 2) {
        if (td.dn == cd.dn) {
          const unsigned a1 = cu.right[0], a2 = cu.right[1], a3 = cu.left[0], a4 = cu.left[1];
          double sf = tr * cu.perm;
          write(a3, a4, a2, a1, sf, id, jd);
          write(a3, a4, a1, a2, -sf, id, jd);
          write(a4, a3, a2, a1, -sf, id, jd);
          write(a4, a3, a1, a2, sf, id, jd);
          sf = tr * tu.perm;
          write(a1, a2, a4, a3, sf, id, jd);
          write(a1, a2, a3, a4, -sf, id, jd);
          write(a2, a1, a4, a3, -sf, id, jd);
          write(a2, a1, a3, a4, sf, id, jd);
        }
      }
    }
  }
};

}  // namespace orc

// ================================================================ C ABI for the test harness
using namespace orc;

struct OrcHandle {
  Solver solver;
  std::string err;
  // rows of the last orc_hbuild_sample (strict upper part, increasing column order)
  std::vector<size_t> sample_rows;
  std::vector<std::vector<std::pair<uint32_t, double>>> sample_elems;
};

extern "C" {

void* orc_create(const char* fcidump, unsigned n_up, unsigned n_dn, const char* point_group,
                 int reorder, const unsigned* occs_up, const unsigned* occs_dn, char* err,
                 size_t err_len) {
  try {
    auto* h = new OrcHandle();
    LoadOptions opt;
    opt.reorder = reorder;
    if (occs_up) opt.occs_up.assign(occs_up, occs_up + n_up);
    if (occs_dn) opt.occs_dn.assign(occs_dn, occs_dn + n_dn);
    h->solver.sys.setup(fcidump, n_up, n_dn, point_group, opt);
    return h;
  } catch (const std::exception& e) {
    if (err && err_len) snprintf(err, err_len, "%s", e.what());
    return nullptr;
  }
}

// orc_create with the HF det options of integrals.cc:163-215 (n_irreps = 0: none).
void* orc_create_hf(const char* fcidump, unsigned n_up, unsigned n_dn, const char* point_group,
                    int reorder, int allow_doubly_occupy, const unsigned* irreps,
                    const unsigned* irrep_occs_up, const unsigned* irrep_occs_dn,
                    unsigned n_irreps, char* err, size_t err_len) {
  try {
    auto* h = new OrcHandle();
    LoadOptions opt;
    opt.reorder = reorder;
    opt.allow_doubly_occupy = allow_doubly_occupy != 0;
    if (n_irreps) {
      opt.irreps.assign(irreps, irreps + n_irreps);
      opt.irrep_occs_up.assign(irrep_occs_up, irrep_occs_up + n_irreps);
      opt.irrep_occs_dn.assign(irrep_occs_dn, irrep_occs_dn + n_irreps);
    }
    h->solver.sys.setup(fcidump, n_up, n_dn, point_group, opt);
    return h;
  } catch (const std::exception& e) {
    if (err && err_len) snprintf(err, err_len, "%s", e.what());
    return nullptr;
  }
}

void orc_destroy(void* h) { delete static_cast<OrcHandle*>(h); }

void orc_set_threads(int n) { omp_set_num_threads(n); }

static Solver& S(void* h) { return static_cast<OrcHandle*>(h)->solver; }

unsigned orc_n_orbs(void* h) { return S(h).sys.n_orbs; }

void orc_info(void* h, double* out) {
  auto& s = S(h).sys;
  out[0] = s.energy_hf;
  out[1] = s.max_hci;
  out[2] = static_cast<double>(s.n_hci_entries);
  out[3] = s.max_singles;
  out[4] = static_cast<double>(s.n_singles_entries);
  out[5] = s.I.energy_core;
}

void orc_hf(void* h, uint64_t* up, uint64_t* dn) {
  *up = S(h).sys.I.det_hf.up;
  *dn = S(h).sys.I.det_hf.dn;
}

// Dense reordered integrals: h1[p*n+q], g2[((p*n+q)*n+r)*n+s] (chemists' (pq|rs)).
void orc_integrals(void* h, double* h1, double* g2, unsigned* orb_sym, unsigned* orb_order) {
  auto& I = S(h).sys.I;
  const unsigned n = I.n_orbs;
  for (unsigned p = 0; p < n; p++)
    for (unsigned q = 0; q < n; q++) {
      if (h1) h1[p * n + q] = I.get_1b(p, q);
      if (g2)
        for (unsigned r = 0; r < n; r++)
          for (unsigned s = 0; s < n; s++)
            g2[((size_t)(p * n + q) * n + r) * n + s] = I.get_2b(p, q, r, s);
    }
  if (orb_sym)
    for (unsigned i = 0; i < n; i++) orb_sym[i] = I.orb_sym[i];
  if (orb_order)
    for (unsigned i = 0; i < n; i++) orb_order[i] = I.orb_order[i];
}

double orc_hamiltonian_elem(void* h, uint64_t ui, uint64_t di, uint64_t uj, uint64_t dj,
                            int n_excite) {
  return S(h).sys.hamiltonian_elem(Det{ui, di}, Det{uj, dj}, n_excite);
}

void orc_diff(uint64_t a, uint64_t b, unsigned* out /*left0,left1,right0,right1,n*/, int* perm) {
  const Diff d = diff(a, b);
  out[0] = d.left[0];
  out[1] = d.left[1];
  out[2] = d.right[0];
  out[3] = d.right[1];
  out[4] = d.n;
  *perm = d.perm;
}

uint64_t orc_det_hash(uint64_t up, uint64_t dn) { return det_hash(Det{up, dn}); }
uint64_t orc_rehash(uint64_t a) { return rehash(a); }

size_t orc_find_connected(void* h, uint64_t up, uint64_t dn, double eps_max, double eps_min,
                          uint64_t* out_up, uint64_t* out_dn, int* out_nex, size_t cap) {
  size_t cnt = 0;
  S(h).sys.find_connected_dets(Det{up, dn}, eps_max, eps_min, [&](const Det& c, int nex) {
    if (cnt < cap) {
      out_up[cnt] = c.up;
      out_dn[cnt] = c.dn;
      out_nex[cnt] = nex;
    }
    cnt++;
  });
  return cnt;
}

// Heat-bath queue of pair index pq (combine2 over spin-orbitals): sorted entries.
size_t orc_hci_queue(void* h, size_t pq, double* H, unsigned* r, unsigned* s, size_t cap) {
  const auto& q = S(h).sys.hci_queue.at(pq);
  for (size_t i = 0; i < q.size() && i < cap; i++) {
    H[i] = q[i].H;
    r[i] = q[i].r;
    s[i] = q[i].s;
  }
  return q.size();
}
size_t orc_singles_queue(void* h, unsigned p, double* Sv, unsigned* r, size_t cap) {
  const auto& q = S(h).sys.singles_queue.at(p);
  for (size_t i = 0; i < q.size() && i < cap; i++) {
    Sv[i] = q[i].S;
    r[i] = q[i].r;
  }
  return q.size();
}

void orc_set_dets(void* h, const uint64_t* up, const uint64_t* dn, const double* coefs, size_t n) {
  auto& s = S(h);
  s.sys.dets.resize(n);
  s.sys.coefs.resize(n);
  for (size_t i = 0; i < n; i++) {
    s.sys.dets[i] = Det{up[i], dn[i]};
    s.sys.coefs[i] = coefs ? coefs[i] : (i == 0 ? 1.0 : 1e-16);
  }
  for (auto& xc : s.sys.xcoefs) xc.assign(n, 1e-16);
  s.var_dets.clear();
  for (const auto& d : s.sys.dets) s.var_dets.insert(d);
  s.ham.clear();
  s.eps_tried_prev.clear();
}

size_t orc_n_dets(void* h) { return S(h).sys.dets.size(); }

void orc_get_dets(void* h, uint64_t* up, uint64_t* dn, double* coefs) {
  auto& s = S(h).sys;
  for (size_t i = 0; i < s.dets.size(); i++) {
    up[i] = s.dets[i].up;
    dn[i] = s.dets[i].dn;
    if (coefs) coefs[i] = s.coefs[i];
  }
}

void orc_set_coefs(void* h, const double* c) {
  auto& s = S(h).sys;
  for (size_t i = 0; i < s.dets.size(); i++) s.coefs[i] = c[i];
}

// Incremental Hamiltonian update (hamiltonian.h:87-112).  Returns upper-triangle nnz.
size_t orc_update_hamiltonian(void* h) {
  auto& s = S(h);
  s.ham.update(s.sys);
  return s.ham.matrix.n_upper();
}

void orc_clear_hamiltonian(void* h) { S(h).ham.clear(); }

// Rows in append order: row_ptr[n+1], cols[nnz], vals[nnz].
void orc_get_hamiltonian(void* h, uint64_t* row_ptr, uint32_t* cols, double* vals) {
  const auto& m = S(h).ham.matrix;
  size_t k = 0;
  for (size_t i = 0; i < m.rows.size(); i++) {
    row_ptr[i] = k;
    for (const auto& e : m.rows[i]) {
      cols[k] = e.first;
      vals[k] = e.second;
      k++;
    }
  }
  row_ptr[m.rows.size()] = k;
}

void orc_hv(void* h, const double* x, double* y) {
  const auto& m = S(h).ham.matrix;
  std::vector<double> xv(x, x + m.rows.size());
  auto yv = m.mul(xv);
  std::copy(yv.begin(), yv.end(), y);
}

// Davidson on the current matrix (davidson.cc).  coefs in/out.  trace gets the eigenvalue
// estimate after each step (up to trace_cap).
int orc_davidson(void* h, double* coefs, double tol, double* eval, double* trace, size_t trace_cap,
                 size_t* n_trace) {
  auto& s = S(h);
  std::vector<double> init(coefs, coefs + s.sys.dets.size());
  std::vector<double> tr;
  auto r = davidson(s.ham.matrix, init, tol, &tr);
  std::copy(r.evec.begin(), r.evec.end(), coefs);
  *eval = r.eval;
  if (trace)
    for (size_t i = 0; i < tr.size() && i < trace_cap; i++) trace[i] = tr[i];
  if (n_trace) *n_trace = tr.size();
  return r.converged ? 1 : 0;
}

// Time-reversal symmetry (config "time_sym"; needs n_up == n_dn).  Set before any variation.
void orc_set_time_sym(void* h, int on) {
  auto& s = S(h);
  s.sys.time_sym = on != 0;
  s.ham.clear();
}

// Solver::run_perturbation's unpack_time_sym (solver.h:593, base_system.h:108-123).
void orc_unpack_time_sym(void* h) {
  auto& s = S(h);
  s.sys.unpack_time_sym();
  s.var_dets.clear();
  for (const auto& d : s.sys.dets) s.var_dets.insert(d);
  s.ham.clear();
  s.eps_tried_prev.clear();
}

// Number of states (ChemSystem::setup, chem_system.cc:24, 52-56): states 1.. start at 1e-16 on
// every current det.
void orc_set_n_states(void* h, unsigned ns) {
  auto& s = S(h).sys;
  s.n_states = ns < 1 ? 1 : ns;
  s.xcoefs.assign(s.n_states - 1, std::vector<double>(s.dets.size(), 1e-16));
  s.xenergy_var.assign(s.n_states - 1, 0.0);
}

// Coefficients of state st (0 = the main vector).
void orc_get_state_coefs(void* h, unsigned st, double* out) {
  auto& s = S(h).sys;
  const auto& v = st == 0 ? s.coefs : s.xcoefs.at(st - 1);
  std::copy(v.begin(), v.end(), out);
}

void orc_set_state_coefs(void* h, unsigned st, const double* c) {
  auto& s = S(h).sys;
  auto& v = st == 0 ? s.coefs : s.xcoefs.at(st - 1);
  std::copy(c, c + s.dets.size(), v.begin());
}

// energies[n_states] of the last variational run; per_iter[n_iter * n_states] if non-null
void orc_state_energies(void* h, double* energies, double* per_iter) {
  auto& S_ = S(h);
  auto& s = S_.sys;
  energies[0] = s.energy_var;
  for (unsigned k = 1; k < s.n_states; k++) energies[k] = s.xenergy_var[k - 1];
  if (per_iter)
    for (size_t it = 0; it < S_.iter_energy.size(); it++) {
      per_iter[it * s.n_states] = S_.iter_energy[it];
      for (unsigned k = 1; k < s.n_states; k++)
        per_iter[it * s.n_states + k] =
            it < S_.iter_xenergy.size() ? S_.iter_xenergy[it][k - 1] : 0.0;
    }
}

// Several-state Davidson on an explicit upper-triangle CSR: init[ns * n] in, evecs[ns * n] and
// evals[ns] out.  Returns 1 when converged.
int orc_davidson_csr_states(size_t n, const uint64_t* row_ptr, const uint32_t* cols,
                            const double* vals, unsigned ns, const double* init, double tol,
                            double* evals, double* evecs) {
  SparseMatrix m;
  m.set_dim(n);
  for (size_t i = 0; i < n; i++)
    for (uint64_t k = row_ptr[i]; k < row_ptr[i + 1]; k++) m.append(i, cols[k], vals[k]);
  std::vector<std::vector<double>> iv(ns);
  for (unsigned s = 0; s < ns; s++) iv[s].assign(init + s * n, init + (s + 1) * n);
  auto r = davidson_states(m, iv, tol);
  for (unsigned s = 0; s < ns; s++) {
    evals[s] = r.evals[s];
    std::copy(r.evecs[s].begin(), r.evecs[s].end(), evecs + s * n);
  }
  return r.converged ? 1 : 0;
}

// Davidson on an explicit upper-triangle CSR (for the Hilbert-matrix golden test).
int orc_davidson_csr(size_t n, const uint64_t* row_ptr, const uint32_t* cols, const double* vals,
                     double* coefs, double tol, double* eval) {
  SparseMatrix m;
  m.set_dim(n);
  for (size_t i = 0; i < n; i++)
    for (uint64_t k = row_ptr[i]; k < row_ptr[i + 1]; k++) m.append(i, cols[k], vals[k]);
  std::vector<double> init(coefs, coefs + n);
  auto r = davidson(m, init, tol);
  std::copy(r.evec.begin(), r.evec.end(), coefs);
  *eval = r.eval;
  return r.converged ? 1 : 0;
}

size_t orc_select(void* h, double eps_var, int var_sd) {
  auto& s = S(h);
  s.var_sd = var_sd != 0;
  if (s.var_dets.size() != s.sys.dets.size()) {
    s.var_dets.clear();
    for (const auto& d : s.sys.dets) s.var_dets.insert(d);
  }
  return s.select(eps_var);
}

void orc_eps_tried(void* h, double* out) {
  auto& s = S(h);
  for (size_t i = 0; i < s.eps_tried_prev.size(); i++) out[i] = s.eps_tried_prev[i];
}

// Full variational stage.  energies[n_eps] out.  Per-iteration trace available after.
void orc_run_all_variations(void* h, const double* eps_vars, size_t n_eps, const double* sched,
                            size_t n_sched, double target_error, int second_rejection,
                            double* energies) {
  auto& s = S(h);
  s.target_error = target_error;
  s.second_rejection = second_rejection != 0;
  std::vector<double> ev(eps_vars, eps_vars + n_eps), sc(sched, sched + n_sched);
  auto e = s.run_all_variations(ev, sc);
  std::copy(e.begin(), e.end(), energies);
}

// Second rejection for single selection steps (orc_select): the flag and energy_hf_1b as
// run_variation sets them (solver.h:426-428, chem_system.cc:812-823).
void orc_set_has_double_excitation(void* h, int on) { S(h).sys.has_double_excitation = on != 0; }

// "chem/active_space" with "chem/irrep_active_space" (integrals.cc:295-326): the lowest
// irrep_active_space[k] orbitals of irrep k + 1 (in orbital order) are active.  n = 0: off.
void orc_set_active_space(void* h, const unsigned* irrep_active_space, unsigned n) {
  auto& sys = S(h).sys;
  sys.enforce_active_space = n > 0;
  sys.highest_occ_orb_in_irrep.clear();
  if (!n) return;
  const unsigned n_irreps = *std::max_element(sys.I.orb_sym.begin(), sys.I.orb_sym.end());
  std::vector<std::vector<unsigned>> active(n_irreps);
  for (unsigned i = 0; i < sys.n_orbs; i++) {
    const unsigned k = sys.I.orb_sym[i] - 1;
    if (k < n && active[k].size() < irrep_active_space[k]) active[k].push_back(i);
  }
  sys.highest_occ_orb_in_irrep.assign(n_irreps, -1);
  for (unsigned k = 0; k < n_irreps; k++)
    if (!active[k].empty()) sys.highest_occ_orb_in_irrep[k] = static_cast<int>(active[k].back());
}

double orc_get_s2(void* h) { return S(h).sys.get_s2(S(h).sys.coefs); }

// "var_sd" for whole variational runs (solver.h:424, 446)
void orc_set_var_sd(void* h, int on) { S(h).var_sd = on != 0; }

void orc_set_second_rejection(void* h, int on) {
  auto& s = S(h);
  s.second_rejection = on != 0;
  s.sys.energy_hf_1b = 0.0;
  if (s.second_rejection) {
    for (unsigned p : occ(s.sys.dets[0].up)) s.sys.energy_hf_1b += s.sys.I.get_1b(p, p);
    if (s.sys.time_sym) s.sys.energy_hf_1b *= 2.;
    else
      for (unsigned p : occ(s.sys.dets[0].dn)) s.sys.energy_hf_1b += s.sys.I.get_1b(p, p);
  }
}

// One run_variation call (solver.h:413-539); returns the energy.
double orc_run_variation_step(void* h, double eps_var, int until_converged, double target_error) {
  auto& s = S(h);
  s.target_error = target_error;
  if (s.var_dets.size() != s.sys.dets.size()) {
    s.var_dets.clear();
    for (const auto& d : s.sys.dets) s.var_dets.insert(d);
  }
  s.run_variation(eps_var, until_converged != 0);
  return s.sys.energy_var;
}

// Timing sample of the Hamiltonian build and H*v on the current dets, for a CPU baseline:
// the full index (update_abdet / abm1 / absingles, hamiltonian.h:157-413) is built, then only
// rows i = offset (mod stride) are computed (update_matrix, :415-598) and multiplied
// (sparse_matrix.cc:28-56).  out[0..4] = {index seconds, row seconds, spmv seconds for the
// sampled rows, sampled upper-triangle nnz (incl. diagonal), sampled rows}.
// Rows of the last orc_hbuild_sample: row ids (count returned), then per row its element count
// and, when cols is non-null, the elements (strict upper part, columns ascending).
size_t orc_sample_rows(void* h, uint64_t* rows, uint64_t* offsets, uint32_t* cols, double* vals) {
  auto* hh = static_cast<OrcHandle*>(h);
  const size_t m = hh->sample_rows.size();
  if (rows)
    for (size_t k = 0; k < m; k++) rows[k] = hh->sample_rows[k];
  if (offsets) {
    offsets[0] = 0;
    for (size_t k = 0; k < m; k++) offsets[k + 1] = offsets[k] + hh->sample_elems[k].size();
  }
  if (cols) {
    size_t p = 0;
    for (size_t k = 0; k < m; k++)
      for (const auto& e : hh->sample_elems[k]) {
        cols[p] = e.first;
        vals[p] = e.second;
        p++;
      }
  }
  return m;
}

void orc_hbuild_sample(void* h, size_t stride, size_t offset, double* out) {
  auto& s = S(h);
  auto& H = s.ham;
  H.clear();
  const auto t0 = omp_get_wtime();
  H.n_dets_prev = 0;
  H.n_dets = s.sys.dets.size();
  H.sort_by_det_id = false;
  H.update_abdet(s.sys);
  H.update_abm1(s.sys);
  H.update_absingles(s.sys);
  H.abm1.clear();
  const auto t1 = omp_get_wtime();
  // rows of the sample, computed exactly as update_matrix computes a new row
  const size_t n = H.n_dets;
  std::vector<size_t> rows;
  for (size_t i = offset; i < n; i += stride) rows.push_back(i);
  SparseMatrix m;
  m.set_dim(n);
  const auto& dets = s.sys.dets;
  const auto& sys = s.sys;
#pragma omp parallel for schedule(dynamic, 4)
  for (size_t r = 0; r < rows.size(); r++) {
    const size_t det_id = rows[r];
    const Det& det = dets[det_id];
    auto& row = m.rows[det_id];
    row.emplace_back(static_cast<uint32_t>(det_id), sys.hamiltonian_elem(det, det, 0));
    const size_t start_id = det_id + 1;
    const size_t bid = H.beta_to_id.at(det.dn);
    for (size_t j : H.b2d[bid]) {
      if (j < start_id) continue;
      const double v = sys.hamiltonian_elem(det, dets[j], -1);
      if (std::abs(v) >= EPS) row.emplace_back(static_cast<uint32_t>(j), v);
    }
    const size_t aid = H.alpha_to_id.at(det.up);
    for (size_t j : H.a2d[aid]) {
      if (j < start_id) continue;
      const double v = sys.hamiltonian_elem(det, dets[j], -1);
      if (std::abs(v) >= EPS) row.emplace_back(static_cast<uint32_t>(j), v);
    }
    const auto& bs_list = H.beta_singles[bid];
    for (size_t as : H.alpha_singles[aid]) {
      const auto& rel_b = H.a2b[as];
      const auto& rel_d = H.a2d[as];
      size_t ptr = 0;
      for (size_t bsd : bs_list) {
        while (ptr < rel_b.size() && rel_b[ptr] < bsd) ptr++;
        if (ptr == rel_b.size()) break;
        if (rel_b[ptr] == bsd) {
          const size_t j = rel_d[ptr++];
          if (j < start_id) continue;
          const double v = sys.hamiltonian_elem(det, dets[j], 2);
          if (std::abs(v) >= EPS) row.emplace_back(static_cast<uint32_t>(j), v);
        }
      }
    }
  }
  const auto t2 = omp_get_wtime();
  size_t nnz = 0;
  for (size_t i : rows) nnz += m.rows[i].size();
  std::vector<double> x(n, 1.0 / std::sqrt((double)n));
  const int nt = omp_get_max_threads();
  std::vector<std::vector<double>> part(nt, std::vector<double>(n, 0.0));
  const auto t3 = omp_get_wtime();
#pragma omp parallel
  {
    auto& y = part[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 64)
    for (size_t r = 0; r < rows.size(); r++) {
      const size_t i = rows[r];
      double acc = 0.0;
      for (const auto& e : m.rows[i]) {
        acc += e.second * x[e.first];
        if (i != e.first) y[e.first] += e.second * x[i];
      }
      y[i] += acc;
    }
  }
  const auto t4 = omp_get_wtime();
  H.clear();
  // keep the sample's rows (diagonal dropped, columns ascending) for orc_sample_rows
  auto* hh = static_cast<OrcHandle*>(h);
  hh->sample_rows = rows;
  hh->sample_elems.assign(rows.size(), {});
  for (size_t r = 0; r < rows.size(); r++) {
    auto& e = hh->sample_elems[r];
    for (const auto& x : m.rows[rows[r]])
      if (x.first != rows[r]) e.emplace_back(x.first, x.second);
    std::sort(e.begin(), e.end());
  }
  out[0] = t1 - t0;
  out[1] = t2 - t1;
  out[2] = t4 - t3;
  out[3] = static_cast<double>(nnz);
  out[4] = static_cast<double>(rows.size());
}

int orc_threads() { return omp_get_max_threads(); }

size_t orc_n_iterations(void* h) { return S(h).iter_ndets.size(); }
void orc_iterations(void* h, uint64_t* ndets, uint64_t* nnz, double* energy) {
  auto& s = S(h);
  for (size_t i = 0; i < s.iter_ndets.size(); i++) {
    ndets[i] = s.iter_ndets[i];
    nnz[i] = s.iter_nnz[i];
    energy[i] = s.iter_energy[i];
  }
}

double orc_energy_var(void* h) { return S(h).sys.energy_var; }
void orc_set_energy_var(void* h, double e) { S(h).sys.energy_var = e; }

void orc_pt_dtm(void* h, double eps_pt_dtm, size_t n_batches, double* value, double* uncert,
                size_t* n_pt_dets) {
  auto r = S(h).pt_dtm(eps_pt_dtm, n_batches);
  *value = r.value;
  *uncert = r.uncert;
  *n_pt_dets = r.n_pt_dets;
}

void orc_pt_psto(void* h, double eps_dtm, double eps_psto, size_t n_batches, double target_error,
                 double eps_pt, double* out /* value, uncert, n_pt_dets, batches */) {
  size_t done = 0;
  auto r = S(h).pt_psto(eps_dtm, eps_psto, n_batches, target_error, eps_pt, &done);
  out[0] = r.value;
  out[1] = r.uncert;
  out[2] = static_cast<double>(r.n_pt_dets);
  out[3] = static_cast<double>(done);
}

size_t orc_pt_sto(void* h, double eps_psto, double eps_pt, size_t n_batches, size_t n_samples,
                  unsigned seed, size_t max_iter, double target_error, double psto_uncert,
                  int semisto, double pt_mem_avail, double mem_usage,
                  double* out /* value, uncert, n_samples, n_dtm, n_unique_target */,
                  double* loops, size_t cap) {
  std::vector<double> lv;
  Solver::StoInfo info;
  Solver::PtResult r;
  try {
    r = S(h).pt_sto(eps_psto, eps_pt, n_batches, n_samples, seed, max_iter, target_error,
                    psto_uncert, &lv, semisto != 0, pt_mem_avail, mem_usage, &info);
  } catch (const std::exception&) {
    out[0] = out[1] = std::nan("");
    return static_cast<size_t>(-1);
  }
  out[0] = r.value;
  out[1] = r.uncert;
  out[2] = static_cast<double>(info.n_samples);
  out[3] = static_cast<double>(info.n_dtm);
  out[4] = static_cast<double>(info.n_unique_target);
  for (size_t k = 0; k < lv.size() && k < cap; k++) loops[k] = lv[k];
  return lv.size();
}

void orc_rdm1(void* h, double* out) {
  std::vector<double> r;
  rdm1(S(h).sys, r);
  std::copy(r.begin(), r.end(), out);
}

// Spatial 2-RDM over the current Hamiltonian connections (rdm.cc:333-371).  out is the
// half-stored array of n^2 (n^2+1)/2 doubles indexed like rdm.cc:233-241.
void orc_rdm2(void* h, double* out) {
  auto& s = S(h);
  const unsigned n = s.sys.n_orbs;
  Rdm2 R;
  R.n = n;
  R.half.assign((size_t)n * n * ((size_t)n * n + 1) / 2, 0.0);
  R.coefs = &s.sys.coefs;
  const auto& m = s.ham.matrix;
  for (size_t i = 0; i < m.rows.size(); i++)
    for (const auto& e : m.rows[i])
      R.elements(s.sys.dets[e.first], e.first, s.sys.dets[i], i, 1.0, s.sys.n_up, s.sys.n_dn);
  std::copy(R.half.begin(), R.half.end(), out);
}

// Generalized Fock matrix (src/chem/optimization.cc:620-650) from given RDMs: g1[n*n] (one_rdm
// (p, q) at p*n+q) and half (two_rdm in the half storage of rdm.cc:233-241).
void orc_generalized_fock(void* h, const double* g1, const double* half, double* F) {
  const auto& sys = S(h).sys;
  const unsigned n = sys.n_orbs;
  auto two = [&](unsigned p, unsigned q, unsigned r, unsigned s) {
    const size_t a = (size_t)p * n + s, b = (size_t)q * n + r;
    return a > b ? half[a * (a + 1) / 2 + b] : half[b * (b + 1) / 2 + a];
  };
#pragma omp parallel for collapse(2) schedule(dynamic)
  for (unsigned i = 0; i < n; i++)
    for (unsigned j = 0; j < n; j++) {
      if (sys.I.orb_sym[i] != sys.I.orb_sym[j]) {
        F[i * n + j] = 0.;
        continue;
      }
      double elem = 0.;  // generalized_Fock_element (:635-650)
      for (unsigned q = 0; q < n; q++) elem += g1[i * n + q] * sys.I.get_1b(j, q);
      for (unsigned q = 0; q < n; q++)
        for (unsigned r = 0; r < n; r++)
          for (unsigned s = 0; s < n; s++) elem += two(i, r, s, q) * sys.I.get_2b(j, q, r, s);
      F[i * n + j] = elem;
    }
}

// Optimization::parameter_indices (optimization.cc:500-522) without an active space: pairs
// i < j of equal irrep.  Returns the count; writes up to cap pairs.
size_t orc_orbital_parameters(void* h, unsigned* p, unsigned* q, size_t cap) {
  const auto& sys = S(h).sys;
  size_t k = 0;
  for (unsigned i = 0; i < sys.n_orbs; i++)
    for (unsigned j = i + 1; j < sys.n_orbs; j++)
      if (sys.I.orb_sym[i] == sys.I.orb_sym[j]) {
        if (k < cap) {
          p[k] = i;
          q[k] = j;
        }
        k++;
      }
  return k;
}

}  // extern "C"

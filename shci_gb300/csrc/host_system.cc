// Host-side chemistry system: FCIDUMP -> reordered dense integrals -> heat-bath queues.
//
// Follows the reference's Integrals::load / read_fcidump / generate_det_hf / reorder_orbs
// (src/chem/integrals.cc:17-384) and ChemSystem::setup_singles_queue / setup_hci_queue
// (src/chem/chem_system.cc:74-196, 237-287).
#include "host_system.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <atomic>
#include <thread>

#include <sched.h>

namespace shci {

namespace {
thread_local unsigned t_host_threads = 0;
}  // namespace

unsigned host_threads() {
  if (t_host_threads) return t_host_threads;
  static const unsigned usable = []() {
    // the CPUs this process may run on (a container's CPU set), else the machine's count
    cpu_set_t set;
    CPU_ZERO(&set);
    if (sched_getaffinity(0, sizeof(set), &set) == 0 && CPU_COUNT(&set) > 0)
      return static_cast<unsigned>(CPU_COUNT(&set));
    return std::max(1u, std::thread::hardware_concurrency());
  }();
  return usable;
}

void set_host_threads(unsigned n) { t_host_threads = n; }

namespace {

constexpr double kReorderEps = 1.0e-12;  // src/util.h:50 (comparison slack in reorder_orbs)

// Header tokens as matched by the reference's regex "([\-]?[^\s,=\-]+)"
// (integrals.cc:44): separators are whitespace, ',' and '='; '-' may only start a token.
std::vector<std::string> header_tokens(const std::string& line) {
  std::vector<std::string> out;
  std::string cur;
  auto flush = [&]() {
    if (!cur.empty() && !(cur.size() == 1 && cur[0] == '-')) out.push_back(cur);
    cur.clear();
  };
  for (char c : line) {
    if (std::isspace(static_cast<unsigned char>(c)) || c == ',' || c == '=') {
      flush();
    } else if (c == '-') {
      flush();
      cur.push_back('-');
    } else {
      cur.push_back(c);
    }
  }
  flush();
  return out;
}

struct RawIntegral {
  double v;
  unsigned p, q, r, s;
};

size_t pack4(size_t a, size_t b, size_t c, size_t d) {
  return combine2(combine2(a, b), combine2(c, d));
}

// Packed 8-fold tables keyed like Integrals::combine2/combine4 (integrals.cc:410-422); on a
// repeated key the value with the larger |v| is kept (integrals.cc:104-111).
struct Packed {
  std::vector<double> h1, g2;
  void init(unsigned n) {
    const size_t n2 = combine2(n - 1, n - 1) + 1;
    h1.assign(n2, 0.0);
    g2.assign(combine2(n2 - 1, n2 - 1) + 1, 0.0);
  }
  static void put(std::vector<double>& t, size_t k, double v) {
    if (t[k] == 0.0 || std::fabs(t[k]) < std::fabs(v)) t[k] = v;
  }
  void fill(const std::vector<RawIntegral>& raw, const std::vector<unsigned>& inv, double& ecore) {
    for (const auto& it : raw) {
      if (it.p == 0 && it.q == 0 && it.r == 0 && it.s == 0) {
        ecore = it.v;
      } else if (it.r == 0 && it.s == 0) {
        put(h1, combine2(inv[it.p - 1], inv[it.q - 1]), it.v);
      } else {
        put(g2, pack4(inv[it.p - 1], inv[it.q - 1], inv[it.r - 1], inv[it.s - 1]), it.v);
      }
    }
  }
  double h(unsigned p, unsigned q) const { return h1[combine2(p, q)]; }
  double g(unsigned p, unsigned q, unsigned r, unsigned s) const { return g2[pack4(p, q, r, s)]; }
};

// Irrep labels with negative entries are converted as integrals.cc:116-153 does.
std::vector<unsigned> convert_syms(const std::vector<int>& raw) {
  std::vector<unsigned> res(raw.size());
  bool neg = false;
  for (int s : raw) neg |= s < 0;
  for (size_t i = 0; i < raw.size(); i++) {
    const int s = raw[i];
    if (!neg || s == 1 || s == 2) {
      res[i] = static_cast<unsigned>(s);
      continue;
    }
    const unsigned a = std::abs(s) >> 1, b = (std::abs(s) + 1) >> 1;
    res[i] = a + 3 * b - 8 + (s < 0 ? 2 : 0);
  }
  return res;
}

}  // namespace

unsigned point_group_order(const std::string& pg, bool* linear) {
  std::string s;
  for (char c : pg) s.push_back(static_cast<char>(std::tolower(static_cast<unsigned char>(c))));
  if (linear) *linear = false;
  if (s == "c1") return 1;
  if (s == "c2" || s == "cs" || s == "ci") return 2;
  if (s == "c2v" || s == "c2h" || s == "d2") return 4;
  if (s == "d2h") return 8;
  if (s == "dooh" || s == "dih" || s == "coov" || s == "civ") {
    if (linear) *linear = true;
    return 128;
  }
  throw std::runtime_error("unsupported point group '" + pg +
                           "' (C1, C2, Cs, Ci, C2v, C2h, D2, D2h, Dooh/Dih, Coov/Civ)");
}

// Labels 1, 2 are Lz = 0 (g, u); from 3 on, four labels per |Lz|: +g, +u, -g, -u.
int linear_lz(int label, int* gu) {
  if (label <= 2) {
    *gu = label - 1;
    return 0;
  }
  const int mag = 1 + ((label - 3) >> 2);
  *gu = (label + 1) & 1;
  return (((label - 1) >> 1) & 1) ? mag : -mag;
}

namespace {

int linear_label(int lz, int gu) {
  if (lz == 0) return gu + 1;
  return (std::abs(lz) << 2) - 1 + gu + (lz < 0 ? 2 : 0);
}

// The irrep of the conjugate (Lz -> -Lz), DoohUtil::get_inverse (dooh_util.cc:35-45).
unsigned linear_inverse(unsigned label) {
  int gu;
  const int lz = linear_lz(static_cast<int>(label), &gu);
  return lz > 0 ? label + 2 : lz < 0 ? label - 2 : label;
}

}  // namespace

unsigned irrep_product(bool linear, unsigned a, unsigned b) {
  if (!linear) return ((a - 1) ^ (b - 1)) + 1;  // C1..D2h: XOR group on (irrep - 1)
  int ga, gb;
  const int la = linear_lz(static_cast<int>(a), &ga), lb = linear_lz(static_cast<int>(b), &gb);
  return static_cast<unsigned>(linear_label(la + lb, (ga + gb) & 1));
}

void screen_linear(HostIntegrals& I) {
  if (!I.linear) return;
  const unsigned n = I.n;
  std::vector<int> lz(n);
  for (unsigned o = 0; o < n; o++) {
    int gu;
    lz[o] = linear_lz(static_cast<int>(I.orb_sym[o]), &gu);
  }
  for (unsigned p = 0; p < n; p++)
    for (unsigned q = 0; q < n; q++)
      for (unsigned r = 0; r < n; r++)
        for (unsigned s = 0; s < n; s++)
          if (lz[p] + lz[r] != lz[q] + lz[s]) I.g2[((size_t)(p * n + q) * n + r) * n + s] = 0.0;
}

void load_fcidump(HostIntegrals& I, const std::string& path, unsigned n_up, unsigned n_dn,
                  const std::string& point_group, int reorder, const unsigned* occs_up,
                  const unsigned* occs_dn, const HfOptions& hf) {
  std::ifstream f(path);
  if (!f.good()) throw std::runtime_error("cannot open FCIDUMP '" + path + "'");
  I.n_syms = point_group_order(point_group, &I.linear);
  unsigned n = 0;
  std::vector<int> raw_syms;
  {
    enum { NONE, ORBSYM, END } state = NONE;
    std::string line;
    while (!f.eof()) {
      std::getline(f, line);
      const auto toks = header_tokens(line);
      for (size_t t = 0; t < toks.size(); t++) {
        const std::string& m = toks[t];
        if (m == "NORB" || m == "NORBS") {
          if (++t >= toks.size()) throw std::runtime_error("FCIDUMP: NORB without value");
          n = static_cast<unsigned>(std::stoul(toks[t]));
        } else if (m == "NELEC") {
          ++t;
        } else if (m == "ORBSYM") {
          state = ORBSYM;
        } else if (state == ORBSYM) {
          raw_syms.push_back(std::stoi(m));
          if (raw_syms.size() == n) state = NONE;
        } else if (m == "&END" || m == "/") {
          state = END;
        }
      }
      if (state == END) break;
    }
  }
  if (n == 0) throw std::runtime_error("FCIDUMP: NORB missing");
  if (n > 64) throw std::runtime_error("n_orbs > 64 is not supported");
  if (raw_syms.size() != n) raw_syms.assign(n, 1);
  std::vector<RawIntegral> raw;
  {
    // Whitespace-separated records "value p q r s" until end of file.  A final record not
    // followed by whitespace is dropped, as the stream loop of integrals.cc:86-91 does.
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string body = ss.str();
    const char* c = body.c_str();
    const char* end = c + body.size();
    while (true) {
      char* e = nullptr;
      while (c < end && std::isspace(static_cast<unsigned char>(*c))) c++;
      if (c >= end) break;
      const double v = std::strtod(c, &e);
      if (e == c) throw std::runtime_error("FCIDUMP: bad integral line");
      c = e;
      unsigned idx[4];
      bool ok = true;
      for (int k = 0; k < 4; k++) {
        while (c < end && std::isspace(static_cast<unsigned char>(*c))) c++;
        if (c >= end) {
          ok = false;
          break;
        }
        idx[k] = static_cast<unsigned>(std::strtoul(c, &e, 10));
        if (e == c) throw std::runtime_error("FCIDUMP: bad index");
        c = e;
      }
      if (!ok || c >= end) break;  // truncated record, or last record at end of file
      if (std::fabs(v) < 1.0e-9) continue;
      for (int k = 0; k < 4; k++)
        if (idx[k] > n) throw std::runtime_error("FCIDUMP: orbital index out of range");
      raw.push_back(RawIntegral{v, idx[0], idx[1], idx[2], idx[3]});
    }
  }
  I.n = n;
  I.n_up = n_up;
  I.n_dn = n_dn;
  if (n_up > n || n_dn > n) throw std::runtime_error("more electrons than orbitals");

  Packed P;
  P.init(n);
  std::vector<unsigned> ident(n);
  std::iota(ident.begin(), ident.end(), 0u);
  double ecore = 0.0;
  P.fill(raw, ident, ecore);

  // HF det (integrals.cc:155-226): explicit occupations, the listed irreps' occupations, or
  // the lowest orbitals.
  const auto syms = convert_syms(raw_syms);
  uint64_t hf_up = 0, hf_dn = 0;
  bool explicit_orbs = false;
  if (occs_up && occs_dn) {
    for (unsigned i = 0; i < n_up; i++) hf_up |= 1ull << occs_up[i];
    for (unsigned i = 0; i < n_dn; i++) hf_dn |= 1ull << occs_dn[i];
    explicit_orbs = true;
  } else if (!hf.irreps.empty()) {
    if (hf.irrep_occs_up.size() != hf.irreps.size() || hf.irrep_occs_dn.size() != hf.irreps.size())
      throw std::runtime_error("chem/irrep_occs_up and chem/irrep_occs_dn need one entry per irrep");
    for (size_t k = 0; k < hf.irreps.size(); k++) {
      unsigned occ_up = hf.irrep_occs_up[k], occ_dn = hf.irrep_occs_dn[k];
      for (unsigned j = 0; j < n; j++) {
        if (syms[j] != hf.irreps[k]) continue;
        if (occ_up > 0) {
          hf_up |= 1ull << j;
          occ_up--;
        } else {
          hf_up &= ~(1ull << j);
        }
        if (occ_dn > 0) {
          hf_dn |= 1ull << j;
          occ_dn--;
        } else {
          hf_dn &= ~(1ull << j);
        }
        if (occ_up == 0 && occ_dn == 0 && j >= n_up && j >= n_dn) break;
      }
      if (occ_up > 0 || occ_dn > 0)
        throw std::runtime_error("unable to construct hf with given irrep");
    }
    if (__builtin_popcountll(hf_up) != (int)n_up || __builtin_popcountll(hf_dn) != (int)n_dn)
      throw std::runtime_error("chem/irrep_occs_up / irrep_occs_dn do not add up to n_up / n_dn");
    explicit_orbs = true;
  } else {
    for (unsigned i = 0; i < n_up; i++) hf_up |= 1ull << i;
    if (hf.allow_doubly_occupy) {
      for (unsigned i = 0; i < n_dn; i++) hf_dn |= 1ull << i;
    } else {
      if (n_up + n_dn > n)
        throw std::runtime_error("allow_doubly_occupy_hf false needs n_up + n_dn <= n_orbs");
      for (unsigned i = 0; i < n_dn; i++) hf_dn |= 1ull << (i + n_up);
    }
  }
  // Orbital energies (integrals.cc:228-255) from the un-reordered tables.
  std::vector<double> e(n);
  for (unsigned i = 0; i < n; i++) {
    e[i] = P.h(i, i);
    double direct = 0.0, exch = 0.0;
    for (int spin = 0; spin < 2; spin++) {
      for (uint64_t m = spin ? hf_dn : hf_up; m; m &= m - 1) {
        const unsigned o = __builtin_ctzll(m);
        if (o == i) {
          direct += P.g(i, i, o, o);
        } else {
          direct += 2 * P.g(i, i, o, o);
          exch -= P.g(i, o, o, i);
        }
      }
    }
    e[i] += 0.5 * (direct + exch);
  }
  // reorder_orbs (integrals.cc:257-384)
  std::vector<unsigned> order(n), inv(n);
  std::iota(order.begin(), order.end(), 0u);
  const bool do_reorder = reorder < 0 ? !explicit_orbs : reorder != 0;
  if (do_reorder)
    std::stable_sort(order.begin(), order.end(),
                     [&](unsigned a, unsigned b) { return e[a] < e[b] - kReorderEps; });
  for (unsigned i = 0; i < n; i++) inv[order[i]] = i;
  I.orb_sym.resize(n);
  I.orb_order = order;
  for (unsigned i = 0; i < n; i++) I.orb_sym[i] = syms[order[i]];
  I.hf_up = I.hf_dn = 0;
  for (unsigned i = 0; i < n; i++) {
    if (hf_up >> order[i] & 1) I.hf_up |= 1ull << i;
    if (hf_dn >> order[i] & 1) I.hf_dn |= 1ull << i;
  }
  Packed R;
  R.init(n);
  ecore = 0.0;
  R.fill(raw, inv, ecore);
  I.e_core = ecore;
  I.h1.assign((size_t)n * n, 0.0);
  I.g2.assign((size_t)n * n * n * n, 0.0);
  for (unsigned p = 0; p < n; p++)
    for (unsigned q = 0; q < n; q++) {
      I.h1[p * n + q] = R.h(p, q);
      for (unsigned r = 0; r < n; r++)
        for (unsigned s = 0; s < n; s++)
          I.g2[((size_t)(p * n + q) * n + r) * n + s] = R.g(p, q, r, s);
    }
  // The orbital energies above read the tables unscreened: the reference sets the integrals'
  // point group only after Integrals::load (chem_system.cc:33-34), and (ii|oo), (io|oi)
  // conserve Lz anyway.
  screen_linear(I);
}

namespace {
static_assert(sizeof(unsigned) == 4, "cache layout stores u32 fields");
constexpr char kCacheMagic[8] = {'S', 'H', 'C', 'I', 'G', 'I', 'C', '1'};

CacheStatus probe_cache(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return kCacheMissing;
  char m[8];
  const bool ours = std::fread(m, 1, 8, f) == 8 && std::memcmp(m, kCacheMagic, 8) == 0;
  std::fclose(f);
  return ours ? kCacheOk : kCacheForeign;
}
}  // namespace

CacheStatus load_integrals_cache(HostIntegrals& I, const std::string& path,
                                 const std::string& point_group) {
  const CacheStatus st = probe_cache(path);
  if (st != kCacheOk) return st;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return kCacheMissing;
  bool ok = true;
  auto rd = [&](void* p, size_t n) { ok = ok && std::fread(p, 1, n, f) == n; };
  char m[8];
  uint32_t hdr[3] = {0, 0, 0};
  rd(m, 8);
  rd(hdr, sizeof(hdr));
  HostIntegrals J;
  const size_t n = hdr[0];
  ok = ok && n >= 1 && n <= 64 && hdr[1] <= n && hdr[2] <= n;
  if (ok) {
    J.n = hdr[0];
    J.n_up = hdr[1];
    J.n_dn = hdr[2];
    rd(&J.e_core, 8);
    J.orb_sym.resize(n);
    J.orb_order.resize(n);
    rd(J.orb_sym.data(), 4 * n);
    rd(J.orb_order.data(), 4 * n);
    rd(&J.hf_up, 8);
    rd(&J.hf_dn, 8);
    J.h1.resize(n * n);
    J.g2.resize(n * n * n * n);
    rd(J.h1.data(), 8 * n * n);
    rd(J.g2.data(), 8 * n * n * n * n);
    char extra;
    ok = ok && std::fread(&extra, 1, 1, f) == 0;  // nothing after g2
  }
  std::fclose(f);
  if (ok) {
    std::vector<bool> seen(n, false);
    for (unsigned o : J.orb_order) {
      ok = ok && o < n && !seen[o];
      if (o < n) seen[o] = true;
    }
    ok = ok && __builtin_popcountll(J.hf_up) == (int)J.n_up &&
         __builtin_popcountll(J.hf_dn) == (int)J.n_dn &&
         (n == 64 || ((J.hf_up | J.hf_dn) >> n) == 0);
  }
  if (!ok) throw std::runtime_error(path + ": truncated or inconsistent integrals cache");
  J.n_syms = point_group_order(point_group, &J.linear);
  I = std::move(J);
  return kCacheOk;
}

CacheStatus save_integrals_cache(const HostIntegrals& I, const std::string& path) {
  if (probe_cache(path) == kCacheForeign) return kCacheForeign;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  const size_t n = I.n;
  bool ok = true;
  auto wr = [&](const void* p, size_t k) { ok = ok && std::fwrite(p, 1, k, f) == k; };
  const uint32_t hdr[3] = {I.n, I.n_up, I.n_dn};
  wr(kCacheMagic, 8);
  wr(hdr, sizeof(hdr));
  wr(&I.e_core, 8);
  wr(I.orb_sym.data(), 4 * n);
  wr(I.orb_order.data(), 4 * n);
  wr(&I.hf_up, 8);
  wr(&I.hf_dn, 8);
  wr(I.h1.data(), 8 * n * n);
  wr(I.g2.data(), 8 * n * n * n * n);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) throw std::runtime_error("cannot write " + path);
  return kCacheOk;
}

uint64_t inactive_orbitals(const HostIntegrals& I, const std::vector<unsigned>& irrep_active_space) {
  unsigned n_irreps = 0;
  for (unsigned s : I.orb_sym) {
    if (s == 0) throw std::invalid_argument("orbital symmetry labels start at 1");
    n_irreps = std::max(n_irreps, s);
  }
  if (irrep_active_space.size() < n_irreps)
    throw std::invalid_argument("chem/irrep_active_space needs an entry for each of the " +
                                std::to_string(n_irreps) + " irreps");
  std::vector<int> highest(n_irreps, -1);
  std::vector<unsigned> taken(n_irreps, 0);
  for (unsigned i = 0; i < I.n; i++) {
    const unsigned k = I.orb_sym[i] - 1;
    if (taken[k] < irrep_active_space[k]) {
      taken[k]++;
      highest[k] = static_cast<int>(i);
    }
  }
  uint64_t mask = 0;
  for (unsigned r = 0; r < I.n; r++)
    if (static_cast<int>(r) > highest[I.orb_sym[r] - 1]) mask |= 1ull << r;
  return mask;
}

double host_diag(const HostIntegrals& I, uint64_t up, uint64_t dn) {
  double ob = 0.0;
  for (uint64_t m = up; m; m &= m - 1) ob += I.h(__builtin_ctzll(m), __builtin_ctzll(m));
  if (up == dn) {
    ob *= 2;
  } else {
    for (uint64_t m = dn; m; m &= m - 1) ob += I.h(__builtin_ctzll(m), __builtin_ctzll(m));
  }
  double direct = 0.0, exch = 0.0;
  auto same = [&](uint64_t s) {
    for (uint64_t m = s; m; m &= m - 1) {
      const unsigned a = __builtin_ctzll(m);
      for (uint64_t m2 = m & (m - 1); m2; m2 &= m2 - 1) {
        const unsigned b = __builtin_ctzll(m2);
        direct += I.g(a, a, b, b);
        exch -= I.g(a, b, b, a);
      }
    }
  };
  same(up);
  if (up == dn) {
    direct *= 2;
    exch *= 2;
  } else {
    same(dn);
  }
  for (uint64_t m = up; m; m &= m - 1)
    for (uint64_t m2 = dn; m2; m2 &= m2 - 1) {
      const unsigned a = __builtin_ctzll(m), b = __builtin_ctzll(m2);
      direct += I.g(a, a, b, b);
    }
  return ob + (direct + exch) + I.e_core;
}

namespace {

// |two-body double| of the queue element (p,q) -> (r,s) (chem_system.cc:261-287, 579-609).
double queue_elem(const HostIntegrals& I, unsigned p, unsigned q, unsigned r, unsigned s) {
  if (p == q || r == s || p == r || q == s || p == s || q == r) return 0.0;
  const unsigned n = I.n;
  if (q < n) return std::fabs(I.g(p, r, q, s) - I.g(p, s, q, r));
  return std::fabs(I.g(p, r, q - n, s - n));
}

// Upper bound on |H| of the single excitation i -> j (chem_system.cc:237-259).
double singles_elem(const HostIntegrals& I, unsigned i, unsigned j) {
  if (i == j) return 0.0;
  const unsigned n = I.n, n_elecs = I.n_up + I.n_dn;
  std::vector<double> el;
  el.reserve(2 * n - 2);
  for (unsigned o = 0; o < n; o++) {
    const double ex = I.g(i, o, o, j), direct = I.g(i, j, o, o);
    el.push_back(direct);
    if (o != i && o != j) el.push_back(direct - ex);
  }
  std::sort(el.begin(), el.end());
  double smin = I.h(i, j), smax = smin;
  const unsigned lim = std::min(n_elecs - 1, 2 * n - 2);
  for (unsigned k = 0; k < lim; k++) {
    smin += el[k];
    smax += el[2 * n - 3 - k];
  }
  return std::max(std::fabs(smin), std::fabs(smax));
}

template <class F>
void parallel_for(unsigned n, F f) {
  unsigned nt = std::max(1u, std::min(n, host_threads()));
  if (nt == 1) {
    for (unsigned i = 0; i < n; i++) f(i);
    return;
  }
  std::vector<std::thread> th;
  std::atomic<unsigned> next{0};
  for (unsigned t = 0; t < nt; t++)
    th.emplace_back([&]() {
      for (unsigned i; (i = next.fetch_add(1)) < n;) f(i);
    });
  for (auto& t : th) t.join();
}

}  // namespace

void build_queues(const HostIntegrals& I, HostQueues& Q) {
  const unsigned n = I.n;
  std::vector<std::vector<unsigned>> sym_orbs(I.n_syms + 1);
  for (unsigned o = 0; o < n; o++) {
    if (I.orb_sym[o] >= sym_orbs.size()) sym_orbs.resize(I.orb_sym[o] + 1);
    sym_orbs[I.orb_sym[o]].push_back(o);
  }
  struct E {
    double H;
    uint32_t rs;
  };
  const size_t n_pairs = combine2(n, 2 * n);
  std::vector<std::vector<E>> dq(n_pairs);
  // irrep that s must have given p, q, r: the product of p, q and r's conjugate (linear groups
  // conjugate r, chem_system.cc:133-135; the other groups are their own conjugates)
  auto sym_r = [&](unsigned r) { return I.linear ? linear_inverse(I.orb_sym[r]) : I.orb_sym[r]; };
  auto sort_desc = [](std::vector<E>& v) {
    std::sort(v.begin(), v.end(), [](const E& a, const E& b) { return a.H > b.H; });
  };
  // same spin: p < q < n, s >= r (chem_system.cc:123-153)
  parallel_for(n, [&](unsigned p) {
    for (unsigned q = p + 1; q < n; q++) {
      auto& v = dq[combine2(p, q)];
      const unsigned sq = irrep_product(I.linear, I.orb_sym[p], I.orb_sym[q]);
      for (unsigned r = 0; r < n; r++) {
        const unsigned sr = irrep_product(I.linear, sq, sym_r(r));
        if (sr >= sym_orbs.size()) continue;
        for (unsigned s : sym_orbs[sr]) {
          if (s < r) continue;
          const double H = queue_elem(I, p, q, r, s);
          if (H != 0.0) v.push_back(E{H, r | (s << 16)});
        }
      }
      sort_desc(v);
    }
  });
  // opposite spin: q in [n + p, 2n) (chem_system.cc:155-183)
  parallel_for(n, [&](unsigned p) {
    for (unsigned q = n + p; q < 2 * n; q++) {
      auto& v = dq[combine2(p, q)];
      const unsigned sq = irrep_product(I.linear, I.orb_sym[p], I.orb_sym[q - n]);
      for (unsigned r = 0; r < n; r++) {
        const unsigned sr = irrep_product(I.linear, sq, sym_r(r));
        if (sr >= sym_orbs.size()) continue;
        for (unsigned s : sym_orbs[sr]) {
          const double H = queue_elem(I, p, q, r, s + n);
          if (H != 0.0) v.push_back(E{H, r | ((s + n) << 16)});
        }
      }
      sort_desc(v);
    }
  });
  Q.d_off.assign(n_pairs + 1, 0);
  Q.max_hci = 0.0;
  for (size_t k = 0; k < n_pairs; k++) {
    Q.d_off[k + 1] = Q.d_off[k] + dq[k].size();
    if (!dq[k].empty()) Q.max_hci = std::max(Q.max_hci, dq[k][0].H);
  }
  Q.d_H.resize(Q.d_off[n_pairs]);
  Q.d_rs.resize(Q.d_off[n_pairs]);
  for (size_t k = 0; k < n_pairs; k++)
    for (size_t e = 0; e < dq[k].size(); e++) {
      Q.d_H[Q.d_off[k] + e] = dq[k][e].H;
      Q.d_rs[Q.d_off[k] + e] = dq[k][e].rs;
    }
  // singles (chem_system.cc:74-113)
  std::vector<std::vector<std::pair<double, unsigned>>> sq(n);
  parallel_for(n, [&](unsigned p) {
    for (unsigned r : sym_orbs[I.orb_sym[p]]) {
      const double S = singles_elem(I, p, r);
      if (S != 0.0) sq[p].push_back({S, r});
    }
    std::sort(sq[p].begin(), sq[p].end(),
              [](const std::pair<double, unsigned>& a, const std::pair<double, unsigned>& b) {
                return a.first > b.first;
              });
  });
  Q.s_off.assign(n + 1, 0);
  Q.max_singles = 0.0;
  for (unsigned p = 0; p < n; p++) {
    Q.s_off[p + 1] = Q.s_off[p] + static_cast<uint32_t>(sq[p].size());
    if (!sq[p].empty()) Q.max_singles = std::max(Q.max_singles, sq[p][0].first);
  }
  Q.s_S.resize(Q.s_off[n]);
  Q.s_r.resize(Q.s_off[n]);
  for (unsigned p = 0; p < n; p++)
    for (size_t e = 0; e < sq[p].size(); e++) {
      Q.s_S[Q.s_off[p] + e] = sq[p][e].first;
      Q.s_r[Q.s_off[p] + e] = sq[p][e].second;
    }
}

}  // namespace shci

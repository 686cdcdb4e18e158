// shci_gpu: the drop-in command line driver.
//
// Run in a directory that holds config.json and FCIDUMP, like the reference's `shci`
// executable (src/main.cc:24-37, src/injector.cc:10-24).  It follows Solver<S>::run
// (src/solver/solver.h:100-160): setup, the variational stages with their eps_vars_schedule
// (:338-539), optional RDM output (src/chem/chem_system.cc:611-623, src/chem/rdm.cc:202-331) and
// the three PT2 stages per eps_var (:541-1153), writing result.json with the reference's keys
// (energy_hf, n_elecs, config, energy_var/<eps>, energy_total/<eps_var>/<eps_pt>/{value,
// uncert}) and printing the reference's grep-able lines ("Final iteration ... energy=",
// "Total energy: ...").  All computation goes through the C ABI of include/shci_gpu.h.
// After each eps_var the wavefunction is saved to wf_eps1_<eps_var>.dat, and an eps_var whose
// file exists is loaded instead of computed (force_var recomputes); the PT2 stage takes its
// wavefunctions from those files under skip_var (solver.h:348-397, 571-575; format in
// wf_file.h).
//
// Also honoured as the reference does: n_states (several states, state-suffixed result keys),
// second_rejection / second_rejection_factor, the linear point groups.
// GPU-specific keys (ignored by the reference): gpu/device (default 0), gpu/precision
// ("mixed" default, or "fp64").
#include <shci_gpu.h>

#include <clocale>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include <unistd.h>

#include "json.h"
#include "wf_file.h"

using shci_cli::Json;

namespace {

Json g_config, g_result;

std::string fmt(const char* f, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, f);
  std::vsnprintf(buf, sizeof(buf), f, ap);
  va_end(ap);
  return buf;
}

[[noreturn]] void die(const std::string& m) {
  std::fprintf(stderr, "shci_gpu: %s\n", m.c_str());
  std::exit(1);
}

void ck(shci_ctx* c, shci_status s, const char* what) {
  if (s != SHCI_OK) die(std::string(what) + ": " + shci_last_error(c));
}

// Util::get_mem_total (src/util.cc:195): MemTotal of /proc/meminfo in kB times 1000 (the
// default of "mem_total"); the physical page count where /proc is unreadable.
double machine_memory() {
  std::ifstream f("/proc/meminfo");
  std::string key;
  double kb = 0.0;
  while (f >> key) {
    if (key == "MemTotal:") {
      f >> kb;
      return kb * 1000.0;
    }
    std::getline(f, key);
  }
  const long pages = sysconf(_SC_PHYS_PAGES), page = sysconf(_SC_PAGE_SIZE);
  return pages > 0 && page > 0 ? static_cast<double>(pages) * static_cast<double>(page) : 0.0;
}

// Config::get (src/config.h:21-50): slash-separated keys, defaults for optional ones.
double cfg_d(const std::string& k, double def, bool required = false) {
  const Json* j = g_config.get(k);
  if (!j) {
    if (required) die("Cannot find '" + k + "' in config.json");
    return def;
  }
  if (j->type != Json::Number) die("'" + k + "' must be a number");
  return j->num;
}
bool cfg_b(const std::string& k, bool def) {
  const Json* j = g_config.get(k);
  if (!j) return def;
  if (j->type != Json::Bool) die("'" + k + "' must be true or false");
  return j->b;
}
std::string cfg_s(const std::string& k, const std::string& def, bool required = false) {
  const Json* j = g_config.get(k);
  if (!j) {
    if (required) die("Cannot find '" + k + "' in config.json");
    return def;
  }
  if (j->type != Json::String) die("'" + k + "' must be a string");
  return j->str;
}
std::vector<double> cfg_v(const std::string& k, bool required) {
  const Json* j = g_config.get(k);
  std::vector<double> out;
  if (!j) {
    if (required) die("Cannot find '" + k + "' in config.json");
    return out;
  }
  if (j->type != Json::Array) die("'" + k + "' must be an array");
  for (const auto& e : j->arr) out.push_back(e.num);
  return out;
}

// Result::put (src/result.h:56-70): rewrites result.json after every put.
void result_dump() {
  std::ofstream f("result.json");
  f << shci_cli::dump(g_result) << std::endl;
}
void result_put(const std::string& k, double v) {
  g_result.put(k) = Json::number(v);
  result_dump();
}

void result_put_str(const std::string& k, const std::string& v) {
  g_result.put(k) = Json::string(v);
  result_dump();
}

std::string key_eps(double e) { return fmt("%#.2e", e); }

std::string wf_filename(double eps_var) { return fmt("wf_eps1_%#.2e.dat", eps_var); }

struct Wavefunction {
  double eps_var = 0.0, energy = 0.0;  // energy of state 0
  std::vector<uint64_t> up, dn;
  std::vector<double> coefs;                // state 0
  std::vector<std::vector<double>> xcoefs;  // states 1..
  std::vector<double> xenergy;              // states 1..
  size_t n_states() const { return 1 + xcoefs.size(); }
  double energy_of(size_t k) const { return k == 0 ? energy : xenergy[k - 1]; }
  const std::vector<double>& coefs_of(size_t k) const { return k == 0 ? coefs : xcoefs[k - 1]; }
};

// "" for state 0, "_<k>" otherwise (Solver::get_state_suffix, solver.h:1406-1412)
std::string state_suffix(size_t k) { return k == 0 ? "" : "_" + std::to_string(k); }

// unpack_time_sym (base_system.h:108-123): each det with up < dn gets its reverse appended,
// both coefficients (every state) times 1/sqrt(2) (Util::SQRT2_INV, src/util.h:60).
Wavefunction unpacked(const Wavefunction& wf) {
  constexpr double kSqrt2Inv = 0.7071067811865475;
  Wavefunction u = wf;
  const size_t n = wf.up.size();
  for (size_t i = 0; i < n; i++)
    if (wf.up[i] < wf.dn[i]) {
      auto half = [&](std::vector<double>& v) {
        const double h = v[i] * kSqrt2Inv;
        v[i] = h;
        v.push_back(h);
      };
      half(u.coefs);
      for (auto& xc : u.xcoefs) half(xc);
      u.up.push_back(wf.dn[i]);
      u.dn.push_back(wf.up[i]);
    }
  return u;
}

// The context's det list and every state's coefficients become wf's.
void put_wf(shci_ctx* c, const Wavefunction& wf) {
  ck(c, shci_set_dets(c, wf.up.data(), wf.dn.data(), wf.coefs.data(), wf.up.size()), "dets");
  for (size_t k = 1; k < wf.n_states(); k++)
    ck(c, shci_set_state_coefs(c, (unsigned)k, wf.xcoefs[k - 1].data(), wf.up.size()),
       "state coefficients");
}

// load_variation_result (solver.h:1179-1211) for this build's files; prints what the
// reference prints on success.  A file of another format is reported and left alone.
bool load_wf(const std::string& fn, unsigned n_up, unsigned n_dn, unsigned n_states,
             bool time_sym, double eps_var, Wavefunction* wf) {
  shci_cli::WfFile w;
  const auto st = shci_cli::wf_load(fn, &w);
  if (st == shci_cli::WfStatus::kForeign || st == shci_cli::WfStatus::kBad) {
    std::printf("%s is not a wavefunction file of this build; not loaded\n", fn.c_str());
    return false;
  }
  if (st != shci_cli::WfStatus::kOk) return false;
  if (w.n_up != n_up || w.n_dn != n_dn || w.n_states != n_states ||
      w.time_sym != (time_sym ? 1u : 0u)) {
    std::printf("%s holds %u/%u electrons, %u states, time_sym %u; not loaded\n", fn.c_str(),
                w.n_up, w.n_dn, w.n_states, w.time_sym);
    return false;
  }
  std::printf("Loaded %'zu dets from: %s\n", w.up.size(), fn.c_str());
  std::printf("HF energy: %.10f Ha\n", w.energy_hf);
  std::printf("Variational energy: ");
  for (double e : w.energy_var) std::printf("%.10f\t", e);
  std::printf("\n");
  const size_t n = w.up.size();
  wf->eps_var = eps_var;
  wf->energy = w.energy_var[0];
  wf->up = std::move(w.up);
  wf->dn = std::move(w.dn);
  wf->coefs.assign(w.coefs.begin(), w.coefs.begin() + n);
  wf->xcoefs.clear();
  wf->xenergy.clear();
  for (unsigned k = 1; k < w.n_states; k++) {
    wf->xcoefs.emplace_back(w.coefs.begin() + k * n, w.coefs.begin() + (k + 1) * n);
    wf->xenergy.push_back(w.energy_var[k]);
  }
  return true;
}

// save_variation_result (solver.h:1213-1221); a file of another format is not overwritten
void save_wf(const std::string& fn, unsigned n_up, unsigned n_dn, bool time_sym, double e_hf,
             const Wavefunction& wf) {
  if (shci_cli::wf_probe(fn) == shci_cli::WfStatus::kForeign) {
    std::printf("%s exists in another format; not overwritten\n", fn.c_str());
    return;
  }
  shci_cli::WfFile w;
  w.n_up = n_up;
  w.n_dn = n_dn;
  w.energy_hf = e_hf;
  w.time_sym = time_sym ? 1u : 0u;
  w.n_states = static_cast<unsigned>(wf.n_states());
  w.up = wf.up;
  w.dn = wf.dn;
  for (size_t k = 0; k < wf.n_states(); k++) {
    w.energy_var.push_back(wf.energy_of(k));
    w.coefs.insert(w.coefs.end(), wf.coefs_of(k).begin(), wf.coefs_of(k).end());
  }
  if (shci_cli::wf_save(fn, w)) std::printf("Variational results saved to: %s\n", fn.c_str());
  else std::printf("cannot write %s\n", fn.c_str());
}

}  // namespace

int main(int, char* argv[]) {
  std::setlocale(LC_ALL, "en_US.UTF-8");
  std::printf("Semistochastic Heat-bath Configuration Interation (SHCI) - GB300 build\n\n");
  std::printf("Executable: %s\n", argv[0]);
  {
    std::ifstream f("config.json");
    if (!f) die("cannot open config.json");
    std::stringstream ss;
    ss << f.rdbuf();
    g_config = shci_cli::Parser(ss.str()).parse();
  }
  {
    std::ifstream f("result.json");
    if (f) {
      std::stringstream ss;
      ss << f.rdbuf();
      try {
        g_result = shci_cli::Parser(ss.str()).parse();
      } catch (const std::exception&) {
        g_result = Json();
      }
    }
    if (g_result.type != Json::Object) {
      g_result = Json();
      g_result.type = Json::Object;
    }
    g_result.put("config") = g_config;
    result_dump();
  }
  std::printf("Configuration:\n%s\n", shci_cli::dump(g_config).c_str());
  const std::string system = cfg_s("system", "", true);
  if (system != "chem") die("system '" + system + "' is not supported.");
  const unsigned n_states = static_cast<unsigned>(cfg_d("n_states", 1));
  const bool time_sym = cfg_b("time_sym", false);
  const unsigned n_up = static_cast<unsigned>(cfg_d("n_up", 0, true));
  const unsigned n_dn = static_cast<unsigned>(cfg_d("n_dn", 0, true));
  const std::string pg = cfg_s("chem/point_group", "", true);
  const int device = static_cast<int>(cfg_d("gpu/device", 0));
  const std::string prec_s = cfg_s("gpu/precision", "mixed");
  const int prec = prec_s == "fp64" ? SHCI_PREC_FP64 : SHCI_PREC_MIXED;
  const double target_error = cfg_d("target_error", 5.0e-5);
  std::vector<double> occ_u = cfg_v("occs_up", false), occ_d = cfg_v("occs_dn", false);
  int reorder = -1;
  if (g_config.get("reorder_orbs")) reorder = cfg_b("reorder_orbs", true) ? 1 : 0;

  shci_ctx* c = nullptr;
  if (shci_create(&c, device, 0) != SHCI_OK) die("cannot create a context on the GPU");
  std::vector<unsigned> ou(occ_u.begin(), occ_u.end()), od(occ_d.begin(), occ_d.end());
  // HF det options (integrals.cc:155-215): "chem/irreps" with "chem/irrep_occs_up/dn", and
  // "allow_doubly_occupy_hf"
  const std::vector<double> irr = cfg_v("chem/irreps", false);
  std::vector<unsigned> irreps(irr.begin(), irr.end()), irr_up, irr_dn;
  if (!irreps.empty() && ou.empty() && od.empty()) {
    const std::vector<double> a = cfg_v("chem/irrep_occs_up", true);
    const std::vector<double> b = cfg_v("chem/irrep_occs_dn", true);
    irr_up.assign(a.begin(), a.end());
    irr_dn.assign(b.begin(), b.end());
    if (irr_up.size() != irreps.size() || irr_dn.size() != irreps.size())
      die("chem/irrep_occs_up and chem/irrep_occs_dn need one entry per entry of chem/irreps");
  } else {
    irreps.clear();
  }
  ck(c, shci_set_hf_options(c, cfg_b("allow_doubly_occupy_hf", true) ? 1 : 0,
                            irreps.empty() ? nullptr : irreps.data(),
                            irr_up.empty() ? nullptr : irr_up.data(),
                            irr_dn.empty() ? nullptr : irr_dn.data(), irreps.size()),
     "HF options");
  const bool explicit_orbs = !ou.empty() || !od.empty() || !irreps.empty();
  // Integrals::load (integrals.cc:17-35): the cache when asked for and present, else FCIDUMP,
  // after which the cache is written
  const char* cache = "integrals_cache.dat";
  int from_cache = 0;
  if (cfg_b("load_integrals_cache", false))
    ck(c, shci_load_integrals_cache(c, cache, n_up, n_dn, pg.c_str(), &from_cache),
       "integrals cache");
  if (from_cache) {
    std::printf("Loaded FCIDUMP cache from: %s\n", cache);
  } else {
    ck(c, shci_load_fcidump(c, "FCIDUMP", n_up, n_dn, pg.c_str(), reorder,
                            ou.empty() ? nullptr : ou.data(), od.empty() ? nullptr : od.data()),
       "load FCIDUMP");
    int written = 0;
    ck(c, shci_save_integrals_cache(c, cache, &written), "integrals cache");
    if (written)
      std::printf("FCIDUMP cache saved to: %s\n", cache);
    else
      std::printf("Note: %s is not in this build's format; it is neither read nor overwritten.\n",
                  cache);
  }
  double e_hf = 0.0;
  uint64_t hf_up = 0, hf_dn = 0;
  ck(c, shci_get_hf(c, &hf_up, &hf_dn, &e_hf), "HF det");
  int n_orbs = 0;
  ck(c, shci_get_integrals(c, &n_orbs, nullptr, nullptr, nullptr, nullptr, nullptr), "integrals");
  ck(c, shci_set_n_states(c, n_states), "n_states");
  if (time_sym) ck(c, shci_set_time_sym(c, 1), "time_sym");
  ck(c, shci_set_second_rejection(c, cfg_b("second_rejection", false) ? 1 : 0,
                                  cfg_d("second_rejection_factor", 0.2)),
     "second rejection");
  ck(c, shci_set_has_double_excitation(c, cfg_b("has_double_excitation", true) ? 1 : 0),
     "has_double_excitation");
  if (cfg_b("chem/active_space", false)) {  // integrals.cc:295-326
    if (reorder < 0 ? !explicit_orbs : reorder != 0)
      die("Set reorder_orbs to false for active space calculations");
    const std::vector<double> as = cfg_v("chem/irrep_active_space", false);
    if (as.empty()) die("Active space specification is missing or incorrect.");
    std::vector<unsigned> asu(as.begin(), as.end());
    ck(c, shci_set_active_space(c, asu.data(), asu.size()), "active space");
  }
  // "var_sd" defaults to "get_pair_contrib" (solver.h:423-424)
  const bool pair_contrib = cfg_b("get_pair_contrib", false);
  ck(c, shci_set_var_sd(c, cfg_b("var_sd", pair_contrib) ? 1 : 0), "var_sd");

  double qinfo[4];
  ck(c, shci_build_queues(c, qinfo), "heat-bath queues");
  std::printf("Max hci queue elem: %.10f Ha\nNumber of entries in hci queue: %'zu\n", qinfo[0],
              (size_t)qinfo[1]);
  std::printf("Max singles_queue elem: %.10f Ha\nNumber of entries in singles_queue: %'zu\n",
              qinfo[2], (size_t)qinfo[3]);
  std::printf("HF energy: %.10f Ha\n", e_hf);
  {
    Json ne = Json::number(n_up + n_dn);
    ne.is_int = true;
    g_result.put("n_elecs") = ne;
  }
  result_put("energy_hf", e_hf);

  const std::vector<double> eps_vars = cfg_v("eps_vars", true);
  const std::vector<double> schedule = cfg_v("eps_vars_schedule", true);
  std::vector<Wavefunction> wfs;
  // Solver<S>::save_pair_contrib (solver.h:1227-1296): the first state's H_0j c_j / c_0 of
  // every det j within a double excitation of det 0, summed per pair (i, j) of the det-0
  // orbitals it vacates (i = j for singles; pairs i != j halved), in det order
  auto save_pair_contrib = [&](const Wavefunction& w, double eps_var) {
    const uint64_t hu = w.up[0], hd = w.dn[0];
    if (hu != hd) die("non sym det_hf not implemented");
    const size_t nd = w.up.size();
    std::vector<uint64_t> iu(nd, hu), id(nd, hd);
    std::vector<double> h(nd, 0.0);
    ck(c, shci_hamiltonian_elems(c, iu.data(), id.data(), w.up.data(), w.dn.data(), nd, h.data()),
       "pair contributions");
    std::vector<double> contrib((size_t)n_up * n_up, 0.0);
    const double c0 = w.coefs[0];
    auto left = [](uint64_t a, uint64_t b, unsigned* o) {  // orbitals in a only, ascending
      unsigned k = 0;
      for (uint64_t m = a & ~b; m && k < 3; m &= m - 1) o[k++] = __builtin_ctzll(m);
      return k;
    };
    for (size_t d = 1; d < nd; d++) {
      unsigned lu[3], ld[3];
      const unsigned nu = left(hu, w.up[d], lu), ndn = left(hd, w.dn[d], ld);
      if (nu + ndn > 2) continue;
      size_t i = 0, j = 0;
      if (nu == 2) {
        i = lu[0];
        j = lu[1];
      } else if (nu == 1) {
        i = lu[0];
        j = ndn == 1 ? ld[0] : i;
        if (j < i) std::swap(i, j);
      } else {
        i = ld[0];
        j = ndn == 2 ? ld[1] : i;
        if (j < i) std::swap(i, j);
      }
      if (i >= n_up || j >= n_up) die("pair contribution outside the first n_up orbitals");
      double v = h[d] * w.coefs[d] / c0;
      if (w.up[d] != w.dn[d] && time_sym) v = h[d] * w.coefs[d] / c0 * 1.4142135623730951;
      contrib[i * n_up + j] += v;
    }
    char name[64];
    std::snprintf(name, sizeof(name), "pair_contrib_%#.2e.csv", eps_var);
    FILE* f = std::fopen(name, "w");
    if (!f) die(std::string("cannot write ") + name);
    std::fprintf(f, "i,j,pair_contrib\n");
    for (size_t i = 0; i < n_up; i++)
      for (size_t j = i; j < n_up; j++) {
        double v = contrib[i * n_up + j];
        if (i != j) v /= 2;
        std::fprintf(f, "%zu,%zu,%.15g\n", i, j, v);
      }
    std::fclose(f);
    result_put_str("pair_contrib/" + key_eps(eps_var), name);
  };
  if (!cfg_b("skip_var", false)) {
    std::printf("Final iteration 0 HF ndets= 1 energy= %.8f\n", e_hf);
    double eps_prev = 1e100;
    size_t it_s = 0;
    size_t it_global = 0;
    for (double eps_var : eps_vars) {
      const std::string fn = wf_filename(eps_var);
      std::printf("Try Loading Wavefunction %s\n", fn.c_str());
      Wavefunction lw;
      if (!cfg_b("force_var", false) &&
          load_wf(fn, n_up, n_dn, n_states, time_sym, eps_var, &lw)) {
        // solver.h:381-388: continue from the loaded wavefunction, memo cleared
        put_wf(c, lw);
        for (size_t k = 0; k < lw.n_states(); k++)
          result_put("energy_var" + state_suffix(k) + "/" + key_eps(eps_var), lw.energy_of(k));
        wfs.push_back(std::move(lw));
        if (pair_contrib) save_pair_contrib(wfs.back(), eps_var);
        eps_prev = eps_var;
        continue;
      }
      std::vector<double> sched;
      while (it_s < schedule.size() && schedule[it_s] >= eps_prev) it_s++;
      while (it_s < schedule.size() && schedule[it_s] > eps_var) sched.push_back(schedule[it_s++]);
      double e = 0.0;
      ck(c, shci_run_variation(c, &eps_var, 1, sched.empty() ? nullptr : sched.data(),
                               sched.size(), target_error, prec, &e),
         "variation");
      size_t n_it = 0;
      ck(c, shci_get_var_trace(c, nullptr, nullptr, nullptr, 0, &n_it), "trace");
      std::vector<uint64_t> nd(n_it), nz(n_it);
      std::vector<double> en(n_it);
      ck(c, shci_get_var_trace(c, nd.data(), nz.data(), en.data(), n_it, &n_it), "trace");
      std::vector<double> es(n_it * n_states);
      ck(c, shci_get_var_trace_states(c, es.data(), es.size(), &n_it), "trace");
      for (size_t k = 0; k < n_it; k++) {
        const double eps_k = k < sched.size() ? sched[k] : eps_var;
        std::printf("Number of nonzero elems: %'zu\n", (size_t)nz[k]);
        std::printf("Iteration %zu eps1= %#.2e ndets= %'zu energy=", ++it_global, eps_k,
                    (size_t)nd[k]);
        for (unsigned st = 0; st < n_states; st++) std::printf(" %.8f", es[k * n_states + st]);
        std::printf("\n");
      }
      Wavefunction wf;
      wf.eps_var = eps_var;
      wf.energy = e;
      size_t n = 0;
      ck(c, shci_get_n_dets(c, &n), "dets");
      wf.up.resize(n);
      wf.dn.resize(n);
      wf.coefs.resize(n);
      ck(c, shci_get_dets(c, wf.up.data(), wf.dn.data(), wf.coefs.data(), n), "dets");
      std::vector<double> se(n_states);
      ck(c, shci_get_state_energies(c, se.data(), n_states), "state energies");
      for (unsigned st = 1; st < n_states; st++) {
        wf.xcoefs.emplace_back(n);
        ck(c, shci_get_state_coefs(c, st, wf.xcoefs.back().data(), n), "state coefficients");
        wf.xenergy.push_back(se[st]);
      }
      std::printf("Final iteration %zu eps1= %#.2e ndets= %'zu energy=", it_global, eps_var, n);
      for (unsigned st = 0; st < n_states; st++) std::printf("  %.8f", wf.energy_of(st));
      std::printf("\n");
      for (unsigned st = 0; st < n_states; st++)
        result_put("energy_var" + state_suffix(st) + "/" + key_eps(eps_var), wf.energy_of(st));
      save_wf(fn, n_up, n_dn, time_sym, e_hf, wf);
      wfs.push_back(std::move(wf));
      if (pair_contrib) save_pair_contrib(wfs.back(), eps_var);
      eps_prev = eps_var;
    }
  }

  const bool want_1rdm = cfg_b("get_1rdm_csv", false);
  const bool want_2rdm = cfg_b("2rdm", false) || cfg_b("get_2rdm_csv", false);
  // from here on the wavefunctions are used unpacked (solver.h:593; the reference's RDM code
  // reads packed time_sym dets with the same result)
  if (time_sym) ck(c, shci_set_time_sym(c, 0), "time_sym");
  if ((want_1rdm || want_2rdm) && !wfs.empty()) {
    const Wavefunction wf = time_sym ? unpacked(wfs.back()) : wfs.back();
    put_wf(c, wf);  // the RDMs sum over the states (rdm.cc:222-231)
    std::vector<unsigned> order(n_orbs), inv(n_orbs);
    ck(c, shci_get_integrals(c, nullptr, nullptr, nullptr, nullptr, nullptr, order.data()), "order");
    for (int i = 0; i < n_orbs; i++) inv[order[i]] = i;
    const size_t n = n_orbs;
    if (want_1rdm) {  // rdm.cc:202-221
      std::vector<double> g1(n * n);
      ck(c, shci_rdm1(c, g1.data()), "1-RDM");
      FILE* f = std::fopen("1rdm.csv", "w");
      std::fprintf(f, "p,r,1rdm\n");
      for (size_t p = 0; p < n; p++)
        for (size_t r = p; r < n; r++) {
          const double v = g1[p * n + r];
          if (std::fabs(v) < 1e-9) continue;
          std::fprintf(f, "%d,%d,%#.15g\n", order[p], order[r], v);
        }
      std::fclose(f);
    }
    if (want_2rdm) {  // rdm.cc:271-331
      size_t nnz[2];
      ck(c, shci_update_hamiltonian(c, SHCI_PREC_FP64, nnz), "Hamiltonian");
      const size_t nn = n * n;
      std::vector<double> half(nn * (nn + 1) / 2);
      ck(c, shci_rdm2(c, half.data()), "2-RDM");
      auto elem = [&](size_t p, size_t q, size_t r, size_t s) {
        size_t a = p * n + s, b = q * n + r;
        if (a < b) std::swap(a, b);
        return half[a * (a + 1) / 2 + b];
      };
      std::printf("writing out 2RDM\n");
      if (cfg_b("get_2rdm_csv", false)) {
        FILE* f = std::fopen("2rdm.csv", "w");
        std::fprintf(f, "p,q,r,s,2rdm\n");
        for (size_t p = 0; p < n; p++)
          for (size_t q = p; q < n; q++)
            for (size_t s = 0; s < n; s++)
              for (size_t r = 0; r < n; r++) {
                if (p == q && s > r) continue;
                const double v = elem(p, q, r, s);
                if (std::fabs(v) < 1.0e-9) continue;
                std::fprintf(f, "%d,%d,%d,%d,%#.15g\n", order[p], order[q], order[r], order[s], v);
              }
        std::fclose(f);
      } else {
        FILE* f = std::fopen("spatialRDM.txt", "w");
        std::fprintf(f, "%d\n", n_orbs);
        for (size_t p = 0; p < n; p++)
          for (size_t q = 0; q < n; q++)
            for (size_t s = 0; s < n; s++)
              for (size_t r = 0; r < n; r++) {
                const double v = elem(inv[p], inv[q], inv[r], inv[s]);
                if (std::fabs(v) > 1.e-6)
                  std::fprintf(f, "%3zu   %3zu   %3zu   %3zu   %10.8g\n", p, q, s, r, v);
              }
        std::fclose(f);
      }
    }
  }
  // <S^2> of the first state (post_variation, chem_system.cc:627-634)
  if (cfg_b("s2", false) && !wfs.empty()) {
    const Wavefunction wf = time_sym ? unpacked(wfs.back()) : wfs.back();
    put_wf(c, wf);
    double s2 = 0.0;
    ck(c, shci_get_s2(c, &s2), "S^2");
    std::printf("s_squared: %15.10f\n", s2);
    result_put("s2", s2);
  }
  if (cfg_b("var_only", false)) {
    shci_destroy(c);
    return 0;
  }

  // Perturbation for each eps_var (solver.h:399-411, 541-634)
  for (const double eps_var_cfg : eps_vars) {
    const Wavefunction* wp = nullptr;
    for (const Wavefunction& w : wfs)
      if (w.eps_var == eps_var_cfg) wp = &w;
    Wavefunction lw;
    if (!wp) {  // skip_var: the wavefunction comes from its file (solver.h:571-575)
      if (!load_wf(wf_filename(eps_var_cfg), n_up, n_dn, n_states, time_sym, eps_var_cfg, &lw))
        die("cannot load variation results from " + wf_filename(eps_var_cfg));
      wp = &lw;
    }
    const Wavefunction uw = time_sym ? unpacked(*wp) : Wavefunction();
    const Wavefunction& wf = time_sym ? uw : *wp;
    const double eps_var = wf.eps_var;
    double eps_pt_dtm = std::max(2.0e-6, cfg_d("eps_pt_dtm_ratio", 0.1) * eps_var);
    double eps_pt_psto = std::max(1.0e-7, cfg_d("eps_pt_psto_ratio", 0.01) * eps_var);
    double eps_pt = cfg_d("eps_pt_ratio", 1.0e-3) * eps_var;
    eps_pt_dtm = cfg_d("eps_pt_dtm", eps_pt_dtm);
    eps_pt_psto = cfg_d("eps_pt_psto", eps_pt_psto);
    eps_pt = cfg_d("eps_pt", eps_pt);
    if (eps_pt_psto < eps_pt) eps_pt_psto = eps_pt;
    if (eps_pt_dtm < eps_pt_psto) eps_pt_dtm = eps_pt_psto;
    // solver.h:546-568: skipped when every state's total is in result.json
    auto base_of = [&](size_t st) {
      return "energy_total" + state_suffix(st) + "/" + key_eps(eps_var) + "/" + key_eps(eps_pt);
    };
    bool missing = false;
    for (size_t st = 0; st < wf.n_states(); st++) {
      const Json* have = g_result.get(base_of(st) + "/value");
      if (have && have->type == Json::Number && have->num != 0.0) {
        const Json* hu = g_result.get(base_of(st) + "/uncert");
        std::printf("Total energy: %.10f +- %.10f (state %zu, loaded from result file)\n",
                    have->num, hu ? hu->num : 0.0, st);
      } else {
        missing = true;
      }
    }
    if (!missing && !cfg_b("force_pt", false)) continue;
    for (size_t st = 0; st < wf.n_states(); st++) {
      // state st: its coefficients and energy (solver.h:620-632)
      const std::string base = base_of(st);
      const double energy = wf.energy_of(st);
      ck(c, shci_set_dets(c, wf.up.data(), wf.dn.data(), wf.coefs_of(st).data(), wf.up.size()),
         "dets");
      double dtm = 0.0, u_dtm = 0.0;
      size_t n_dtm = 0;
      ck(c, shci_pt2_dtm(c, energy, eps_pt_dtm, (size_t)cfg_d("n_batches_pt_dtm", 0), &dtm,
                         &u_dtm, &n_dtm),
         "PT2 dtm");
      std::printf("Number of dtm pt dets: %'zu\n", n_dtm);
      std::printf("PT dtm correction (eps1= %.2e, eps_pt_dtm= %.2e): %.10f +- %.10f Ha\n", eps_var,
                  eps_pt_dtm, dtm, u_dtm);
      double value = energy + dtm, uncert = 0.0;
      double psto = 0.0, u_psto = 0.0;
      double pt_mem = 0.0;
      if (eps_pt_psto < eps_pt_dtm || eps_pt < eps_pt_psto)
        ck(c, shci_pt_mem_avail(c, cfg_d("mem_total", machine_memory()), &pt_mem), "PT memory");
      if (eps_pt_psto < eps_pt_dtm) {
        size_t n_psto = 0, nb = 0;
        // n_batches_pt_psto, or the reference's estimate from a pilot and the PT memory
        // (solver.h:772-814)
        size_t nb_psto = (size_t)cfg_d("n_batches_pt_psto", 0);
        if (nb_psto == 0) {
          ck(c, shci_pt2_psto_auto_batches(c, eps_pt_psto, pt_mem,
                                           cfg_d("pt_psto_mem_usage", 1.0), &nb_psto, nullptr),
             "psto batches");
          std::printf("Number of psto batches: %zu\n", nb_psto);
        }
        ck(c, shci_pt2_psto(c, energy, eps_pt_dtm, eps_pt_psto, nb_psto, target_error, eps_pt,
                            &psto, &u_psto, &n_psto, &nb),
           "PT2 psto");
        std::printf("PT psto correction (eps1= %.2e, eps_pt_psto= %.2e): %.10f +- %.10f Ha\n",
                    eps_var, eps_pt_psto, psto, u_psto);
        value += psto;
        uncert = u_psto;
      }
      if (eps_pt < eps_pt_psto) {
        // solver.h:905-1036: the sample size comes from the pilot and the PT memory unless
        // n_dets_in_sample_pt_sto is set; semisto_sto (default true) needs the pilot
        const size_t n_samples = (size_t)cfg_d("n_dets_in_sample_pt_sto", 0);
        const bool semisto = cfg_b("semisto_sto", true);
        double sto = 0.0, u_sto = 0.0;
        size_t iters = 0, info[3] = {0, 0, 0};
        size_t nb_sto = (size_t)cfg_d("n_batches_pt_sto", 0);
        if (nb_sto == 0) nb_sto = 64;  // solver.h:907-908
        ck(c, shci_pt2_sto(c, energy, eps_pt_psto, eps_pt, nb_sto,
                           n_samples, semisto ? 1 : 0, (unsigned)cfg_d("random_seed", 347634253),
                           (size_t)cfg_d("max_pt_iterations", 100), target_error, u_psto, pt_mem,
                           cfg_d("pt_sto_mem_usage", 0.4), &sto, &u_sto, &iters, info, nullptr, 0),
           "PT2 sto");
        if (n_samples == 0) {
          std::printf("Number of unique var dets in sample target: %'zu\n", info[2]);
          std::printf("Number of dets chosen: %'zu\n", info[0]);
        }
        if (semisto) std::printf("Number of deterministic var dets: %'zu\n", info[1]);
        std::printf("PT sto correction (eps1= %.2e, eps_pt= %.2e): %.10f +- %.10f Ha\n", eps_var,
                    eps_pt, sto, u_sto);
        value += sto;
        uncert = std::sqrt(uncert * uncert + u_sto * u_sto);
      }
      std::printf("Total energy: %.10f +- %.10f Ha (state %zu)\n", value, uncert, st);
      result_put(base + "/value", value);
      result_put(base + "/uncert", uncert);
    }
  }
  shci_destroy(c);
  return 0;
}

// Variational wavefunction checkpoints: Solver<S>::save_variation_result /
// load_variation_result (src/solver/solver.h:1179-1224), file name get_wf_filename
// ("wf_eps1_%#.2e.dat", solver.h:1415-1417).
//
// The reference serialises the BaseSystem fields n_up, n_dn, dets, coefs, energy_hf,
// energy_var, time_sym (src/base_system.h:125-133) with hps, an un-vendored library whose
// byte format is not available here.  This build stores the same fields in its own
// little-endian layout, documented here and readable with a few lines of any language:
//
//   offset 0   8 bytes   magic "SHCIGWF1"
//              u32       n_up
//              u32       n_dn
//              u32       n_states
//              u32       time_sym (1: dets in the form up <= dn stand for time-reversal pairs)
//              u64       n_dets
//              f64       energy_hf
//              f64       energy_var[n_states]
//              u64       up[n_dets]      alpha strings, bit k = orbital k (reordered basis)
//              u64       dn[n_dets]      beta strings
//              f64       coefs[n_states][n_dets]
//
// A file that does not start with the magic (for instance one the reference wrote) is not
// read and is never overwritten.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace shci_cli {

constexpr char kWfMagic[8] = {'S', 'H', 'C', 'I', 'G', 'W', 'F', '1'};

struct WfFile {
  unsigned n_up = 0, n_dn = 0, n_states = 1, time_sym = 0;
  double energy_hf = 0.0;
  std::vector<double> energy_var;  // [n_states]
  std::vector<uint64_t> up, dn;
  std::vector<double> coefs;       // [n_states * n_dets], state by state
};

enum class WfStatus { kOk, kMissing, kForeign, kBad };

inline WfStatus wf_probe(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return WfStatus::kMissing;
  char m[8];
  const bool ours = std::fread(m, 1, 8, f) == 8 && std::memcmp(m, kWfMagic, 8) == 0;
  std::fclose(f);
  return ours ? WfStatus::kOk : WfStatus::kForeign;
}

inline WfStatus wf_load(const std::string& path, WfFile* w) {
  const WfStatus st = wf_probe(path);
  if (st != WfStatus::kOk) return st;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return WfStatus::kMissing;
  bool ok = true;
  auto rd = [&](void* p, size_t n) { ok = ok && std::fread(p, 1, n, f) == n; };
  char m[8];
  uint32_t hdr[4] = {0, 0, 0, 0};
  uint64_t n = 0;
  rd(m, 8);
  rd(hdr, sizeof(hdr));
  rd(&n, 8);
  ok = ok && hdr[2] >= 1 && hdr[2] <= 64 && hdr[3] <= 1 && n > 0 && n < (1ull << 40);
  if (ok) {
    w->n_up = hdr[0];
    w->n_dn = hdr[1];
    w->n_states = hdr[2];
    w->time_sym = hdr[3];
    rd(&w->energy_hf, 8);
    w->energy_var.resize(w->n_states);
    rd(w->energy_var.data(), 8 * w->n_states);
    w->up.resize(n);
    w->dn.resize(n);
    w->coefs.resize(n * w->n_states);
    rd(w->up.data(), n * 8);
    rd(w->dn.data(), n * 8);
    rd(w->coefs.data(), n * 8 * w->n_states);
  }
  std::fclose(f);
  return ok ? WfStatus::kOk : WfStatus::kBad;
}

inline bool wf_save(const std::string& path, const WfFile& w) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = true;
  auto wr = [&](const void* p, size_t n) { ok = ok && std::fwrite(p, 1, n, f) == n; };
  const uint32_t hdr[4] = {w.n_up, w.n_dn, w.n_states, w.time_sym};
  const uint64_t n = w.up.size();
  wr(kWfMagic, 8);
  wr(hdr, sizeof(hdr));
  wr(&n, 8);
  wr(&w.energy_hf, 8);
  wr(w.energy_var.data(), 8 * w.n_states);
  wr(w.up.data(), n * 8);
  wr(w.dn.data(), n * 8);
  wr(w.coefs.data(), n * 8 * w.n_states);
  return std::fclose(f) == 0 && ok;
}

}  // namespace shci_cli

// C ABI of libshci_gpu.so (declared in include/shci_gpu.h).  Every entry point catches
// exceptions and CUDA errors and turns them into a status plus shci_last_error().
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "ctx.h"
#include "kernels.h"
#include "solver.h"

using namespace shci;

namespace {

template <class F>
shci_status guard(shci_ctx* c, F f) {
  try {
    if (c) {
      c->err.clear();
      SHCI_CUDA(cudaSetDevice(c->device));
    }
    f();
    return SHCI_OK;
  } catch (const OomError& e) {
    if (c) c->err = e.what();
    return SHCI_ERR_OOM;
  } catch (const ArgError& e) {
    if (c) c->err = e.what();
    return SHCI_ERR_ARG;
  } catch (const OverflowError& e) {
    if (c) c->err = e.what();
    return SHCI_ERR_OVERFLOW;
  } catch (const CudaError& e) {
    if (c) c->err = e.what();
    return e.code == cudaErrorMemoryAllocation ? SHCI_ERR_OOM : SHCI_ERR_CUDA;
  } catch (const std::bad_alloc&) {
    if (c) c->err = "host allocation failed";
    return SHCI_ERR_OOM;
  } catch (const std::exception& e) {
    if (c) c->err = e.what();
    return SHCI_ERR_IO;
  }
}

void need_integrals(shci_ctx* c) {
  if (!c->have_integrals) throw ArgError("no integrals loaded");
}

void need_dets(shci_ctx* c) {
  if (c->up.empty()) throw ArgError("no determinants set");
}

// States 1 .. n_states - 1 start at 1e-16 on each of the n current dets (chem_system.cc:52-56)
void reset_states(shci_ctx* c, size_t n) {
  const std::vector<double> tiny(n, 1e-16);
  for (unsigned k = 1; k < c->n_states; k++) {
    auto& xc = c->d_xcoef[k - 1];
    xc.mt = &c->mem;
    xc.resize(n, 1.1);
    SHCI_CUDA(cudaMemcpyAsync(xc.p, tiny.data(), n * 8, cudaMemcpyHostToDevice, c->stream));
  }
  SHCI_CUDA(cudaStreamSynchronize(c->stream));
  c->state_energy.assign(c->n_states, 0.0);
}

// The Hamiltonian drops opposite-spin doubles when the system has no double excitations and
// no time-reversal symmetry (hamiltonian.h:97-104, 487).
void apply_excitation_flags(shci_ctx* c) {
  c->dI.no_mixed_doubles = (!c->has_doubles && !c->time_sym) ? 1 : 0;
}

void after_integrals(shci_ctx* c) {
  upload_integrals(c);
  apply_excitation_flags(c);
  c->inactive_orbs = 0;  // an active space refers to the previous integrals' orbitals
  c->have_integrals = true;
  c->Q.built = false;
  c->up.assign(1, c->I.hf_up);
  c->dn.assign(1, c->I.hf_dn);
  c->coefs.assign(1, 1.0);
  c->dets_dirty = true;
  c->eps_tried.clear();
  c->H.valid = false;
  c->H.prefix_ok = false;
  c->H.build_id++;
  reset_states(c, 1);
}

// An explicit upper-triangle CSR (FP64) becomes the context's Hamiltonian (Davidson tests).
void load_csr(shci_ctx* c, size_t n, const uint64_t* row_ptr, const uint32_t* cols,
              const double* vals, const double* diag) {
  auto& H = c->H;
  cudaStream_t s = c->stream;
  const size_t nnz = row_ptr[n];
  H.older.clear();
  H.prefix_ok = false;
  H.n = n;
  H.nnz = nnz;
  H.nnz_current = nnz;
  H.precision = SHCI_PREC_FP64;
  H.row_ptr.resize(n + 1);
  H.col.resize(nnz ? nnz : 1);
  H.val64.resize(nnz ? nnz : 1);
  H.diag.resize(n);
  SHCI_CUDA(cudaMemcpyAsync(H.row_ptr.p, row_ptr, (n + 1) * 8, cudaMemcpyHostToDevice, s));
  std::vector<uint32_t> len(n);
  for (size_t i = 0; i < n; i++) len[i] = static_cast<uint32_t>(row_ptr[i + 1] - row_ptr[i]);
  H.row_cnt.resize(n + 1);
  SHCI_CUDA(cudaMemcpyAsync(H.row_cnt.p, len.data(), n * 4, cudaMemcpyHostToDevice, s));
  H.packed = true;
  H.bound_valid = false;
  SHCI_CUDA(cudaStreamSynchronize(s));
  if (nnz) {
    SHCI_CUDA(cudaMemcpyAsync(H.col.p, cols, nnz * 4, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(H.val64.p, vals, nnz * 8, cudaMemcpyHostToDevice, s));
  }
  SHCI_CUDA(cudaMemcpyAsync(H.diag.p, diag, n * 8, cudaMemcpyHostToDevice, s));
  H.valid = true;
  H.build_id++;
}

// After a CSR Davidson the context's own Hamiltonian and coefficients are gone.
void drop_csr(shci_ctx* c) {
  c->H.valid = false;
  c->H.prefix_ok = false;
  c->H.older.clear();
  c->H.build_id++;
  c->dets_dirty = true;
}


}  // namespace

extern "C" {

shci_status shci_create(shci_ctx** out, int device, size_t hbm_budget_bytes) {
  if (!out) return SHCI_ERR_ARG;
  *out = nullptr;
  shci_ctx* c = new (std::nothrow) shci_ctx();
  if (!c) return SHCI_ERR_OOM;
  c->device = device;
  c->mem.budget = hbm_budget_bytes;
  shci_status st = guard(c, [&]() {
    int n = 0;
    SHCI_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) throw ArgError("no such CUDA device");
    SHCI_CUDA(cudaSetDevice(device));
    SHCI_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    // every device buffer of the context is accounted against the budget
    for (auto* b : {&c->h1, &c->g2, &c->dtab, &c->xtab, &c->jtab, &c->ktab, &c->d_coef, &c->f0,
                    &c->f1})
      b->mt = &c->mem;
    for (auto* b : {&c->d_up, &c->d_dn, &c->set_up, &c->set_dn, &c->k0, &c->k1, &c->k2})
      b->mt = &c->mem;
    for (auto* b : {&c->u0, &c->u1, &c->u2}) b->mt = &c->mem;
    c->err_word.mt = &c->mem;
    c->sort.set_tracker(&c->mem);
    auto& ix = c->idx;
    for (auto* b : {&ix.det_aid, &ix.det_bid, &ix.a_start, &ix.b_start, &ix.am_idx, &ix.ad_idx,
                    &ix.bd_idx, &ix.as_off, &ix.as_list, &ix.bs_off, &ix.bs_list})
      b->mt = &c->mem;
    for (auto* b : {&ix.am_dn, &ix.ad_dn, &ix.bd_up, &ix.ua, &ix.ub, &ix.bs_str}) b->mt = &c->mem;
    c->join.pairs.mt = c->join.jdet.mt = &c->mem;
    c->join.keys.mt = c->join.span.mt = c->join.keys32.mt = &c->mem;
    c->join.scan.mt = c->join.bstart.mt = &c->mem;
    auto& H = c->H;
    H.row_ptr.mt = H.col.mt = H.row_cnt.mt = &c->mem;
    H.val64.mt = H.diag.mt = &c->mem;
    H.val32.mt = H.res32.mt = &c->mem;
    H.scal.mt = H.xs.mt = H.yfix.mt = H.rowabs.mt = &c->mem;
    c->dav.scal.mt = c->dav.partial.mt = &c->mem;
  });
  if (st != SHCI_OK) {
    delete c;
    return st;
  }
  *out = c;
  return SHCI_OK;
}

shci_status shci_destroy(shci_ctx* c) {
  if (!c) return SHCI_ERR_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaStream_t s = c->stream;
  delete c;  // buffers free themselves
  if (s) cudaStreamDestroy(s);
  return SHCI_OK;
}

const char* shci_last_error(const shci_ctx* c) { return c ? c->err.c_str() : "null context"; }

void* shci_stream(shci_ctx* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

shci_status shci_load_fcidump(shci_ctx* c, const char* path, unsigned n_up, unsigned n_dn,
                              const char* point_group, int reorder, const unsigned* occs_up,
                              const unsigned* occs_dn) {
  if (!c) return SHCI_ERR_ARG;
  shci_status st = guard(c, [&]() {
    if (!path) throw ArgError("null path");
    HostIntegrals I;
    try {
      load_fcidump(I, path, n_up, n_dn, point_group ? point_group : "C1", reorder, occs_up,
                   occs_dn, c->hf_opts);
    } catch (const std::runtime_error& e) {
      throw;  // mapped to SHCI_ERR_IO below
    }
    c->I = std::move(I);
    after_integrals(c);
  });
  return st;
}

shci_status shci_save_integrals_cache(shci_ctx* c, const char* path, int* written) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (!path) throw ArgError("null path");
    need_integrals(c);
    const CacheStatus st = save_integrals_cache(c->I, path);
    if (written) *written = st == kCacheOk ? 1 : 0;
  });
}

shci_status shci_load_integrals_cache(shci_ctx* c, const char* path, unsigned n_up, unsigned n_dn,
                                      const char* point_group, int* loaded) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (!path) throw ArgError("null path");
    if (loaded) *loaded = 0;
    HostIntegrals I;
    if (load_integrals_cache(I, path, point_group ? point_group : "C1") != kCacheOk) return;
    if (I.n_up != n_up || I.n_dn != n_dn)
      throw ArgError(std::string(path) + " holds integrals for n_up = " +
                     std::to_string(I.n_up) + ", n_dn = " + std::to_string(I.n_dn));
    c->I = std::move(I);
    after_integrals(c);
    if (loaded) *loaded = 1;
  });
}

shci_status shci_set_integrals(shci_ctx* c, int n_orbs, unsigned n_up, unsigned n_dn,
                               double e_core, const double* h1, const double* g2,
                               const unsigned* orb_sym, const char* point_group, uint64_t hf_up,
                               uint64_t hf_dn) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (n_orbs <= 0 || n_orbs > 64) throw ArgError("n_orbs must be in [1, 64]");
    if (!h1 || !g2) throw ArgError("null integral array");
    HostIntegrals I;
    const size_t n = n_orbs;
    I.n = n_orbs;
    I.n_up = n_up;
    I.n_dn = n_dn;
    I.e_core = e_core;
    I.n_syms = point_group_order(point_group ? point_group : "C1", &I.linear);
    I.h1.assign(h1, h1 + n * n);
    I.g2.assign(g2, g2 + n * n * n * n);
    I.orb_sym.resize(n);
    I.orb_order.resize(n);
    for (size_t i = 0; i < n; i++) {
      I.orb_sym[i] = orb_sym ? orb_sym[i] : 1u;
      I.orb_order[i] = static_cast<unsigned>(i);
    }
    if (__builtin_popcountll(hf_up) != (int)n_up || __builtin_popcountll(hf_dn) != (int)n_dn)
      throw ArgError("HF det does not match n_up / n_dn");
    screen_linear(I);
    I.hf_up = hf_up;
    I.hf_dn = hf_dn;
    c->I = std::move(I);
    after_integrals(c);
  });
}

shci_status shci_get_integrals(shci_ctx* c, int* n_orbs, double* e_core, double* h1, double* g2,
                               unsigned* orb_sym, unsigned* orb_order) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    const auto& I = c->I;
    if (n_orbs) *n_orbs = static_cast<int>(I.n);
    if (e_core) *e_core = I.e_core;
    if (h1) std::memcpy(h1, I.h1.data(), I.h1.size() * 8);
    if (g2) std::memcpy(g2, I.g2.data(), I.g2.size() * 8);
    if (orb_sym) std::memcpy(orb_sym, I.orb_sym.data(), I.n * sizeof(unsigned));
    if (orb_order) std::memcpy(orb_order, I.orb_order.data(), I.n * sizeof(unsigned));
  });
}

shci_status shci_get_hf(shci_ctx* c, uint64_t* up, uint64_t* dn, double* e) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    if (up) *up = c->I.hf_up;
    if (dn) *dn = c->I.hf_dn;
    if (e) *e = c->energy_hf;
  });
}

shci_status shci_build_queues(shci_ctx* c, double* info) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    upload_queues(c);
    if (info) {
      info[0] = c->Q.max_hci;
      info[1] = static_cast<double>(c->Q.n_hci);
      info[2] = c->Q.max_singles;
      info[3] = static_cast<double>(c->Q.n_singles);
    }
  });
}

shci_status shci_set_dets(shci_ctx* c, const uint64_t* up, const uint64_t* dn,
                          const double* coefs, size_t n) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    if (n == 0 || !up || !dn) throw ArgError("empty det list");
    const uint64_t full = c->I.n == 64 ? ~0ull : ((1ull << c->I.n) - 1ull);
    // checks and host copies in chunks over the host threads
    const size_t n_chunks = std::min<size_t>(host_threads(), (n + 65535) / 65536);
    auto chunked = [&](auto f) {
      std::vector<std::thread> th;
      for (size_t t = 1; t < n_chunks; t++) th.emplace_back(f, n * t / n_chunks, n * (t + 1) / n_chunks);
      f(size_t{0}, n / n_chunks);
      for (auto& x : th) x.join();
    };
    std::atomic<size_t> bad{n};
    chunked([&](size_t b, size_t e) {
      for (size_t i = b; i < e; i++)
        if ((up[i] & ~full) || (dn[i] & ~full) ||
            __builtin_popcountll(up[i]) != (int)c->I.n_up ||
            __builtin_popcountll(dn[i]) != (int)c->I.n_dn) {
          size_t cur = bad.load();
          while (i < cur && !bad.compare_exchange_weak(cur, i)) {
          }
          break;
        }
    });
    if (bad.load() < n)
      throw ArgError("det " + std::to_string(bad.load()) +
                     " has the wrong electron count or orbitals");
    // device copies straight from the caller's buffers (pinned buffers give async DMA), the
    // host copies meanwhile
    cudaStream_t s = c->stream;
    c->d_up.resize(n, 1.1);
    c->d_dn.resize(n, 1.1);
    c->d_coef.resize(n, 1.1);
    SHCI_CUDA(cudaMemcpyAsync(c->d_up.p, up, n * 8, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(c->d_dn.p, dn, n * 8, cudaMemcpyHostToDevice, s));
    if (coefs) SHCI_CUDA(cudaMemcpyAsync(c->d_coef.p, coefs, n * 8, cudaMemcpyHostToDevice, s));
    c->up.resize(n);
    c->dn.resize(n);
    if (coefs) c->coefs.resize(n);
    chunked([&](size_t b, size_t e) {
      std::memcpy(c->up.data() + b, up + b, (e - b) * 8);
      std::memcpy(c->dn.data() + b, dn + b, (e - b) * 8);
      if (coefs) std::memcpy(c->coefs.data() + b, coefs + b, (e - b) * 8);
    });
    if (!coefs) {
      c->coefs.assign(n, 1e-16);
      c->coefs[0] = 1.0;
      SHCI_CUDA(cudaMemcpyAsync(c->d_coef.p, c->coefs.data(), n * 8, cudaMemcpyHostToDevice, s));
    }
    SHCI_CUDA(cudaStreamSynchronize(s));
    c->dets_dirty = false;
    c->eps_tried.clear();
    c->H.valid = false;
    c->H.prefix_ok = false;
    c->H.build_id++;
    reset_states(c, n);
  });
}

shci_status shci_set_n_states(shci_ctx* c, unsigned n_states) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    if (n_states < 1 || n_states > kMaxStates)
      throw ArgError("n_states must be in [1, " + std::to_string(kMaxStates) + "]");
    c->n_states = n_states;
    reset_states(c, c->up.size());
  });
}

shci_status shci_set_time_sym(shci_ctx* c, int on) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    if (on) {
      if (c->I.n_up != c->I.n_dn) throw ArgError("time_sym needs n_up == n_dn");
      for (size_t i = 0; i < c->up.size(); i++)
        if (c->up[i] > c->dn[i])
          throw ArgError("time_sym needs every det in the form up <= dn (det " +
                         std::to_string(i) + ")");
    }
    c->time_sym = on != 0;
    apply_excitation_flags(c);
    c->H.valid = false;
    c->H.prefix_ok = false;
    c->H.build_id++;
    c->eps_tried.clear();
  });
}

shci_status shci_unpack_time_sym(shci_ctx* c) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_dets(c);
    if (!c->time_sym) throw ArgError("the context is not in time_sym mode");
    const size_t n = c->up.size();
    const unsigned ns = c->n_states;
    std::vector<std::vector<double>> cs(ns, std::vector<double>(n));
    sync_dets(c);
    for (unsigned k = 0; k < ns; k++)
      SHCI_CUDA(cudaMemcpyAsync(cs[k].data(), state_coef(c, k), n * 8, cudaMemcpyDeviceToHost,
                                c->stream));
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<uint64_t> up(c->up), dn(c->dn);
    constexpr double kSqrt2Inv = 0.7071067811865475;  // Util::SQRT2_INV (src/util.h:60)
    for (size_t i = 0; i < n; i++)  // base_system.h:108-123
      if (up[i] < dn[i]) {
        for (auto& v : cs) {
          const double h = v[i] * kSqrt2Inv;
          v[i] = h;
          v.push_back(h);
        }
        up.push_back(dn[i]);
        dn.push_back(up[i]);
      }
    c->time_sym = false;
    const shci_status st = shci_set_dets(c, up.data(), dn.data(), cs[0].data(), up.size());
    if (st != SHCI_OK) throw ArgError(c->err);
    for (unsigned k = 1; k < ns; k++) {
      const shci_status sk = shci_set_state_coefs(c, k, cs[k].data(), up.size());
      if (sk != SHCI_OK) throw ArgError(c->err);
    }
  });
}

shci_status shci_get_state_coefs(shci_ctx* c, unsigned state, double* coefs, size_t cap) {
  if (!c || !coefs) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_dets(c);
    if (state >= c->n_states) throw ArgError("state index >= n_states");
    const size_t n = c->up.size();
    if (cap < n) throw ArgError("coefficient buffer too small");
    sync_dets(c);
    SHCI_CUDA(cudaMemcpyAsync(coefs, state_coef(c, state), n * 8, cudaMemcpyDeviceToHost,
                              c->stream));
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
  });
}

shci_status shci_set_state_coefs(shci_ctx* c, unsigned state, const double* coefs, size_t n) {
  if (!c || !coefs) return SHCI_ERR_ARG;
  if (state == 0) return shci_set_coefs(c, coefs, n);
  return guard(c, [&]() {
    need_dets(c);
    if (state >= c->n_states) throw ArgError("state index >= n_states");
    if (n != c->up.size()) throw ArgError("coefficient count != det count");
    SHCI_CUDA(cudaMemcpyAsync(state_coef(c, state), coefs, n * 8, cudaMemcpyHostToDevice,
                              c->stream));
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
    c->dav.ritz = false;
  });
}

shci_status shci_get_state_energies(shci_ctx* c, double* energies, size_t cap) {
  if (!c || !energies) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    for (size_t k = 0; k < c->n_states && k < cap; k++)
      energies[k] = k < c->state_energy.size() ? c->state_energy[k] : 0.0;
  });
}

shci_status shci_set_coefs_dev(shci_ctx* c, const double* coefs_dev, size_t n) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (n != c->up.size() || !coefs_dev) throw ArgError("coefficient count != det count");
    sync_dets(c);
    SHCI_CUDA(cudaMemcpyAsync(c->d_coef.p, coefs_dev, n * 8, cudaMemcpyDeviceToDevice, c->stream));
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
  });
}

shci_status shci_get_n_dets(shci_ctx* c, size_t* n) {
  if (!c || !n) return SHCI_ERR_ARG;
  *n = c->up.size();
  return SHCI_OK;
}

shci_status shci_get_dets(shci_ctx* c, uint64_t* up, uint64_t* dn, double* coefs, size_t cap) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    const size_t n = c->up.size();
    if (cap < n) throw ArgError("buffer too small for " + std::to_string(n) + " dets");
    if (up) std::memcpy(up, c->up.data(), n * 8);
    if (dn) std::memcpy(dn, c->dn.data(), n * 8);
    if (coefs) {
      sync_dets(c);
      SHCI_CUDA(cudaMemcpyAsync(coefs, c->d_coef.p, n * 8, cudaMemcpyDeviceToHost, c->stream));
      SHCI_CUDA(cudaStreamSynchronize(c->stream));
    }
  });
}

shci_status shci_set_coefs(shci_ctx* c, const double* coefs, size_t n) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (n != c->up.size() || !coefs) throw ArgError("coefficient count != det count");
    sync_dets(c);
    SHCI_CUDA(cudaMemcpyAsync(c->d_coef.p, coefs, n * 8, cudaMemcpyHostToDevice, c->stream));
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
  });
}

shci_status shci_hamiltonian_elems(shci_ctx* c, const uint64_t* ui, const uint64_t* di,
                                   const uint64_t* uj, const uint64_t* dj, size_t n, double* out) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    hamiltonian_elems(c, ui, di, uj, dj, n, out);
  });
}

shci_status shci_hamiltonian_elems_noalloc(shci_ctx* c, const uint64_t* ui, const uint64_t* di,
                                           const uint64_t* uj, const uint64_t* dj, size_t n,
                                           double* out) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    hamiltonian_elems_noalloc(c, ui, di, uj, dj, n, out);
  });
}

shci_status shci_update_hamiltonian(shci_ctx* c, int precision, size_t* nnz_out) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    if (precision != SHCI_PREC_FP64 && precision != SHCI_PREC_MIXED)
      throw ArgError("unknown precision");
    sync_dets(c);
    const size_t nnz = build_hamiltonian(c, precision);
    if (nnz_out) {
      nnz_out[0] = nnz;
      nnz_out[1] = 2 * (nnz + c->up.size()) - c->up.size();
    }
  });
}

shci_status shci_hamiltonian_stats(shci_ctx* c, uint64_t* stats) {
  if (!c || !stats) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (!c->H.valid) throw ArgError("no Hamiltonian built");
    const bool scan = !c->H.join;
    uint32_t n_as = 0;
    if (scan && c->idx.n_alpha)
      SHCI_CUDA(cudaMemcpy(&n_as, c->idx.as_off.p + c->idx.n_alpha, 4, cudaMemcpyDeviceToHost));
    stats[0] = c->H.n;
    stats[1] = c->H.nnz;
    stats[2] = scan ? c->idx.n_alpha : 0;
    stats[3] = scan ? c->idx.n_beta : 0;
    stats[4] = n_as;
    stats[5] = c->H.candidates;
    for (int k = 0; k < 3; k++) stats[6 + k] = c->H.cand_parts[k];
    if (c->H.join) stats[7] = c->H.packed ? 0 : 1;  // 1: single pass, rows sized by a bound
    stats[9] = c->H.join ? 1 : 0;
  });
}

shci_status shci_memory_stats(shci_ctx* c, size_t* out) {
  if (!c || !out) return SHCI_ERR_ARG;
  out[0] = c->mem.used;
  out[1] = c->mem.peak;
  out[2] = c->mem.budget;
  out[3] = c->mem.cached;
  out[4] = c->mem.peak_live;
  return SHCI_OK;
}

shci_status shci_get_hamiltonian(shci_ctx* c, uint64_t* row_ptr, uint32_t* cols, double* vals,
                                 double* diag) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    auto& H = c->H;
    if (!H.valid) throw ArgError("no Hamiltonian built");
    cudaStream_t s = c->stream;
    const size_t n = H.n, nnz = H.nnz;
    if (!H.older.empty()) {
      // several segments (incremental updates): each row merged, in increasing column order
      std::vector<uint64_t> all(n), off(n + 1);
      for (size_t i = 0; i < n; i++) all[i] = i;
      get_rows(c, all.data(), n, off.data(), cols, vals);
      if (row_ptr) std::memcpy(row_ptr, off.data(), (n + 1) * 8);
      if (diag) SHCI_CUDA(cudaMemcpyAsync(diag, H.diag.p, n * 8, cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
      return;
    }
    if (!H.packed) {
      // rows sized by an upper bound: hand out a packed copy, made on the device when there is
      // room for it and on the host otherwise (no device memory needed)
      DevBuf<uint64_t> p;
      DevBuf<uint32_t> cl;
      DevBuf<double> v;
      p.mt = &c->mem;
      cl.mt = &c->mem;
      v.mt = &c->mem;
      try {
        pack_hamiltonian(c, p, cl, v);
      } catch (const OomError&) {
        p.release();
        cl.release();
        v.release();
        std::vector<uint64_t> rp(n + 1);
        std::vector<uint32_t> rc(n);
        const size_t cap = H.col.cap;
        std::vector<uint32_t> hc(cap);
        std::vector<double> hv;
        std::vector<float> h32, r32;
        SHCI_CUDA(cudaMemcpyAsync(rp.data(), H.row_ptr.p, (n + 1) * 8, cudaMemcpyDeviceToHost, s));
        SHCI_CUDA(cudaMemcpyAsync(rc.data(), H.row_cnt.p, n * 4, cudaMemcpyDeviceToHost, s));
        SHCI_CUDA(cudaMemcpyAsync(hc.data(), H.col.p, cap * 4, cudaMemcpyDeviceToHost, s));
        const bool fp64 = H.precision == SHCI_PREC_FP64;
        if (vals) {
          if (fp64) {
            hv.resize(cap);
            SHCI_CUDA(cudaMemcpyAsync(hv.data(), H.val64.p, cap * 8, cudaMemcpyDeviceToHost, s));
          } else {
            h32.resize(cap);
            r32.resize(cap);
            SHCI_CUDA(cudaMemcpyAsync(h32.data(), H.val32.p, cap * 4, cudaMemcpyDeviceToHost, s));
            SHCI_CUDA(cudaMemcpyAsync(r32.data(), H.res32.p, cap * 4, cudaMemcpyDeviceToHost, s));
          }
        }
        if (diag) SHCI_CUDA(cudaMemcpyAsync(diag, H.diag.p, n * 8, cudaMemcpyDeviceToHost, s));
        SHCI_CUDA(cudaStreamSynchronize(s));
        uint64_t pos = 0;
        for (size_t i = 0; i < n; i++) {
          if (row_ptr) row_ptr[i] = pos;
          for (uint32_t k = 0; k < rc[i]; k++) {
            const uint64_t src = rp[i] + k;
            if (cols) cols[pos] = hc[src];
            if (vals) vals[pos] = fp64 ? hv[src] : (double)h32[src] + (double)r32[src];
            pos++;
          }
        }
        if (row_ptr) row_ptr[n] = pos;
        return;
      }
      if (row_ptr) SHCI_CUDA(cudaMemcpyAsync(row_ptr, p.p, (n + 1) * 8, cudaMemcpyDeviceToHost, s));
      if (cols) SHCI_CUDA(cudaMemcpyAsync(cols, cl.p, nnz * 4, cudaMemcpyDeviceToHost, s));
      if (vals) SHCI_CUDA(cudaMemcpyAsync(vals, v.p, nnz * 8, cudaMemcpyDeviceToHost, s));
      if (diag) SHCI_CUDA(cudaMemcpyAsync(diag, H.diag.p, n * 8, cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
      return;
    }
    if (row_ptr) SHCI_CUDA(cudaMemcpyAsync(row_ptr, H.row_ptr.p, (n + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (cols) SHCI_CUDA(cudaMemcpyAsync(cols, H.col.p, nnz * 4, cudaMemcpyDeviceToHost, s));
    if (diag) SHCI_CUDA(cudaMemcpyAsync(diag, H.diag.p, n * 8, cudaMemcpyDeviceToHost, s));
    if (vals) {
      if (H.precision == SHCI_PREC_FP64) {
        SHCI_CUDA(cudaMemcpyAsync(vals, H.val64.p, nnz * 8, cudaMemcpyDeviceToHost, s));
      } else {
        std::vector<float> hi(nnz), lo(nnz);
        SHCI_CUDA(cudaMemcpyAsync(hi.data(), H.val32.p, nnz * 4, cudaMemcpyDeviceToHost, s));
        SHCI_CUDA(cudaMemcpyAsync(lo.data(), H.res32.p, nnz * 4, cudaMemcpyDeviceToHost, s));
        SHCI_CUDA(cudaStreamSynchronize(s));
        for (size_t k = 0; k < nnz; k++) vals[k] = (double)hi[k] + (double)lo[k];
      }
    }
    SHCI_CUDA(cudaStreamSynchronize(s));
  });
}

shci_status shci_get_hamiltonian_rows(shci_ctx* c, const uint64_t* rows, size_t n_rows,
                                      uint64_t* offsets, uint32_t* cols, double* vals) {
  if (!c || !offsets || (n_rows && !rows)) return SHCI_ERR_ARG;
  return guard(c, [&]() { get_rows(c, rows, n_rows, offsets, cols, vals); });
}

shci_status shci_hv(shci_ctx* c, const double* x_dev, double* y_dev, int use_residual) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() { spmv(c, x_dev, y_dev, use_residual != 0); });
}

shci_status shci_hv_host(shci_ctx* c, const double* x, double* y, int use_residual) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    const size_t n = c->H.n;
    if (!c->H.valid) throw ArgError("no Hamiltonian built");
    c->f0.resize(n, 1.1);
    c->f1.resize(n, 1.1);
    SHCI_CUDA(cudaMemcpyAsync(c->f0.p, x, n * 8, cudaMemcpyHostToDevice, c->stream));
    spmv(c, c->f0.p, c->f1.p, use_residual != 0);
    SHCI_CUDA(cudaMemcpyAsync(y, c->f1.p, n * 8, cudaMemcpyDeviceToHost, c->stream));
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
  });
}

shci_status shci_davidson(shci_ctx* c, double tol, double* eval, int* converged, double* trace,
                          size_t trace_cap, size_t* n_trace) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (!c->H.valid || c->H.n != c->up.size()) throw ArgError("Hamiltonian not up to date");
    sync_dets(c);
    auto r = davidson(c, tol);
    if (eval) *eval = r.eval;
    if (converged) *converged = r.converged ? 1 : 0;
    if (trace)
      for (size_t i = 0; i < r.trace.size() && i < trace_cap; i++) trace[i] = r.trace[i];
    if (n_trace) *n_trace = r.trace.size();
  });
}

shci_status shci_energy_fp64(shci_ctx* c, double* energy) {
  if (!c || !energy) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (!c->H.valid) throw ArgError("no Hamiltonian built");
    *energy = rayleigh_fp64(c);
  });
}


shci_status shci_davidson_csr(shci_ctx* c, size_t n, const uint64_t* row_ptr,
                              const uint32_t* cols, const double* vals, const double* diag,
                              const double* init, double tol, double* eval, double* evec,
                              int* converged) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    cudaStream_t s = c->stream;
    load_csr(c, n, row_ptr, cols, vals, diag);
    c->d_coef.resize(n);
    SHCI_CUDA(cudaMemcpyAsync(c->d_coef.p, init, n * 8, cudaMemcpyHostToDevice, s));
    const unsigned ns = c->n_states;
    c->n_states = 1;
    DavidsonOut r;
    try {
      r = davidson(c, tol);
    } catch (...) {
      c->n_states = ns;
      drop_csr(c);
      throw;
    }
    c->n_states = ns;
    SHCI_CUDA(cudaMemcpyAsync(evec, c->d_coef.p, n * 8, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    *eval = r.eval;
    if (converged) *converged = r.converged ? 1 : 0;
    drop_csr(c);
  });
}

shci_status shci_davidson_csr_states(shci_ctx* c, size_t n, const uint64_t* row_ptr,
                                     const uint32_t* cols, const double* vals,
                                     const double* diag, unsigned n_states, const double* init,
                                     double tol, double* evals, double* evecs, int* converged) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (n_states < 1 || n_states > kMaxStates)
      throw ArgError("n_states must be in [1, " + std::to_string(kMaxStates) + "]");
    if (!init || !evals || !evecs || n == 0) throw ArgError("null or empty argument");
    cudaStream_t s = c->stream;
    load_csr(c, n, row_ptr, cols, vals, diag);
    const unsigned ns_ctx = c->n_states;
    c->n_states = n_states;
    auto restore = [&]() {
      c->n_states = ns_ctx;
      drop_csr(c);
      if (!c->up.empty()) reset_states(c, c->up.size());
    };
    try {
      for (unsigned k = 0; k < n_states; k++) {
        auto& b = k == 0 ? c->d_coef : c->d_xcoef[k - 1];
        b.mt = &c->mem;
        b.resize(n, 1.1);
        SHCI_CUDA(cudaMemcpyAsync(b.p, init + k * n, n * 8, cudaMemcpyHostToDevice, s));
      }
      DavidsonStatesOut r;
      if (n_states == 1) {
        DavidsonOut r1 = davidson(c, tol);
        r.evals.assign(1, r1.eval);
        r.converged = r1.converged;
      } else {
        r = davidson_states(c, tol);
      }
      for (unsigned k = 0; k < n_states; k++) {
        SHCI_CUDA(cudaMemcpyAsync(evecs + k * n, state_coef(c, k), n * 8, cudaMemcpyDeviceToHost,
                                  s));
        evals[k] = r.evals[k];
      }
      SHCI_CUDA(cudaStreamSynchronize(s));
      if (converged) *converged = r.converged ? 1 : 0;
    } catch (...) {
      restore();
      throw;
    }
    restore();
  });
}

shci_status shci_select(shci_ctx* c, double eps_var, int var_sd, size_t* n_new) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    const size_t k = select_dets(c, eps_var, var_sd != 0);
    if (n_new) *n_new = k;
    c->H.valid = false;
    c->H.build_id++;
  });
}

shci_status shci_set_second_rejection(shci_ctx* c, int enable, double factor) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (!(factor >= 0.0)) throw ArgError("second_rejection_factor must be >= 0");
    c->second_rejection = enable != 0;
    c->second_rejection_factor = factor;
  });
}

shci_status shci_set_has_double_excitation(shci_ctx* c, int on) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    c->has_doubles = on != 0;
    apply_excitation_flags(c);
    c->H.valid = false;
    c->H.prefix_ok = false;
    c->H.build_id++;
    c->eps_tried.clear();
  });
}

shci_status shci_set_active_space(shci_ctx* c, const unsigned* irrep_active_space, size_t n) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    if (n == 0) {
      c->inactive_orbs = 0;
    } else {
      if (!irrep_active_space) throw ArgError("null irrep_active_space");
      try {
        c->inactive_orbs = inactive_orbitals(
            c->I, std::vector<unsigned>(irrep_active_space, irrep_active_space + n));
      } catch (const std::invalid_argument& e) {
        throw ArgError(e.what());
      }
    }
    c->eps_tried.clear();
  });
}

shci_status shci_get_inactive_orbitals(shci_ctx* c, uint64_t* mask) {
  if (!c || !mask) return SHCI_ERR_ARG;
  return guard(c, [&]() { *mask = c->inactive_orbs; });
}

shci_status shci_set_var_sd(shci_ctx* c, int on) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() { c->var_sd = on != 0; });
}

shci_status shci_set_hf_options(shci_ctx* c, int allow_doubly_occupy, const unsigned* irreps,
                                const unsigned* irrep_occs_up, const unsigned* irrep_occs_dn,
                                size_t n_irreps) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (n_irreps && (!irreps || !irrep_occs_up || !irrep_occs_dn))
      throw ArgError("null irrep array");
    HfOptions o;
    o.allow_doubly_occupy = allow_doubly_occupy != 0;
    if (n_irreps) {
      o.irreps.assign(irreps, irreps + n_irreps);
      o.irrep_occs_up.assign(irrep_occs_up, irrep_occs_up + n_irreps);
      o.irrep_occs_dn.assign(irrep_occs_dn, irrep_occs_dn + n_irreps);
    }
    c->hf_opts = o;
  });
}

shci_status shci_natural_orbitals(shci_ctx* c, double* rot, double* occ) {
  if (!c || !rot || !occ) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    std::vector<double> g1((size_t)c->I.n * c->I.n);
    const shci_status st = shci_rdm1(c, g1.data());
    if (st != SHCI_OK) throw std::runtime_error(c->err);
    natural_orbitals(c, g1.data(), rot, occ);
  });
}

shci_status shci_rotate_integrals(shci_ctx* c, const double* rot) {
  if (!c || !rot) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    const size_t n = c->I.n;
    for (size_t p = 0; p < n; p++)
      for (size_t q = 0; q < n; q++) {
        double d = 0.0;
        for (size_t i = 0; i < n; i++) d += rot[i * n + p] * rot[i * n + q];
        if (std::fabs(d - (p == q ? 1.0 : 0.0)) > 1e-8)
          throw ArgError("rotation matrix is not orthogonal");
        // the orbital symmetry labels stay valid only for rotations within each irrep
        if (c->I.orb_sym[p] != c->I.orb_sym[q] && std::fabs(rot[p * n + q]) > 1e-12)
          throw ArgError("rotation matrix mixes orbitals of different irreps");
      }
    rotate_integrals(c, rot);
    after_integrals(c);
  });
}

shci_status shci_get_s2(shci_ctx* c, double* s2) {
  if (!c || !s2) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    if (c->time_sym)
      throw ArgError("S^2 needs the unpacked wavefunction (shci_unpack_time_sym first)");
    *s2 = get_s2(c);
  });
}

shci_status shci_get_eps_tried(shci_ctx* c, double* out, size_t cap) {
  if (!c || !out) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    if (cap < c->eps_tried.size()) throw ArgError("buffer too small");
    std::memcpy(out, c->eps_tried.data(), c->eps_tried.size() * 8);
  });
}

shci_status shci_run_variation(shci_ctx* c, const double* eps_vars, size_t n_eps,
                               const double* schedule, size_t n_sched, double target_error,
                               int precision, double* energies) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    if (!eps_vars || n_eps == 0) throw ArgError("no eps_vars");
    std::vector<double> ev(eps_vars, eps_vars + n_eps);
    std::vector<double> sc;
    if (schedule) sc.assign(schedule, schedule + n_sched);
    c->var_trace.clear();
    auto e = run_all_variations(c, ev, sc, target_error, precision, c->var_sd, &c->var_trace);
    if (energies)
      for (size_t i = 0; i < e.size(); i++) energies[i] = e[i];
  });
}

shci_status shci_get_launch_count(shci_ctx* c, uint64_t* n) {
  if (!c || !n) return SHCI_ERR_ARG;
  *n = c->launches;
  return SHCI_OK;
}

shci_status shci_profile(shci_ctx* c, int enable) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
    c->prof.reset();
    c->prof.on = enable != 0;
  });
}

shci_status shci_profile_get(shci_ctx* c, char* names, double* total_ms, uint64_t* count,
                             size_t cap, size_t* n) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    SHCI_CUDA(cudaStreamSynchronize(c->stream));
    c->prof.flush();
    size_t k = 0;
    for (const auto& kv : c->prof.acc) {
      if (k < cap) {
        if (names) {
          std::memset(names + 32 * k, 0, 32);
          std::strncpy(names + 32 * k, kv.first.c_str(), 31);
        }
        if (total_ms) total_ms[k] = kv.second.first;
        if (count) count[k] = kv.second.second;
      }
      k++;
    }
    if (n) *n = k;
  });
}

shci_status shci_get_var_trace(shci_ctx* c, uint64_t* n_dets, uint64_t* nnz, double* energy,
                               size_t cap, size_t* n) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    const auto& t = c->var_trace;
    if (n) *n = t.size();
    for (size_t i = 0; i < t.size() && i < cap; i++) {
      if (n_dets) n_dets[i] = t[i].n_dets;
      if (nnz) nnz[i] = t[i].nnz_sym;
      if (energy) energy[i] = t[i].energy;
    }
  });
}

shci_status shci_get_var_trace_states(shci_ctx* c, double* energies, size_t cap, size_t* n) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    const auto& t = c->var_trace;
    const size_t ns = c->n_states;
    if (n) *n = t.size();
    if (!energies) return;
    for (size_t i = 0; i < t.size() && (i + 1) * ns <= cap; i++)
      for (size_t k = 0; k < ns; k++)
        energies[i * ns + k] =
            k < t[i].energies.size() ? t[i].energies[k] : (k == 0 ? t[i].energy : 0.0);
  });
}

shci_status shci_pt2_dtm(shci_ctx* c, double energy_var, double eps_pt_dtm, size_t n_batches,
                         double* correction, double* uncert, size_t* n_pt_dets) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    auto r = pt2_dtm(c, energy_var, eps_pt_dtm, n_batches);
    if (correction) *correction = r.value;
    if (uncert) *uncert = r.uncert;
    if (n_pt_dets) *n_pt_dets = r.n_pt_dets;
  });
}

shci_status shci_mapreduce_sum(shci_ctx* c, const double* x, size_t n, double* out) {
  if (!c || !out || (n && !x)) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    out[0] = out[1] = 0.0;
    if (n == 0) return;
    cudaStream_t s = c->stream;
    DevBuf<double> dx, res;
    DevBuf<uint64_t> starts;
    dx.mt = res.mt = &c->mem;
    starts.mt = &c->mem;
    dx.resize(n);
    res.resize(2);
    starts.resize(2);
    const uint64_t st[2] = {0, n};
    SHCI_CUDA(cudaMemcpyAsync(dx.p, x, n * 8, cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(starts.p, st, 16, cudaMemcpyHostToDevice, s));
    seg_reduce2(c, dx.p, starts.p, 1, n, res.p);
    SHCI_CUDA(cudaMemcpyAsync(out, res.p, 16, cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
  });
}

shci_status shci_find_connected_dets(shci_ctx* c, const uint64_t* up, const uint64_t* dn,
                                     const double* eps_max, const double* eps_min, size_t n,
                                     uint64_t* offsets, uint64_t* out_up, uint64_t* out_dn,
                                     uint8_t* n_excite) {
  if (!c || !offsets) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    find_connected(c, up, dn, eps_max, eps_min, n, offsets, out_up, out_dn, n_excite);
  });
}

shci_status shci_rdm1(shci_ctx* c, double* out) {
  if (!c || !out) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    if (c->n_states == 1) {
      rdm1(c, out);
      return;
    }
    // rdm.cc:222-231: the sum over the states of c_i c_j, formed state by state
    const size_t nn = static_cast<size_t>(c->I.n) * c->I.n;
    std::vector<double> acc(nn, 0.0), t(nn);
    sync_dets(c);
    for (unsigned k = 0; k < c->n_states; k++) {
      if (k) c->d_coef.swap(c->d_xcoef[k - 1]);
      rdm1(c, t.data());
      if (k) c->d_coef.swap(c->d_xcoef[k - 1]);
      for (size_t i = 0; i < nn; i++) acc[i] += t[i];
    }
    std::memcpy(out, acc.data(), nn * 8);
  });
}

shci_status shci_rdm2(shci_ctx* c, double* out_half) {
  if (!c || !out_half) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    if (c->n_states == 1) {
      rdm2(c, out_half);
      return;
    }
    const size_t nn = static_cast<size_t>(c->I.n) * c->I.n, m = nn * (nn + 1) / 2;
    std::vector<double> acc(m, 0.0), t(m);
    sync_dets(c);
    for (unsigned k = 0; k < c->n_states; k++) {  // rdm.cc:648-657, state by state
      if (k) c->d_coef.swap(c->d_xcoef[k - 1]);
      rdm2(c, t.data());
      if (k) c->d_coef.swap(c->d_xcoef[k - 1]);
      for (size_t i = 0; i < m; i++) acc[i] += t[i];
    }
    std::memcpy(out_half, acc.data(), m * 8);
  });
}

shci_status shci_generalized_fock(shci_ctx* c, double* F) {
  if (!c || !F) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    sync_dets(c);
    if (!c->H.valid || c->H.n != c->up.size()) build_hamiltonian(c, SHCI_PREC_FP64);
    generalized_fock(c, F);
  });
}

shci_status shci_orbital_parameters(shci_ctx* c, uint32_t* p, uint32_t* q, size_t cap,
                                    size_t* n) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    const auto& sym = c->I.orb_sym;
    size_t k = 0;
    for (unsigned i = 0; i < c->I.n; i++)
      for (unsigned j = i + 1; j < c->I.n; j++)
        if (sym[i] == sym[j]) {
          if (k < cap && p && q) {
            p[k] = i;
            q[k] = j;
          }
          k++;
        }
    if (n) *n = k;
  });
}

shci_status shci_orbital_gradient(shci_ctx* c, const uint32_t* p, const uint32_t* q,
                                  size_t n_param, double* grad) {
  if (!c || (n_param && (!p || !q || !grad))) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    const size_t n = c->I.n;
    for (size_t k = 0; k < n_param; k++)
      if (p[k] >= n || q[k] >= n) throw ArgError("orbital index out of range");
    std::vector<double> F(n * n);
    sync_dets(c);
    if (!c->H.valid || c->H.n != c->up.size()) build_hamiltonian(c, SHCI_PREC_FP64);
    generalized_fock(c, F.data());
    for (size_t k = 0; k < n_param; k++)  // optimization.cc:571-575
      grad[k] = 2 * (F[p[k] * n + q[k]] - F[q[k] * n + p[k]]);
  });
}

shci_status shci_orbital_hessian_diagonal(shci_ctx* c, const uint32_t* p, const uint32_t* q,
                                          size_t n_param, double* hdiag) {
  if (!c || (n_param && (!p || !q || !hdiag))) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    const size_t n = c->I.n;
    for (size_t k = 0; k < n_param; k++)
      if (p[k] >= n || q[k] >= n || p[k] == q[k]) throw ArgError("bad orbital pair");
    sync_dets(c);
    if (!c->H.valid || c->H.n != c->up.size()) build_hamiltonian(c, SHCI_PREC_FP64);
    orbital_hessian_diagonal(c, p, q, n_param, hdiag);
  });
}

shci_status shci_orbital_rotation(shci_ctx* c, const uint32_t* p, const uint32_t* q,
                                  const double* kappa, size_t n_param, double* rot) {
  if (!c || !rot || (n_param && (!p || !q || !kappa))) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    const size_t n = c->I.n;
    for (size_t k = 0; k < n_param; k++)
      if (p[k] >= n || q[k] >= n || p[k] == q[k]) throw ArgError("bad orbital pair");
    rotation_from_parameters(static_cast<int>(n), p, q, kappa, n_param, rot);
  });
}

shci_status shci_pt2_psto(shci_ctx* c, double energy_var, double eps_pt_dtm, double eps_pt_psto,
                          size_t n_batches, double target_error, double eps_pt,
                          double* correction, double* uncert, size_t* n_pt_dets,
                          size_t* n_batches_done) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    auto r = pt2_psto(c, energy_var, eps_pt_dtm, eps_pt_psto, n_batches, target_error, eps_pt);
    if (correction) *correction = r.value;
    if (uncert) *uncert = r.uncert;
    if (n_pt_dets) *n_pt_dets = r.n_pt_dets;
    if (n_batches_done) *n_batches_done = r.n_batches_done;
  });
}

shci_status shci_pt2_psto_auto_batches(shci_ctx* c, double eps_pt_psto, double pt_mem_avail,
                                       double mem_usage, size_t* n_batches, size_t* n_pilot) {
  if (!c || !n_batches) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    if (!(pt_mem_avail >= 1.0) || !(mem_usage > 0.0))
      throw ArgError("pt_mem_avail and mem_usage must be positive");
    size_t np = 0;
    *n_batches = psto_auto_batches(c, eps_pt_psto, pt_mem_avail, mem_usage, &np);
    if (n_pilot) *n_pilot = np;
  });
}

shci_status shci_pt2_sto(shci_ctx* c, double energy_var, double eps_pt_psto, double eps_pt,
                         size_t n_batches, size_t n_dets_in_sample, int semisto,
                         unsigned random_seed, size_t max_iterations, double target_error,
                         double psto_uncert, double pt_mem_avail, double mem_usage,
                         double* correction, double* uncert, size_t* n_iterations,
                         size_t* sample_info, double* loops, size_t cap) {
  if (!c) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    need_dets(c);
    std::vector<double> lv;
    size_t info[3] = {0, 0, 0};
    auto r = pt2_sto(c, energy_var, eps_pt_psto, eps_pt, n_batches, n_dets_in_sample,
                     semisto != 0, random_seed, max_iterations, target_error, psto_uncert,
                     pt_mem_avail, mem_usage, &lv, info);
    if (correction) *correction = r.value;
    if (uncert) *uncert = r.uncert;
    if (n_iterations) *n_iterations = r.n_batches_done;
    if (sample_info)
      for (int k = 0; k < 3; k++) sample_info[k] = info[k];
    if (loops)
      for (size_t k = 0; k < lv.size() && k < cap; k++) loops[k] = lv[k];
  });
}

shci_status shci_pt_mem_avail(shci_ctx* c, double mem_total, double* out) {
  if (!c || !out) return SHCI_ERR_ARG;
  return guard(c, [&]() {
    need_integrals(c);
    if (!c->Q.built) throw ArgError("heat-bath queues not built (call shci_build_queues)");
    // solver.h:601-611 with one process: bytes per det = two 64-bit chunks per spin (32 B),
    // helper size = 32 B per heat-bath queue entry (chem_system.cc:112, 195)
    const size_t mt = static_cast<size_t>(mem_total);
    const size_t mem_var = c->up.size() * (32 * 3 + 8);
    const size_t helper = 32 * (c->Q.n_hci + c->Q.n_singles);
    const double left = static_cast<double>(mt) * 0.7 - static_cast<double>(mem_var) -
                        static_cast<double>(helper);
    if (!(left > 0)) throw ArgError("mem_total leaves no memory for PT2");
    *out = static_cast<double>(static_cast<size_t>(left));
  });
}

}  // extern "C"

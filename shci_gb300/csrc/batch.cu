// Batched solves of many small SHCI instances (variation + PT2 each) on one GPU.
//
// Each instance alone is latency bound: a few thousand dets, hundreds of short kernels and
// host round trips per solve.  The batch runner keeps the GPU busy by solving instances
// concurrently: W worker threads, each owning one context (its own stream and device
// buffers), pull instances from a shared queue ordered largest first, so the kernels and
// copies of different instances overlap.  The worker count is chosen by a small autotuner
// when the caller passes n_workers <= 0: on a long queue it solves interleaved slices with a
// quarter, a half and one worker per host CPU, measures instances per second on each, and
// finishes the queue with the fastest; a short queue takes one worker per two host CPUs.  An instance's results do not depend on W.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>

#include "ctx.h"
#include "kernels.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void solve_one(shci_ctx* c, const shci_batch_item& it, shci_batch_result& r) {
  const double t0 = now_s();
  r = shci_batch_result{};
  shci_status st = shci_load_fcidump(c, it.fcidump, it.n_up, it.n_dn,
                                     it.point_group ? it.point_group : "C1", -1, nullptr, nullptr);
  if (st == SHCI_OK) st = shci_get_hf(c, nullptr, nullptr, &r.energy_hf);
  if (st == SHCI_OK) st = shci_build_queues(c, nullptr);
  std::vector<double> e(it.n_eps > 0 ? it.n_eps : 1);
  if (st == SHCI_OK)
    st = shci_run_variation(c, it.eps_vars, it.n_eps, it.schedule, it.n_sched, it.target_error,
                            it.precision, e.data());
  if (st == SHCI_OK) {
    r.energy_var = e[it.n_eps - 1];
    size_t n = 0;
    shci_get_n_dets(c, &n);
    r.n_dets = n;
  }
  if (st == SHCI_OK && it.eps_pt_dtm > 0.0) {
    double dtm = 0.0, u = 0.0;
    size_t npt = 0;
    st = shci_pt2_dtm(c, r.energy_var, it.eps_pt_dtm, 1, &dtm, &u, &npt);
    r.correction_pt = dtm;
    r.n_pt_dets = npt;
    double unc = 0.0;
    if (st == SHCI_OK && it.eps_pt_psto > 0.0 && it.eps_pt_psto < it.eps_pt_dtm) {
      double ps = 0.0, up = 0.0;
      size_t n1 = 0, nb = 0;
      st = shci_pt2_psto(c, r.energy_var, it.eps_pt_dtm, it.eps_pt_psto, 16, it.target_error,
                         it.eps_pt, &ps, &up, &n1, &nb);
      r.correction_pt += ps;
      unc = up;
    }
    r.uncert_pt = unc;
  }
  r.status = st;
  r.seconds = now_s() - t0;
}

// Rough cost of an instance: the size of its determinant space, C(n, n_up) C(n, n_dn).
double instance_cost(const shci_batch_item& it, int n_orbs) {
  auto lc = [](int n, int k) {
    return std::lgamma(n + 1.0) - std::lgamma(k + 1.0) - std::lgamma(n - k + 1.0);
  };
  return lc(n_orbs, it.n_up) + lc(n_orbs, it.n_dn);
}

int fcidump_norb(const char* path) {
  FILE* f = std::fopen(path, "r");
  if (!f) return 0;
  char buf[4096];
  int n = 0;
  while (std::fgets(buf, sizeof(buf), f)) {
    const char* p = std::strstr(buf, "NORB");
    if (p) {
      p += 4;
      while (*p && (*p == 'S' || *p == '=' || *p == ' ')) p++;
      n = std::atoi(p);
      break;
    }
  }
  std::fclose(f);
  return n;
}

// Runs the items idx[...] with W workers; returns elapsed seconds.  Each worker's host-side
// loops (integral loading, PT2 sampling) use its share of the host CPUs.
double run_slice(int device, const shci_batch_item* items, const std::vector<size_t>& idx, int W,
                 shci_batch_result* out, std::atomic<int>& create_fail) {
  std::atomic<size_t> next{0};
  const double t0 = now_s();
  const unsigned share = std::max(1u, shci::host_threads() / static_cast<unsigned>(W));
  std::vector<std::thread> th;
  for (int w = 0; w < W; w++)
    th.emplace_back([&]() {
      shci::set_host_threads(share);
      shci_ctx* c = nullptr;
      if (shci_create(&c, device, 0) != SHCI_OK) {
        create_fail++;
        return;
      }
      // the workers share the device: each keeps a cache of released blocks of at most its
      // share of a quarter of the device (a worker's failing allocation returns only its own)
      size_t f = 0, t = 0;
      if (cudaMemGetInfo(&f, &t) == cudaSuccess) c->mem.cache_cap = std::max<size_t>(t / 4 / W, 1);
      for (size_t k; (k = next.fetch_add(1)) < idx.size();) solve_one(c, items[idx[k]], out[idx[k]]);
      shci_destroy(c);
    });
  for (auto& t : th) t.join();
  return now_s() - t0;
}

}  // namespace

extern "C" shci_status shci_batch_solve(int device, const shci_batch_item* items, size_t n,
                                        int n_workers, shci_batch_result* out, int* workers_used) {
  if (!items || !out) return SHCI_ERR_ARG;
  if (n == 0) return SHCI_OK;
  // largest instances first
  std::vector<size_t> order(n);
  std::vector<double> cost(n);
  for (size_t k = 0; k < n; k++) {
    order[k] = k;
    cost[k] = instance_cost(items[k], fcidump_norb(items[k].fcidump));
  }
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
  std::atomic<int> create_fail{0};
  int W = n_workers;
  size_t done = 0;
  if (W <= 0) {
    // Each solve is host-latency bound (launches, synchronisations, host-side sampling), so
    // the useful worker count is set by the host CPUs; beyond about one worker per two CPUs
    // the workers contend for the GPU and the driver and the rate falls.
    // Candidates: a quarter, a half and one worker per CPU.  The first n_cand * L items of
    // the queue are dealt round robin to the candidates, so each candidate's slice spans the
    // same range of sizes; the one with the highest rate solves the rest.  A slice's time is
    // set by its largest instances as much as by the rate, so the tuner runs only on queues
    // at least four times as long as the slices; shorter ones take a worker per two CPUs.
    const int cpus = static_cast<int>(shci::host_threads());
    std::vector<int> cand;
    for (int w : {cpus / 4, cpus / 2, cpus}) {
      w = std::min(std::max(w, 1), 64);
      if (cand.empty() || cand.back() != w) cand.push_back(w);
    }
    const size_t nc = cand.size();
    const size_t L = 2 * static_cast<size_t>(cand.back());
    W = std::min(std::max(cpus / 2, 1), 64);
    if (nc > 1 && 4 * nc * L <= n) {
      double best_rate = 0.0;
      for (size_t j = 0; j < nc; j++) {
        std::vector<size_t> idx;
        for (size_t k = j; k < nc * L; k += nc) idx.push_back(order[k]);
        const double t = run_slice(device, items, idx, cand[j], out, create_fail);
        const double rate = idx.size() / std::max(t, 1e-9);
        if (rate > best_rate) {
          best_rate = rate;
          W = cand[j];
        }
      }
      done = nc * L;
    }
  }
  if (done < n) {
    std::vector<size_t> idx(order.begin() + done, order.end());
    run_slice(device, items, idx, W, out, create_fail);
  }
  if (workers_used) *workers_used = W;
  if (create_fail.load() > 0) return SHCI_ERR_CUDA;
  for (size_t k = 0; k < n; k++)
    if (out[k].status != SHCI_OK) return static_cast<shci_status>(out[k].status);
  return SHCI_OK;
}

// Per-kernel timing with CUDA events on the context stream (enabled by shci_profile).
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <map>
#include <string>
#include <vector>

namespace shci {

struct Profiler {
  bool on = false;
  struct Pending {
    const char* name;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::map<std::string, std::pair<double, unsigned long long>> acc;  // name -> (ms, launches)

  void reset() {
    flush();
    acc.clear();
  }
  // Resolves recorded event pairs (call after the stream has been synchronised).
  void flush() {
    for (auto& p : pending) {
      float ms = 0.f;
      if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
        auto& e = acc[p.name];
        e.first += ms;
        e.second += 1;
      }
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    pending.clear();
  }
  // Host time of a named stage (wall clock, ms).
  void host(const char* name, double ms) {
    auto& e = acc[name];
    e.first += ms;
    e.second += 1;
  }
};

// Wall-clock timing of host work when profiling is on.
class HostScope {
 public:
  HostScope(Profiler& p, const char* name)
      : p_(p), name_(name), t0_(std::chrono::steady_clock::now()) {}
  ~HostScope() { stop(); }
  // records the time so far (once)
  void stop() {
    if (p_.on && !done_)
      p_.host(name_, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() -
                                                               t0_).count());
    done_ = true;
  }

 private:
  Profiler& p_;
  const char* name_;
  std::chrono::steady_clock::time_point t0_;
  bool done_ = false;
};

// Records an event pair around the enclosed launches when profiling is on.
class ProfScope {
 public:
  ProfScope(Profiler& p, cudaStream_t s, const char* name) : p_(p), s_(s), name_(name) {
    if (!p_.on) return;
    cudaEventCreate(&a_);
    cudaEventCreate(&b_);
    cudaEventRecord(a_, s_);
  }
  ~ProfScope() {
    if (!p_.on) return;
    cudaEventRecord(b_, s_);
    p_.pending.push_back(Profiler::Pending{name_, a_, b_});
  }

 private:
  Profiler& p_;
  cudaStream_t s_;
  const char* name_;
  cudaEvent_t a_ = nullptr, b_ = nullptr;
};

}  // namespace shci

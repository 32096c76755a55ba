// Optional per-kernel timing with CUDA events on the launching stream.
// Disabled by default; when enabled every instrumented launch records an
// event pair, and read() returns per name the launch count and total time.
#pragma once

#include "common.cuh"

#include <map>
#include <string>
#include <vector>

namespace prtcl_gpu {

class Profiler {
public:
  ~Profiler() { clear(); }
  bool enabled = false;
  void begin(char const *name, cudaStream_t s) {
    if (!enabled) return;
    cudaEvent_t a = get(), b = get();
    PG_CUDA(cudaEventRecord(a, s));
    open_.push_back({name, a, b, s});
  }
  void end(cudaStream_t s) {
    if (!enabled || open_.empty()) return;
    Rec r = open_.back();
    open_.pop_back();
    PG_CUDA(cudaEventRecord(r.b, s));
    done_.push_back(r);
  }
  // accumulate finished records; names in order of first appearance
  struct Stat {
    long long count = 0;
    double ms = 0.0;
  };
  std::vector<std::pair<std::string, Stat>> read() {
    for (auto &r : done_) {
      PG_CUDA(cudaEventSynchronize(r.b));
      float ms = 0.0f;
      PG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
      auto it = idx_.find(r.name);
      if (it == idx_.end()) {
        idx_[r.name] = stats_.size();
        stats_.push_back({r.name, Stat{}});
        it = idx_.find(r.name);
      }
      stats_[it->second].second.count += 1;
      stats_[it->second].second.ms += ms;
      pool_.push_back(r.a);
      pool_.push_back(r.b);
    }
    done_.clear();
    return stats_;
  }
  void reset() {
    read();
    stats_.clear();
    idx_.clear();
  }
  void clear() {
    for (auto &r : done_) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    for (auto e : pool_) cudaEventDestroy(e);
    done_.clear();
    pool_.clear();
  }

private:
  struct Rec {
    std::string name;
    cudaEvent_t a, b;
    cudaStream_t s;
  };
  cudaEvent_t get() {
    if (!pool_.empty()) {
      cudaEvent_t e = pool_.back();
      pool_.pop_back();
      return e;
    }
    cudaEvent_t e;
    PG_CUDA(cudaEventCreate(&e));
    return e;
  }
  std::vector<Rec> open_, done_;
  std::vector<cudaEvent_t> pool_;
  std::vector<std::pair<std::string, Stat>> stats_;
  std::map<std::string, size_t> idx_;
};

// RAII scope: times the launches queued on `s` while it lives
struct ProfScope {
  Profiler &p;
  cudaStream_t s;
  ProfScope(Profiler &p_, char const *name, cudaStream_t s_) : p(p_), s(s_) { p.begin(name, s); }
  ~ProfScope() {
    try {
      p.end(s);
    } catch (...) {
    }
  }
};

} // namespace prtcl_gpu

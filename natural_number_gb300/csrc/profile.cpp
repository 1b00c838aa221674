// profile.cpp — launch accounting: every kernel launch site reports its name;
// the library counts launches always and, when enabled, brackets each launch
// with CUDA events on its stream so per-kernel device time can be read back.
#include <cuda_runtime.h>

#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "nn_internal.h"

namespace nn {

namespace {
struct Rec {
  const char* name;
  cudaEvent_t a, b;
};
struct Prof {
  std::mutex mu;
  bool enabled = false;
  unsigned long long launches = 0;
  std::vector<Rec> open;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t take() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
};
Prof& prof() {
  static Prof p;
  return p;
}
thread_local cudaEvent_t t_pending = nullptr;
}  // namespace

void launch_begin(const char* name, cudaStream_t st) {
  Prof& P = prof();
  std::lock_guard<std::mutex> g(P.mu);
  ++P.launches;
  if (!P.enabled) return;
  Rec r{name, P.take(), P.take()};
  cudaEventRecord(r.a, st);
  P.open.push_back(r);
  t_pending = r.b;
}

void launch_end(cudaStream_t st) {
  if (!t_pending) return;
  cudaEventRecord(t_pending, st);
  t_pending = nullptr;
}

unsigned long long launch_count() { return prof().launches; }

void profile_enable(bool on) {
  Prof& P = prof();
  std::lock_guard<std::mutex> g(P.mu);
  P.enabled = on;
}

// Per-kernel "name count total_ms" lines; consumes the records (call after a sync).
std::string profile_report() {
  Prof& P = prof();
  std::lock_guard<std::mutex> g(P.mu);
  std::map<std::string, std::pair<unsigned long long, double>> agg;
  for (Rec& r : P.open) {
    float ms = 0.f;
    cudaEventSynchronize(r.b);
    cudaEventElapsedTime(&ms, r.a, r.b);
    auto& x = agg[r.name];
    x.first += 1;
    x.second += ms;
    P.pool.push_back(r.a);
    P.pool.push_back(r.b);
  }
  P.open.clear();
  std::string out;
  char line[256];
  for (auto& kv : agg) {
    std::snprintf(line, sizeof line, "%s %llu %.6f\n", kv.first.c_str(), kv.second.first, kv.second.second);
    out += line;
  }
  return out;
}

}  // namespace nn

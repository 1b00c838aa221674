// host_glue.cpp — the host-side limb arithmetic between GPU products, spread
// over the host's cores for large operands.
//
// The drop-in natural runs the reference's division, pi/e and decimal code on
// the host around its GPU products; their O(n) steps are the reference's
// carry/borrow chains and shifts (asm.h:7-33: asmAdd0/1, asmSub0/1, asmShl,
// asmShr).  For operands of millions of limbs one core spends longer on them
// than the GPU spends on the products, so they run here in chunks:
//  - shifts: each chunk writes its own outputs; the inputs a chunk shares with
//    its neighbour are read before any chunk writes, so in-place shifts stay
//    correct;
//  - add/sub: each chunk adds with carry-in 0, then a pass in chunk order
//    applies each chunk's incoming carry (it stops at the first limb that does
//    not wrap).
// The results are those of the sequential loops, limb for limb.
#include <sched.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/natural_gb300.h"

namespace {

using u64 = uint64_t;

// Usable cores: the affinity mask, capped by a cgroup v2 CPU quota if set.
unsigned usable_cores() {
  unsigned c = std::thread::hardware_concurrency();
  if (c == 0) c = 1;
  cpu_set_t set;
  if (sched_getaffinity(0, sizeof set, &set) == 0) c = std::min<unsigned>(c, (unsigned)CPU_COUNT(&set));
  if (FILE* f = std::fopen("/sys/fs/cgroup/cpu.max", "r")) {
    char quota[32] = {0};
    unsigned long long period = 0;
    if (std::fscanf(f, "%31s %llu", quota, &period) == 2 && std::strcmp(quota, "max") != 0 && period) {
      const unsigned long long q = std::strtoull(quota, nullptr, 10);
      c = std::min<unsigned>(c, (unsigned)std::max<unsigned long long>(1, (q + period - 1) / period));
    }
    std::fclose(f);
  }
  return std::max(1u, std::min(c, 64u));
}

// Persistent workers; one parallel operation at a time (a caller that finds
// the pool busy runs its operation alone).  Never destroyed: the workers
// outlive static destruction.
//
// Each operation is a Job of its own with its own task and completion
// counters, shared by reference count.  A worker that wakes for one job but
// reaches it only after the job has finished (and the next has started)
// still holds the old job: it finds every task claimed and goes back to
// sleep, and never claims or counts a task of the newer job.
class Pool {
 public:
  static Pool& get() {
    static Pool* p = new Pool;
    return *p;
  }
  unsigned size() const { return n_; }

  // f(k) for k in [0, tasks); the caller takes part.  false if busy.
  bool run(unsigned tasks, const std::function<void(unsigned)>& f) {
    std::unique_lock<std::mutex> busy(run_mu_, std::try_to_lock);
    if (!busy.owns_lock()) return false;
    auto job = std::make_shared<Job>(f, tasks);
    {
      std::lock_guard<std::mutex> g(mu_);
      job_ = job;
      ++gen_;
    }
    cv_.notify_all();
    work(*job);
    {
      std::unique_lock<std::mutex> g(job->mu);
      job->done_cv.wait(g, [&] { return job->left.load() == 0; });
    }
    std::lock_guard<std::mutex> g(mu_);
    job_.reset();  // workers still inside work() keep their own reference
    return true;
  }

 private:
  struct Job {
    Job(const std::function<void(unsigned)>& f_, unsigned tasks_) : f(f_), tasks(tasks_), left(tasks_) {}
    const std::function<void(unsigned)>& f;  // lives in run()'s caller until every task is counted
    const unsigned tasks;
    std::atomic<unsigned> next{0}, left;
    std::mutex mu;
    std::condition_variable done_cv;
  };

  Pool() : n_(usable_cores()) {
    for (unsigned t = 1; t < n_; ++t) std::thread([this] { loop(); }).detach();
  }
  // Claims and runs tasks of `J` until none is left.  f is touched only for
  // a claimed task, and run() returns only after every claimed task is
  // counted, so f outlives every use.
  static void work(Job& J) {
    for (;;) {
      const unsigned k = J.next.fetch_add(1);
      if (k >= J.tasks) return;
      J.f(k);
      if (J.left.fetch_sub(1) == 1) {
        std::lock_guard<std::mutex> g(J.mu);
        J.done_cv.notify_all();
      }
    }
  }
  void loop() {
    unsigned long long seen = 0;
    for (;;) {
      std::shared_ptr<Job> J;
      {
        std::unique_lock<std::mutex> g(mu_);
        cv_.wait(g, [&] { return gen_ != seen && job_ != nullptr; });
        seen = gen_;
        J = job_;
      }
      work(*J);
    }
  }
  const unsigned n_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_;
  std::shared_ptr<Job> job_;
  unsigned long long gen_ = 0;
};

constexpr u64 kMinChunk = 1 << 14;  // limbs per task at least

unsigned chunks_for(u64 n) {
  const u64 by_size = n / kMinChunk;
  return (unsigned)std::max<u64>(1, std::min<u64>(by_size, 4ull * Pool::get().size()));
}

// Runs f(k, lo, hi) over `chunks` equal ranges of [0, n).
template <class F>
void for_chunks(u64 n, unsigned chunks, F&& f) {
  auto task = [&](unsigned k) {
    const u64 lo = n * k / chunks, hi = n * (k + 1) / chunks;
    f(k, lo, hi);
  };
  if (chunks <= 1 || !Pool::get().run(chunks, task))
    for (unsigned k = 0; k < chunks; ++k) task(k);
}

inline bool overlaps(const u64* a, u64 na, const u64* b, u64 nb) { return a < b + nb && b < a + na; }

// Sequential add with carry-in over [lo, hi); returns the carry out.
inline u64 add_range(u64* d, const u64* a, const u64* b, u64 lo, u64 hi, u64 c) {
  for (u64 i = lo; i < hi; ++i) {
    const u64 s = a[i] + c;
    const u64 c1 = s < c;
    const u64 t = s + b[i];
    d[i] = t;
    c = c1 | (t < s);
  }
  return c;
}
inline u64 sub_range(u64* d, const u64* a, const u64* b, u64 lo, u64 hi, u64 br) {
  for (u64 i = lo; i < hi; ++i) {
    const u64 x = a[i], y = b[i];
    const u64 t = x - y;
    const u64 r = t - br;
    br = (x < y) | (t < br);
    d[i] = r;
  }
  return br;
}

}  // namespace

extern "C" {

int nn_host_add_n(uint64_t n, uint64_t* d, const uint64_t* a, const uint64_t* b) {
  const unsigned T = chunks_for(n);
  if (T <= 1) return (int)add_range(d, a, b, 0, n, 0);
  std::vector<u64> carry(T);
  for_chunks(n, T, [&](unsigned k, u64 lo, u64 hi) { carry[k] = add_range(d, a, b, lo, hi, 0); });
  u64 c = 0;
  for (unsigned k = 0; k < T; ++k) {
    const u64 lo = n * k / T, hi = n * (k + 1) / T;
    u64 out = carry[k];
    if (c) {  // the chunk's incoming carry: ripple until a limb does not wrap
      u64 i = lo;
      while (i < hi && ++d[i] == 0) ++i;
      if (i == hi) out = 1;
    }
    c = out;
  }
  return (int)c;
}

int nn_host_sub_n(uint64_t n, uint64_t* d, const uint64_t* a, const uint64_t* b) {
  const unsigned T = chunks_for(n);
  if (T <= 1) return (int)sub_range(d, a, b, 0, n, 0);
  std::vector<u64> borrow(T);
  for_chunks(n, T, [&](unsigned k, u64 lo, u64 hi) { borrow[k] = sub_range(d, a, b, lo, hi, 0); });
  u64 br = 0;
  for (unsigned k = 0; k < T; ++k) {
    const u64 lo = n * k / T, hi = n * (k + 1) / T;
    u64 out = borrow[k];
    if (br) {  // the chunk's incoming borrow: ripple until a limb does not wrap
      u64 i = lo;
      while (i < hi && d[i]-- == 0) ++i;
      if (i == hi) out = 1;
    }
    br = out;
  }
  return (int)br;
}

// d[0..n] = s[0..n) << cl, 1 <= cl <= 63 (asmShl: d has n + 1 limbs); d may be s.
// Output j is (s[j] << cl) | (s[j-1] >> (64-cl)) with s[-1] = s[n] = 0.  Chunk k
// writes outputs [lo, hi) (the last chunk also output n), top-down, so an
// in-place shift reads each input before overwriting it; the one input it
// shares with the chunk below, s[lo-1], is read before any chunk writes.
void nn_host_shl_n(unsigned cl, uint64_t n, const uint64_t* s, uint64_t* d) {
  // partial overlap (d = s + k, k != 0): only the sequential order is safe
  const unsigned T = (d != s && overlaps(d, n + 1, s, n)) ? 1 : chunks_for(n);
  std::vector<u64> below(T);
  for (unsigned k = 0; k < T; ++k) {
    const u64 lo = n * k / T;
    below[k] = lo ? s[lo - 1] : 0;
  }
  for_chunks(n, T, [&](unsigned k, u64 lo, u64 hi) {
    const u64 end = k + 1 == T ? n + 1 : hi;
    for (u64 j = end; j-- > lo;) {
      const u64 sj = j < n ? s[j] : 0;
      const u64 sb = j == lo ? below[k] : s[j - 1];
      d[j] = (sj << cl) | (sb >> (64 - cl));
    }
  });
}

// d[0..n) = s[0..n) >> cl, 1 <= cl <= 63 (asmShr); d may be s.
void nn_host_shr_n(unsigned cl, uint64_t n, const uint64_t* s, uint64_t* d) {
  const unsigned T = (d != s && overlaps(d, n, s, n)) ? 1 : chunks_for(n);
  std::vector<u64> above(T);  // s[hi] of each chunk (0 past the end), read before any write
  for (unsigned k = 0; k < T; ++k) {
    const u64 hi = n * (k + 1) / T;
    above[k] = hi < n ? s[hi] : 0;
  }
  for_chunks(n, T, [&](unsigned k, u64 lo, u64 hi) {
    if (hi == lo) return;
    u64 cur = s[lo];
    for (u64 i = lo; i + 1 < hi; ++i) {
      const u64 nx = s[i + 1];
      d[i] = (cur >> cl) | (nx << (64 - cl));
      cur = nx;
    }
    d[hi - 1] = (cur >> cl) | (above[k] << (64 - cl));
  });
}

void nn_host_copy(uint64_t* d, const uint64_t* s, uint64_t n) {
  if (d == s || n == 0) return;
  if (overlaps(d, n, s, n)) {
    std::memmove(d, s, n * 8);
    return;
  }
  for_chunks(n, chunks_for(n), [&](unsigned, u64 lo, u64 hi) { std::memcpy(d + lo, s + lo, (hi - lo) * 8); });
}

}  // extern "C"

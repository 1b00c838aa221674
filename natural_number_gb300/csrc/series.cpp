// series.cpp — pi and e to many digits with per-level GPU batches.
//
// The reference evaluates its binary-splitting series (calc_pi, calc_e,
// natural.h:841-902) and its decimal output (_dec_split/_format_dec,
// natural.h:953-1011) recursively, one product at a time.  For a number of
// terms that is a power of two both recursion trees are perfect, so here they
// are evaluated with the same node formulas in two parts:
//  - the bottom of each tree (subtrees whose values stay below `host_below`
//    limbs: millions of products of a few limbs) runs on host threads, one
//    whole subtree per task, on flat limb spans in per-thread scratch (no
//    allocation per node);
//  - the levels above run level by level in device memory: every product of
//    one level is independent, and the level's products go to the GPU as one
//    batch (nn_batch_create/nn_batch_launch, the persistent work-queue
//    kernel) on device pointers, its sums and differences as batched
//    launches; values cross the host link once each way.
// The values are the reference's: products are exact whichever way they are
// computed, and the adds, |a - b| subtractions, shifts and correction loops
// between them are the reference's own steps.
#include <cuda_runtime.h>
#include <sched.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/natural_gb300.h"
#include "../../include/natural_gb300.hpp"
#include "context_access.h"
#include "nn_internal.h"

namespace {

using u64 = uint64_t;
using u32 = uint32_t;
using u128 = unsigned __int128;
using Clock = std::chrono::steady_clock;

double since(Clock::time_point t) { return std::chrono::duration<double>(Clock::now() - t).count(); }

// ---------------------------------------------------------------------------
// Host threads
// ---------------------------------------------------------------------------

// Usable cores: the affinity mask, capped by a cgroup v2 CPU quota if one is set.
unsigned host_threads() {
  static const unsigned n = [] {
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
    return std::max(1u, std::min(c, 128u));
  }();
  return n;
}

// f(i) for i in [0, n), threads taking blocks of `grain` indices in turn; the
// first exception thrown by any task is rethrown here.
template <class F>
void parallel_for(u64 n, u64 grain, F&& f) {
  grain = std::max<u64>(grain, 1);
  const unsigned T = (unsigned)std::min<u64>(host_threads(), (n + grain - 1) / grain);
  if (T <= 1) {
    for (u64 i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<u64> next{0};
  std::exception_ptr err;
  std::mutex mu;
  auto work = [&] {
    try {
      for (;;) {
        const u64 i0 = next.fetch_add(grain);
        if (i0 >= n) break;
        const u64 i1 = std::min(n, i0 + grain);
        for (u64 i = i0; i < i1; ++i) f(i);
      }
    } catch (...) {
      std::lock_guard<std::mutex> g(mu);
      if (!err) err = std::current_exception();
      next.store(n);
    }
  };
  std::vector<std::thread> ts;
  ts.reserve(T - 1);
  for (unsigned t = 1; t < T; ++t) ts.emplace_back(work);
  work();
  for (auto& th : ts) th.join();
  if (err) std::rethrow_exception(err);
}

// ---------------------------------------------------------------------------
// Limb spans (little-endian u64; length 0 is the value 0)
// ---------------------------------------------------------------------------

inline u64 norm(const u64* a, u64 n) {
  while (n && a[n - 1] == 0) --n;
  return n;
}

// out[0..na+nb) = a * b (schoolbook); returns the normalised length.  out
// must not overlap a or b.
u64 mul_span(u64* out, const u64* a, u64 na, const u64* b, u64 nb) {
  if (!na || !nb) return 0;
  if (na < nb) {
    std::swap(a, b);
    std::swap(na, nb);
  }
  std::memset(out, 0, 8 * (na + nb));
  for (u64 j = 0; j < nb; ++j) {
    const u64 bj = b[j];
    u64* o = out + j;
    u64 c = 0;
    for (u64 i = 0; i < na; ++i) {
      const u128 t = (u128)a[i] * bj + o[i] + c;
      o[i] = (u64)t;
      c = (u64)(t >> 64);
    }
    o[na] = c;
  }
  return norm(out, na + nb);
}

// out = a + b; out may be a or b (it needs max(na, nb) + 1 words).
u64 add_span(u64* out, const u64* a, u64 na, const u64* b, u64 nb) {
  if (na < nb) {
    std::swap(a, b);
    std::swap(na, nb);
  }
  u64 c = 0;
  for (u64 i = 0; i < nb; ++i) {
    const u128 t = (u128)a[i] + b[i] + c;
    out[i] = (u64)t;
    c = (u64)(t >> 64);
  }
  for (u64 i = nb; i < na; ++i) {
    const u64 t = a[i] + c;
    c = t < c;
    out[i] = t;
  }
  out[na] = c;
  return norm(out, na + 1);
}

int cmp_span(const u64* a, u64 na, const u64* b, u64 nb) {
  if (na != nb) return na < nb ? -1 : 1;
  for (u64 i = na; i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

// out = a - b for a >= b (normalised lengths); out may be a or b.
u64 sub_span(u64* out, const u64* a, u64 na, const u64* b, u64 nb) {
  u64 br = 0;
  for (u64 i = 0; i < nb; ++i) {
    const u64 x = a[i], y = b[i];
    out[i] = x - y - br;
    br = (x < y) | ((x == y) & br);
  }
  for (u64 i = nb; i < na; ++i) {
    const u64 x = a[i];
    out[i] = x - br;
    br = x < br;
  }
  return norm(out, na);
}

// |a - b| as natural::operator- computes it (natural.h:324-343); out may be a or b.
u64 absdiff_span(u64* out, const u64* a, u64 na, const u64* b, u64 nb) {
  return cmp_span(a, na, b, nb) >= 0 ? sub_span(out, a, na, b, nb) : sub_span(out, b, nb, a, na);
}

natural to_natural(const u64* a, u64 n) {
  natural x;
  x.resize(std::max<u64>(n, 1));
  if (n)
    std::memcpy(x.data, a, 8 * n);
  else
    x.data[0] = 0;
  return x.std();
}

inline u64 span_len(const natural& x) { return (x.size == 1 && x.data[0] == 0) ? 0 : x.size; }

// Per-thread scratch, grown on demand and kept for the thread's lifetime.
u64* scratch_words(u64 words) {
  static thread_local std::vector<u64> buf;
  if (buf.size() < words) buf.resize(words);
  return buf.data();
}

// ---------------------------------------------------------------------------
// GPU batches of products through pinned staging
// ---------------------------------------------------------------------------

struct Stats {
  double gpu_s = 0, host_s = 0;
  u64 gpu_products = 0, host_products = 0, batches = 0;
};

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string("natural_gb300: ") + what + ": " + cudaGetErrorString(e));
}

// Grow-only pinned host buffer.
struct Pinned {
  u64* p = nullptr;
  u64 cap = 0;
  u64* get(u64 words) {
    if (words > cap) {  // from the recycled page-locked pool, so later calls pin nothing new
      if (p) nn_host_free(p, 8 * cap);
      p = nullptr;
      cap = 0;
      const u64 w = std::max<u64>(words + words / 4, 1 << 16);
      p = static_cast<u64*>(nn_host_alloc(8 * w));
      if (!p) throw std::bad_alloc();
      cap = w;
    }
    return p;
  }
  Pinned() = default;
  Pinned(const Pinned&) = delete;
  Pinned& operator=(const Pinned&) = delete;
  ~Pinned() {
    if (p) nn_host_free(p, 8 * cap);
  }
};

struct Staging {
  Pinned in, out;
};

// ---------------------------------------------------------------------------
// Device-resident tree levels: the levels above the host subtrees keep their
// values in device memory; each level's products go to the GPU as one batch
// on device pointers and its sums as one batched add, and only the root comes
// back.  Values carry their product lengths (the top limbs may be zero).
// ---------------------------------------------------------------------------

constexpr u64 kTreeSlabs = 8;  // pi's host subtrees come in this many slabs

struct DNum {  // n limbs at p in device memory
  u64* p = nullptr;
  u64 n = 0;
};

// The device memory of one tree level, released on the stream (after the
// work queued on it) when the level is replaced.
struct DLevel {
  cudaStream_t st;
  u64* p = nullptr;
  u64 used = 0;
  explicit DLevel(cudaStream_t s) : st(s) {}
  DLevel(const DLevel&) = delete;
  DLevel(DLevel&& o) noexcept : st(o.st), p(o.p), used(o.used) { o.p = nullptr; }
  DLevel& operator=(DLevel&& o) noexcept {
    if (this != &o) {
      if (p) cudaFreeAsync(p, st);
      st = o.st;
      p = o.p;
      used = o.used;
      o.p = nullptr;
    }
    return *this;
  }
  ~DLevel() {
    if (p) cudaFreeAsync(p, st);
  }
  static u64 words(u64 n) { return (n + 1) & ~1ull; }  // even offsets: 16-byte aligned values
  void reserve(u64 w) { check_cuda(cudaMallocAsync((void**)&p, 8 * std::max<u64>(w, 2), st), "tree level"); }
  DNum take(u64 n) {
    DNum d{p + used, n};
    used += words(n);
    return d;
  }
};

// Host naturals into a fresh level: packed into the page-locked buffer `buf`,
// one copy.  `copied` marks the end of the buffer's last copy: the packing
// waits for it (and for nothing else queued on the stream), and it is
// recorded again after this copy.
void upload_level(DLevel& L, const std::vector<const natural*>& xs, std::vector<DNum>& out, Pinned& buf,
                  cudaEvent_t copied) {
  u64 w = 0;
  for (const natural* x : xs) w += DLevel::words(x->size);
  L.reserve(w);
  out.resize(xs.size());
  std::vector<u64> off(xs.size());
  for (size_t k = 0; k < xs.size(); ++k) {
    off[k] = L.used;
    out[k] = L.take(xs[k]->size);
  }
  check_cuda(cudaEventSynchronize(copied), "staging reuse");
  u64* h = buf.get(std::max<u64>(w, 1));
  parallel_for(xs.size(), 256, [&](u64 k) { std::memcpy(h + off[k], xs[k]->data, 8 * xs[k]->size); });
  check_cuda(cudaMemcpyAsync(L.p, h, 8 * w, cudaMemcpyHostToDevice, L.st), "tree upload");
  check_cuda(cudaEventRecord(copied, L.st), "tree upload");
}

struct Event {  // a CUDA event for the duration of a scope
  cudaEvent_t e = nullptr;
  Event() { check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event"); }
  Event(const Event&) = delete;
  ~Event() {
    if (e) cudaEventDestroy(e);
  }
};

// Sums out = x + y (or differences x - y, x >= y): short ones in one batched
// launch (one warp a sum), long ones one multiword scan each (a long
// difference writes one limb past its nout).
constexpr u64 kWarpAddLimbs = 1 << 15;
void device_adds(nn_context* c, const std::vector<nn::AddJob>& jobs) {
  cudaStream_t st = (cudaStream_t)nn_context_stream(c);
  std::vector<nn::AddJob> small;
  for (const nn::AddJob& j : jobs) {
    if (j.nout <= kWarpAddLimbs) {
      small.push_back(j);
      continue;
    }
    // a sum's carry goes to its top limb; a difference's (1: no borrow) to
    // one limb past it, which its caller allocates
    check_cuda(nn::lin_combine(j.out, j.sub ? j.nout : j.nout - 1, j.x, j.nx, 0, j.y, j.ny, 0, j.sub != 0,
                               j.sub ? 1 : 0, nn::ctx_scan(c), st),
               "tree sum");
  }
  if (small.empty()) return;
  DLevel tab(st);
  const u64 w = (small.size() * sizeof(nn::AddJob) + 7) / 8;
  tab.reserve(w);
  check_cuda(nn::ctx_upload(c, tab.p, small.data(), small.size() * sizeof(nn::AddJob)), "sum table");
  check_cuda(nn::add_batch(reinterpret_cast<const nn::AddJob*>(tab.p), small.size(), st), "tree sums");
}

// One level's products as one batch on device pointers; the plan is released
// by the caller once its run is no longer needed (releasing waits for it).
nn_batch* device_products(nn_context* c, const std::vector<nn_mul_job>& jobs) {
  std::vector<u64> na(jobs.size()), nb(jobs.size());
  for (size_t k = 0; k < jobs.size(); ++k) {
    na[k] = jobs[k].n_a;
    nb[k] = jobs[k].n_b;
  }
  nn_batch* B = nullptr;
  nn_status s = nn_batch_create(c, na.data(), nb.data(), nullptr, jobs.size(), &B);
  if (s == NN_OK) s = nn_batch_launch(c, B, jobs.data());
  if (s != NN_OK) {
    if (B) nn_batch_destroy(c, B);
    nn_gb300::check(s, "tree products");
  }
  return B;
}

// A device value back into a normalised natural (waits for the stream).
natural download(nn_context* c, DNum d) {
  natural x;
  x.resize(d.n);
  check_cuda(cudaMemcpyAsync(x.data, d.p, 8 * d.n, cudaMemcpyDeviceToHost, (cudaStream_t)nn_context_stream(c)),
             "root download");
  nn_gb300::check(nn_context_synchronize(c), "tree levels");
  return std::move(x.std());
}

// ---------------------------------------------------------------------------
// pi: calc_pi (natural.h:874-902) over terms [1, terms], terms a power of two
// ---------------------------------------------------------------------------

// Capacities (limbs) of a node covering c terms: a leaf's den and numc take at
// most 4 limbs and its num at most 6; a parent's den and numc are products of
// its children's, its num a sum (or difference) of two products.
inline u64 pi_cap_den(u64 c) { return 4 * c; }
inline u64 pi_cap_numc(u64 c) { return 4 * c; }
inline u64 pi_cap_num(u64 c) { return 4 * c + 72; }
u64 pi_scratch(u64 c) {
  if (c == 1) return 32;
  const u64 h = c / 2;
  return 2 * (pi_cap_num(h) + pi_cap_den(h) + pi_cap_numc(h)) + 2 * pi_cap_num(c) + pi_scratch(h);
}

struct Len3 {
  u64 num, den, numc;
};

// Terms [b, b + c), c a power of two: num/den/numc of calc_pi(b, b + c).
Len3 pi_subtree(u64 b, u64 c, u64* num, u64* den, u64* numc, u64* tmp) {
  if (c == 1) {  // natural.h:875-884
    const u64 one_b[1] = {b};
    u64* t = tmp;
    u64 n = mul_span(t, one_b, 1, one_b, 1);
    const u64 n2 = mul_span(t + 4, t, n, one_b, 1);
    const u64 k0[1] = {0x26dd041d878000ull};
    Len3 r;
    r.den = mul_span(den, t + 4, n2, k0, 1);
    const u64 f1[1] = {2 * b - 1}, f2[1] = {6 * b - 1}, f3[1] = {6 * b - 5};
    n = mul_span(t, f1, 1, f2, 1);
    r.numc = mul_span(numc, t, n, f3, 1);
    const u64 k1[1] = {0x207e2da6ull}, k2[1] = {0xcf6371};
    n = mul_span(t + 8, k1, 1, one_b, 1);
    n = add_span(t + 8, t + 8, n, k2, 1);
    r.num = mul_span(num, t + 8, n, numc, r.numc);
    return r;
  }
  const u64 h = c / 2;
  u64* Ln = tmp;
  u64* Ld = Ln + pi_cap_num(h);
  u64* Lc = Ld + pi_cap_den(h);
  u64* Rn = Lc + pi_cap_numc(h);
  u64* Rd = Rn + pi_cap_num(h);
  u64* Rc = Rd + pi_cap_den(h);
  u64* t1 = Rc + pi_cap_numc(h);
  u64* t2 = t1 + pi_cap_num(c);
  u64* rest = t2 + pi_cap_num(c);
  const Len3 L = pi_subtree(b, h, Ln, Ld, Lc, rest);
  const Len3 R = pi_subtree(b + h, h, Rn, Rd, Rc, rest);
  Len3 out;
  if (c == 2) {  // natural.h:888-893: num = |numc * num1 - num * den1|
    const u64 n1 = mul_span(t1, Lc, L.numc, Rn, R.num);
    const u64 n2 = mul_span(t2, Ln, L.num, Rd, R.den);
    out.num = absdiff_span(t1, t1, n1, t2, n2);
    std::memcpy(num, t1, 8 * out.num);
  } else {  // natural.h:894-900: num = den1 * num + numc * num1
    const u64 n1 = mul_span(t1, Rd, R.den, Ln, L.num);
    const u64 n2 = mul_span(t2, Lc, L.numc, Rn, R.num);
    out.num = add_span(num, t1, n1, t2, n2);
  }
  out.den = mul_span(den, Rd, R.den, Ld, L.den);
  out.numc = mul_span(numc, Lc, L.numc, Rc, R.numc);
  return out;
}

struct PiNode {
  natural num, den, numc;
};

struct DPi {
  DNum num, den, numc;
};

// Levels on the device until one node is left: dl's values live in `cur`
// (or in arenas the caller keeps); each level's plan goes to `plans`, to be
// released once its run is over (releasing waits for the run).
void pi_reduce(nn_context* c, std::vector<DPi>& dl, DLevel& cur, std::vector<nn_batch*>& plans, Stats& S) {
  cudaStream_t st = (cudaStream_t)nn_context_stream(c);
  while (dl.size() > 1) {
    const u64 m = dl.size() / 2;
    u64 w = 0;
    for (u64 j = 0; j < m; ++j) {
      const DPi &L = dl[2 * j], &R = dl[2 * j + 1];
      const u64 n1 = R.den.n + L.num.n, n2 = L.numc.n + R.num.n;
      w += DLevel::words(n1) + DLevel::words(n2) + DLevel::words(R.den.n + L.den.n) +
           DLevel::words(L.numc.n + R.numc.n) + DLevel::words(std::max(n1, n2) + 1);
    }
    DLevel nxt(st);
    nxt.reserve(w);
    std::vector<DPi> up(m);
    std::vector<nn_mul_job> jobs;
    std::vector<nn::AddJob> sums(m);
    jobs.reserve(4 * m);
    for (u64 j = 0; j < m; ++j) {
      const DPi &L = dl[2 * j], &R = dl[2 * j + 1];
      const DNum t1 = nxt.take(R.den.n + L.num.n), t2 = nxt.take(L.numc.n + R.num.n);
      up[j].den = nxt.take(R.den.n + L.den.n);
      up[j].numc = nxt.take(L.numc.n + R.numc.n);
      up[j].num = nxt.take(std::max(t1.n, t2.n) + 1);
      jobs.push_back(nn_mul_job{R.den.p, R.den.n, L.num.p, L.num.n, t1.p});              // num = den1 * num
      jobs.push_back(nn_mul_job{L.numc.p, L.numc.n, R.num.p, R.num.n, t2.p});            // num1 = numc * num1
      jobs.push_back(nn_mul_job{R.den.p, R.den.n, L.den.p, L.den.n, up[j].den.p});       // den = den1 * den
      jobs.push_back(nn_mul_job{L.numc.p, L.numc.n, R.numc.p, R.numc.n, up[j].numc.p});  // numc = numc * numc1
      sums[j] = nn::AddJob{t1.p, t1.n, t2.p, t2.n, up[j].num.p, up[j].num.n};
    }
    plans.push_back(device_products(c, jobs));
    device_adds(c, sums);
    S.gpu_products += 4 * m;
    S.batches += 1;
    cur = std::move(nxt);
    dl.swap(up);
  }
}

void release_plans(nn_context* c, std::vector<nn_batch*>& plans) {
  for (nn_batch* B : plans) nn_batch_destroy(c, B);
  plans.clear();
}

// calc_pi over [1, terms]: the bottom subtrees on host threads, the levels
// above them on the device.  The subtrees come in slabs, computed by a
// producer thread (with all host cores) while this thread hands the slabs
// before to the device (whose calls may wait for the GPU); each slab is
// reduced to its root on the device, and the roots meet in the top levels.
void calc_pi_levels(nn_context* c, u64 terms, natural& num, natural& den, natural& numc, u64 host_below,
                    Staging& stg, Stats& S) {
  // subtrees of `chunk` terms on the host: their den reaches about host_below limbs
  const u64 chunk = std::min(std::bit_floor(std::max<u64>(2, host_below / 2)), terms);
  const u64 nodes = terms / chunk;
  S.host_products += terms * 6 + (terms - nodes) * 4;
  std::atomic<u64> host_ns{0};
  auto subtrees = [&](u64 k0, u64 q, std::vector<PiNode>& lv) {
    const auto t0 = Clock::now();
    lv.assign(q, PiNode{});
    parallel_for(q, 1, [&](u64 i) {
      const u64 cn = pi_cap_num(chunk), cd = pi_cap_den(chunk), cc = pi_cap_numc(chunk);
      u64* w = scratch_words(cn + cd + cc + pi_scratch(chunk));
      const Len3 r = pi_subtree(1 + (k0 + i) * chunk, chunk, w, w + cn, w + cn + cd, w + cn + cd + cc);
      lv[i].num = to_natural(w, r.num);
      lv[i].den = to_natural(w + cn, r.den);
      lv[i].numc = to_natural(w + cn + cd, r.numc);
    });
    host_ns += (u64)(since(t0) * 1e9);
  };
  if (nodes == 1) {
    std::vector<PiNode> lv;
    subtrees(0, 1, lv);
    S.host_s += host_ns * 1e-9;
    num = std::move(lv[0].num);
    den = std::move(lv[0].den);
    numc = std::move(lv[0].numc);
    return;
  }
  const auto tg = Clock::now();
  cudaStream_t st = (cudaStream_t)nn_context_stream(c);
  const u64 slabs = std::min<u64>(kTreeSlabs, nodes / 2), q = nodes / slabs;  // powers of two
  // the producer: slab after slab into `ready`; `stop` ends it early
  std::vector<std::vector<PiNode>> ready(slabs);
  std::mutex mu;
  std::condition_variable cv;
  u64 produced = 0;
  bool stop = false;
  std::exception_ptr perr;
  std::thread producer([&] {
    for (u64 sl = 0; sl < slabs; ++sl) {
      {
        std::lock_guard<std::mutex> g(mu);
        if (stop) return;
      }
      try {
        subtrees(sl * q, q, ready[sl]);
      } catch (...) {
        std::lock_guard<std::mutex> g(mu);
        perr = std::current_exception();
        produced = slabs;
        cv.notify_all();
        return;
      }
      std::lock_guard<std::mutex> g(mu);
      produced = sl + 1;
      cv.notify_all();
    }
  });
  struct Join {  // the producer ends before this function does, however it is left
    std::thread& t;
    std::mutex& mu;
    bool& stop;
    ~Join() {
      {
        std::lock_guard<std::mutex> g(mu);
        stop = true;
      }
      if (t.joinable()) t.join();
    }
  } join{producer, mu, stop};
  Event copied[2];
  std::vector<DLevel> slab_mem;  // each slab's last level, holding its root
  slab_mem.reserve(slabs);
  std::vector<DPi> roots(slabs);
  std::vector<nn_batch*> plans[3];
  struct Release {  // every plan is released, however the function is left
    nn_context* c;
    std::vector<nn_batch*>* p;
    ~Release() {
      for (int i = 0; i < 3; ++i) release_plans(c, p[i]);
    }
  } release{c, plans};
  for (u64 sl = 0; sl < slabs; ++sl) {
    {
      std::unique_lock<std::mutex> g(mu);
      cv.wait(g, [&] { return produced > sl; });
      if (perr) std::rethrow_exception(perr);
    }
    std::vector<PiNode> lv;
    lv.swap(ready[sl]);
    DLevel cur(st);
    std::vector<DPi> dl(q);
    {
      std::vector<const natural*> xs;
      for (const PiNode& nd : lv) {
        xs.push_back(&nd.num);
        xs.push_back(&nd.den);
        xs.push_back(&nd.numc);
      }
      std::vector<DNum> d;
      upload_level(cur, xs, d, sl % 2 ? stg.out : stg.in, copied[sl % 2].e);
      for (u64 k = 0; k < q; ++k) dl[k] = DPi{d[3 * k], d[3 * k + 1], d[3 * k + 2]};
    }
    std::vector<nn_batch*>& mine = plans[sl % 3];
    release_plans(c, mine);  // slab sl - 3's: long done
    pi_reduce(c, dl, cur, mine, S);
    roots[sl] = dl[0];
    slab_mem.push_back(std::move(cur));
  }
  DLevel top(st);
  pi_reduce(c, roots, top, plans[slabs % 3], S);
  num = download(c, roots[0].num);
  den = download(c, roots[0].den);
  numc = download(c, roots[0].numc);
  S.host_s += host_ns * 1e-9;
  S.gpu_s += since(tg);
}

// ---------------------------------------------------------------------------
// e: calc_e (natural.h:841-857) over [0, terms), terms a power of two >= 2
// ---------------------------------------------------------------------------

// A node of c pairs: den at most 2c limbs, num at most 2c + log2(c) + 1.
inline u64 e_cap_den(u64 c) { return 2 * c + 2; }
inline u64 e_cap_num(u64 c) { return 2 * c + 66; }
u64 e_scratch(u64 c) {
  if (c == 1) return 0;
  const u64 h = c / 2;
  return 2 * (e_cap_num(h) + e_cap_den(h)) + e_cap_num(c) + e_scratch(h);
}

struct Len2 {
  u64 num, den;
};

// Pairs [i0, i0 + c): pair i is calc_e(2i, 2i + 2).
Len2 e_subtree(u64 i0, u64 c, u64* num, u64* den, u64* tmp) {
  if (c == 1) {
    const u64 b = 2 * i0;
    num[0] = b + 2;
    Len2 r{1, 1};
    if (b) {
      const u64 x[1] = {b + 1}, y[1] = {b};
      r.den = mul_span(den, x, 1, y, 1);
    } else {
      den[0] = 1;
    }
    return r;
  }
  const u64 h = c / 2;
  u64* Ln = tmp;
  u64* Ld = Ln + e_cap_num(h);
  u64* Rn = Ld + e_cap_den(h);
  u64* Rd = Rn + e_cap_num(h);
  u64* t = Rd + e_cap_den(h);
  u64* rest = t + e_cap_num(c);
  const Len2 L = e_subtree(i0, h, Ln, Ld, rest);
  const Len2 R = e_subtree(i0 + h, h, Rn, Rd, rest);
  Len2 out;
  const u64 nt = mul_span(t, Rd, R.den, Ln, L.num);  // num = den1 * num + num1
  out.num = add_span(num, t, nt, Rn, R.num);
  out.den = mul_span(den, Rd, R.den, Ld, L.den);  // den = den1 * den
  return out;
}

struct ENode {
  natural num, den;
};

void calc_e_levels(nn_context* c, u64 terms, natural& num, natural& den, u64 host_below, Staging& stg,
                   Stats& S) {
  const u64 pairs = terms / 2;
  const u64 chunk = std::min(std::bit_floor(std::max<u64>(1, host_below / 2)), pairs);
  const u64 nodes = pairs / chunk;
  std::vector<ENode> lv(nodes);
  const auto t0 = Clock::now();
  parallel_for(nodes, 1, [&](u64 k) {
    const u64 cn = e_cap_num(chunk), cd = e_cap_den(chunk);
    u64* w = scratch_words(cn + cd + e_scratch(chunk));
    const Len2 r = e_subtree(k * chunk, chunk, w, w + cn, w + cn + cd);
    lv[k].num = to_natural(w, r.num);
    lv[k].den = to_natural(w + cn, r.den);
  });
  S.host_s += since(t0);
  S.host_products += pairs + (pairs - nodes) * 2;
  if (lv.size() == 1) {
    num = std::move(lv[0].num);
    den = std::move(lv[0].den);
    return;
  }
  // the levels above the host subtrees, on the device
  const auto tg = Clock::now();
  cudaStream_t st = (cudaStream_t)nn_context_stream(c);
  struct DE {
    DNum num, den;
  };
  DLevel cur(st);
  std::vector<DE> dl(nodes);
  {
    std::vector<const natural*> xs;
    for (const ENode& nd : lv) {
      xs.push_back(&nd.num);
      xs.push_back(&nd.den);
    }
    std::vector<DNum> d;
    Event copied;
    upload_level(cur, xs, d, stg.in, copied.e);
    for (u64 k = 0; k < nodes; ++k) dl[k] = DE{d[2 * k], d[2 * k + 1]};
    check_cuda(cudaEventSynchronize(copied.e), "tree upload");  // the staging is reused later
    std::vector<ENode>().swap(lv);
  }
  nn_batch* prev = nullptr;
  while (dl.size() > 1) {
    const u64 m = dl.size() / 2;
    u64 w = 0;
    for (u64 j = 0; j < m; ++j) {
      const DE &L = dl[2 * j], &R = dl[2 * j + 1];
      const u64 nt = R.den.n + L.num.n;
      w += DLevel::words(nt) + DLevel::words(R.den.n + L.den.n) + DLevel::words(std::max(nt, R.num.n) + 1);
    }
    DLevel nxt(st);
    nxt.reserve(w);
    std::vector<DE> up(m);
    std::vector<nn_mul_job> jobs;
    std::vector<nn::AddJob> sums(m);
    jobs.reserve(2 * m);
    for (u64 j = 0; j < m; ++j) {
      const DE &L = dl[2 * j], &R = dl[2 * j + 1];
      const DNum t = nxt.take(R.den.n + L.num.n);
      up[j].den = nxt.take(R.den.n + L.den.n);
      up[j].num = nxt.take(std::max(t.n, R.num.n) + 1);
      jobs.push_back(nn_mul_job{R.den.p, R.den.n, L.num.p, L.num.n, t.p});          // num = den1 * num
      jobs.push_back(nn_mul_job{R.den.p, R.den.n, L.den.p, L.den.n, up[j].den.p});  // den = den1 * den
      sums[j] = nn::AddJob{t.p, t.n, R.num.p, R.num.n, up[j].num.p, up[j].num.n};   // ... + num1
    }
    nn_batch* plan = device_products(c, jobs);
    device_adds(c, sums);
    if (prev) nn_batch_destroy(c, prev);
    prev = plan;
    S.gpu_products += 2 * m;
    S.batches += 1;
    cur = std::move(nxt);
    dl.swap(up);
  }
  if (prev) nn_batch_destroy(c, prev);
  num = download(c, dl[0].num);
  den = download(c, dl[0].den);
  S.gpu_s += since(tg);
}

// ---------------------------------------------------------------------------
// Decimal output: _format_dec / _dec_split (natural.h:953-1011)
// ---------------------------------------------------------------------------


// a / b with every step of the division on the device (nn_divmod_host: the
// quotient is unique, so it is natural::_div's); trivial and one-limb
// divisors through the drop-in natural.
natural div_on_device(nn_context* c, const natural& a, const natural& b) {
  if (b.size == 1 || a < b) return a / b;
  natural q, r;
  q.resize(a.size - b.size + 1);
  r.resize(b.size);
  nn_gb300::check(nn_divmod_host(c, q.data, r.data, a.data, a.size, b.data, b.size), "division");
  return std::move(q.std());
}

char* export_str(const std::string& s, u64* n) {
  *n = s.size();
  char* p = (char*)std::malloc(s.size() + 1);
  if (p) {
    std::memcpy(p, s.data(), s.size());
    p[s.size()] = 0;
  }
  return p;
}

// A device copy of a host natural on the stream (the copy has read the
// natural when this returns: pageable sources are staged at once, page-locked
// ones are waited for).
DNum to_device(DLevel& L, const natural& x) {
  L.reserve(DLevel::words(x.size));
  const DNum d = L.take(x.size);
  check_cuda(cudaMemcpyAsync(d.p, x.data, 8 * x.size, cudaMemcpyHostToDevice, L.st), "upload");
  check_cuda(cudaStreamSynchronize(L.st), "upload");
  return d;
}

// A small host table into device memory freed with the level `L` (on the
// context's stream, which is L's; v may change once this returns).
template <class T>
const T* table(nn_context* c, DLevel& L, const std::vector<T>& v) {
  L.reserve((v.size() * sizeof(T) + 7) / 8);
  check_cuda(nn::ctx_upload(c, L.p, v.data(), v.size() * sizeof(T)), "table");
  return reinterpret_cast<const T*>(L.p);
}

// Decimal digits (std::formatter<natural>, natural.h:1089-1091) into a
// malloc'd, NUL-terminated buffer of *len digits: the split tree of
// _format_dec, level by level while the split powers have at least
// host_below limbs, all in device memory: a level's products (hi = base_r *
// (v >> ..) >> shift, then base * hi) run as two batches, the shift as one
// launch, lo = v - base * hi as one batched difference and the correction
// loop (natural.h:962-965) as one launch, one warp a node; the nodes left
// become digits on the device, one warp a node (decimal.cu), and the string
// comes back in one copy.  Only node 0, the first, can end with hi = 0 and
// then splits into its lo alone: one flag a level comes back for it.
// The split's correction for a level of a few long nodes: dec_fix walks each
// node with one warp, which for nodes of hundreds of thousands of limbs is a
// long serial walk; here the test runs one warp a node, every subtraction
// lo -= base is a multiword scan over the whole GPU (into `tmp`, then copied
// back: a scan does not run in place), and hi += 1 one warp a node (the
// walk stops once no carry is left).  Rounds end when no node has
// lo >= base, after at most kMaxFixRounds (dec_fix, which runs next, then
// reports any node still off).
constexpr u64 kFixLoopNodes = 16, kFixLoopLimbs = 1 << 16;
constexpr int kMaxFixRounds = 8;
void fix_long_nodes(nn_context* c, const std::vector<nn::DecFixJob>& fix, const nn::DecFixJob* d_fix,
                    const DNum& base, cudaStream_t st) {
  const u64 n = fix.size();
  u64 longest = 0;
  for (const nn::DecFixJob& f : fix) longest = std::max(longest, f.n_lo);
  DLevel tmp(st), flags(st);
  tmp.reserve(longest + 2);
  flags.reserve((n + 1) / 2);
  u32* need = reinterpret_cast<u32*>(flags.p);
  std::vector<u32> h_need(n);
  for (int r = 0; r < kMaxFixRounds; ++r) {
    check_cuda(nn::dec_need(d_fix, n, base.p, base.n, need, st), "split test");
    check_cuda(cudaMemcpyAsync(h_need.data(), need, 4 * n, cudaMemcpyDeviceToHost, st), "split test");
    check_cuda(cudaStreamSynchronize(st), "split test");
    bool any = false;
    for (u64 k = 0; k < n; ++k) {
      if (!h_need[k]) continue;
      any = true;
      const nn::DecFixJob& f = fix[k];
      check_cuda(nn::lin_combine(tmp.p, f.n_lo, f.lo, f.n_lo, 0, base.p, base.n, 0, true, 1, nn::ctx_scan(c), st),
                 "split correction");
      check_cuda(cudaMemcpyAsync(f.lo, tmp.p, 8 * f.n_lo, cudaMemcpyDeviceToDevice, st), "split correction");
    }
    if (!any) return;
    check_cuda(nn::dec_inc(d_fix, n, need, st), "split correction");
  }
}

char* to_dec_levels(nn_context* c, const natural& x, u64 host_below, Staging& stg, Stats& S, u64* len) {
  using namespace nn_gb300;
  (void)stg;
  const int top = dec_init(x);
  if (top < 0) return export_str(std::to_string(x[0]), len);
  DecCache& C = dec_cache();
  const auto t0 = Clock::now();
  cudaStream_t st = (cudaStream_t)nn_context_stream(c);
  // Split levels while the split powers have at least host_below limbs: the
  // device leaves below cost less than another level down to about there
  // (measured on GB300, a 5 Mi-limb value to 10^8 digits with the levels on
  // host and device: 0.192 s with levels down to 128 limbs, 0.167 s to 256,
  // 0.181 s to 512); at most 4000 limbs, so the leaves stay within 8192 limbs
  // a node.
  const u64 dec_below = std::min<u64>(std::max<u64>(host_below, 16), 4000);
  DLevel consts(st);  // a zero limb, the flags of a level and an error word
  consts.reserve(4);
  check_cuda(cudaMemsetAsync(consts.p, 0, 32, st), "constants");
  const DNum zero1{consts.p, 1};
  u32* err = reinterpret_cast<u32*>(consts.p + 2);
  DLevel cur(st);
  std::vector<DNum> nodes{to_device(cur, x)};
  int i = top;
  for (; i >= 1 && std::min(C.base[i].size, C.base_r[i].size) >= dec_below; --i) {
    const natural& base = C.base[i];
    const natural& base_r = C.base_r[i];
    const u64 nb = base.size, nr = base_r.size;
    const unsigned n_shl = (unsigned)(std::countl_zero(base[nb - 1]) + 1) & 63;
    const u64 shift = ((nb + 2) << 6) - n_shl;  // natural.h:958-960
    DLevel bases(st), br(st);
    const DNum dbase = to_device(bases, base), dbase_r = to_device(br, base_r);
    const u64 n = nodes.size();
    std::vector<DNum> y(n), hp(n), hi(n), p(n), lo(n);
    u64 w = 0;
    for (u64 k = 0; k < n; ++k) {
      const DNum v = nodes[k];
      y[k] = v.n > nb - 1 ? DNum{v.p + nb - 1, v.n - (nb - 1)} : zero1;
      const u64 nhp = nr + y[k].n, nhi = (nhp > (shift >> 6) ? nhp - (shift >> 6) : 1) + 1;
      w += DLevel::words(nhp) + DLevel::words(nhi) + DLevel::words(nb + nhi) + DLevel::words(std::min(v.n, nb + 1) + 1);
    }
    DLevel nxt(st);
    nxt.reserve(w);
    std::vector<nn_mul_job> j1(n), j2(n);
    std::vector<nn::ShrJob> sh(n);
    std::vector<nn::AddJob> sub(n);
    std::vector<nn::DecFixJob> fix(n);
    for (u64 k = 0; k < n; ++k) {
      const DNum v = nodes[k];
      hp[k] = nxt.take(nr + y[k].n);
      hi[k] = nxt.take((hp[k].n > (shift >> 6) ? hp[k].n - (shift >> 6) : 1) + 1);  // a limb for the corrections
      p[k] = nxt.take(nb + hi[k].n);
      // lo = v - base * hi is below a few times base (hi is at most a few
      // short of the quotient), so nb + 1 limbs hold it and the difference is
      // taken mod B^(nb+1); a long difference writes one limb past its length
      const u64 nlo = std::min(v.n, nb + 1);
      lo[k] = nxt.take(nlo + 1);
      lo[k].n = nlo;
      j1[k] = nn_mul_job{dbase_r.p, nr, y[k].p, y[k].n, hp[k].p};  // mul_load(hi, base_r, x >> .., ni)
      sh[k] = nn::ShrJob{hp[k].p, hp[k].n, hi[k].p, hi[k].n, shift};
      j2[k] = nn_mul_job{dbase.p, nb, hi[k].p, hi[k].n, p[k].p};  // mul_load(lo, base, hi, ni)
      sub[k] = nn::AddJob{v.p, std::min(v.n, nlo), p[k].p, std::min(p[k].n, nlo), lo[k].p, nlo, 1};  // lo = *this - lo
      fix[k] = nn::DecFixJob{lo[k].p, lo[k].n, hi[k].p, hi[k].n};
    }
    std::vector<nn_batch*> plans;
    struct Release {
      nn_context* c;
      std::vector<nn_batch*>& p;
      ~Release() { release_plans(c, p); }
    } release{c, plans};
    plans.push_back(device_products(c, j1));
    DLevel tsh(st), tfix(st), flags(st);
    check_cuda(nn::shr_batch(table(c, tsh, sh), sh, st), "split shift");
    plans.push_back(device_products(c, j2));
    device_adds(c, sub);
    flags.reserve((n + 1) / 2);
    u32* zero = reinterpret_cast<u32*>(flags.p);
    const nn::DecFixJob* d_fix = table(c, tfix, fix);
    if (n <= kFixLoopNodes && nb >= kFixLoopLimbs) fix_long_nodes(c, fix, d_fix, dbase, st);
    check_cuda(nn::dec_fix(d_fix, n, dbase.p, nb, zero, err, st), "split correction");
    u32 hz[2] = {0, 0};  // node 0's hi == 0, the error word
    check_cuda(cudaMemcpyAsync(&hz[0], zero, 4, cudaMemcpyDeviceToHost, st), "flag");
    check_cuda(cudaMemcpyAsync(&hz[1], err, 4, cudaMemcpyDeviceToHost, st), "flag");
    check_cuda(cudaStreamSynchronize(st), "split level");
    if (hz[1]) throw std::runtime_error("natural_gb300: decimal split correction did not converge");
    std::vector<DNum> next;
    next.reserve(2 * n);
    for (u64 k = 0; k < n; ++k) {
      const DNum h{hi[k].p, std::min(hi[k].n, nb)}, l{lo[k].p, std::min(lo[k].n, nb)};  // both below base
      if (k == 0 && hz[0]) {  // the first node with hi = 0 goes on as its lo (natural.h:1000-1003)
        next.push_back(l);
      } else {
        next.push_back(h);
        next.push_back(l);
      }
    }
    S.gpu_products += 2 * n;
    nodes.swap(next);
    cur = std::move(nxt);
  }
  // The nodes left, each below base[i]^2 = 10^(18 * 2^(i+1)): 2^(i+1) groups
  // of 18 digits a node written in place of the tree's leaves
  // (natural.h:994-1011); node 0, the first, is written at the same width and
  // loses its leading zeros on the way back.
  const u64 n = nodes.size();
  const u32 groups = 2u << i;
  const u64 width = 18ull * groups;
  u64 maxlen = 2;
  std::vector<const u64*> ptrs(n);
  std::vector<u32> lens(n);
  for (u64 k = 0; k < n; ++k) {
    ptrs[k] = nodes[k].p;
    lens[k] = (u32)nodes[k].n;
    maxlen = std::max(maxlen, nodes[k].n);
  }
  DLevel tp(st), tl(st), bo(st);
  const u64* const* dptrs = table(c, tp, ptrs);
  const u32* dlens = table(c, tl, lens);
  bo.reserve((n * width + 7) / 8);
  char* dout = reinterpret_cast<char*>(bo.p);
  check_cuda(nn::dec_groups(dptrs, (maxlen + 1) & ~1ull, dlens, n, groups, dout, st), "decimal kernel");
  std::string head(width, '0');
  check_cuda(cudaMemcpyAsync(head.data(), dout, width, cudaMemcpyDeviceToHost, st), "download");
  check_cuda(cudaStreamSynchronize(st), "decimal digits");
  u64 off = 0;
  while (off + 1 < width && head[off] == '0') ++off;
  const u64 total = n * width - off;
  char* out = static_cast<char*>(std::malloc(total + 1));
  if (!out) throw std::bad_alloc();
  cudaError_t e = cudaMemcpyAsync(out, dout + off, total, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    std::free(out);
    check_cuda(e, "download");
  }
  out[total] = 0;
  *len = total;
  S.gpu_s += since(t0);
  return out;
}

void fill_timing(double* t, const double* v, int k) {
  if (t)
    for (int i = 0; i < k; ++i) t[i] = v[i];
}

}  // namespace

extern "C" {

nn_status nn_pi_dec_levels(nn_context* c, uint64_t terms, uint64_t acc, uint64_t digits, uint64_t host_below,
                           char** out, uint64_t* len, double* timing) {
  if (!c || !out || !len || terms < 2 || (terms & (terms - 1))) return NN_ERR_INVALID;
  nn_gb300::ScopedContext scope(c);
  try {
    Stats S;
    Staging stg;
    const auto t0 = Clock::now();
    natural num, den, numc, denc;
    calc_pi_levels(c, terms, num, den, numc, host_below, stg, S);  // test.cpp:22-32 recipe
    const double t_tree = since(t0);
    sqrt_10005(numc, denc, acc);
    num = 0xcf6371 * den - num;
    den *= 0x68380 * numc * pow(natural(10), digits);
    num *= denc;
    den = div_on_device(c, den, num);
    const double t_div = since(t0) - t_tree;
    char* digits_out = to_dec_levels(c, den, host_below, stg, S, len);
    const double t_all = since(t0);
    const double tv[8] = {t_all, t_tree, t_div, t_all - t_tree - t_div, S.gpu_s, S.host_s, (double)S.gpu_products,
                          (double)S.host_products};
    fill_timing(timing, tv, 8);
    *out = digits_out;
    return *out ? NN_OK : NN_ERR_OOM;
  } catch (const std::bad_alloc&) {
    return NN_ERR_OOM;
  } catch (const std::exception&) {
    return NN_ERR_CUDA;
  }
}

nn_status nn_e_dec_levels(nn_context* c, uint64_t terms, uint64_t digits, uint64_t host_below, char** out,
                          uint64_t* len, double* timing) {
  if (!c || !out || !len || terms < 2 || (terms & (terms - 1))) return NN_ERR_INVALID;
  nn_gb300::ScopedContext scope(c);
  try {
    Stats S;
    Staging stg;
    const auto t0 = Clock::now();
    natural num, den;
    calc_e_levels(c, terms, num, den, host_below, stg, S);  // test.cpp:12-19 recipe
    const double t_tree = since(t0);
    num *= pow(natural(10), digits);
    num = div_on_device(c, num, den);
    const double t_div = since(t0) - t_tree;
    char* digits_out = to_dec_levels(c, num, host_below, stg, S, len);
    const double t_all = since(t0);
    const double tv[8] = {t_all, t_tree, t_div, t_all - t_tree - t_div, S.gpu_s, S.host_s, (double)S.gpu_products,
                          (double)S.host_products};
    fill_timing(timing, tv, 8);
    *out = digits_out;
    return *out ? NN_OK : NN_ERR_OOM;
  } catch (const std::bad_alloc&) {
    return NN_ERR_OOM;
  } catch (const std::exception&) {
    return NN_ERR_CUDA;
  }
}

nn_status nn_to_dec_levels(nn_context* c, const uint64_t* a, uint64_t na, uint64_t host_below, char** out,
                           uint64_t* len) {
  if (!c || !a || !na || !out || !len) return NN_ERR_INVALID;
  nn_gb300::ScopedContext scope(c);
  try {
    const natural x = to_natural(a, na);
    Stats S;
    Staging stg;
    *out = to_dec_levels(c, x, host_below, stg, S, len);
    return *out ? NN_OK : NN_ERR_OOM;
  } catch (const std::bad_alloc&) {
    return NN_ERR_OOM;
  } catch (const std::exception&) {
    return NN_ERR_CUDA;
  }
}

}  // extern "C"

// series.cpp — pi and e to many digits with per-level GPU batches.
//
// The reference evaluates its binary-splitting series (calc_pi, calc_e,
// natural.h:841-902) and its decimal output (_dec_split/_format_dec,
// natural.h:953-1011) recursively, one product at a time.  For a number of
// terms that is a power of two both recursion trees are perfect, so here they
// are evaluated level by level with the same node formulas: every product of
// one level is independent, and the level's products go to the GPU as one
// batch (nn_batch_create/nn_batch_launch, the persistent work-queue kernel).
// Products whose shorter operand is below `host_below` limbs (the bottom
// levels: millions of products of a few limbs) run on host threads with a
// schoolbook loop.  The values are the reference's: products are exact
// whichever way they are computed, and the adds, |a - b| subtractions, shifts
// and correction loops between them are the reference's own steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/natural_gb300.h"
#include "../../include/natural_gb300.hpp"

namespace {

using u64 = uint64_t;
using Clock = std::chrono::steady_clock;

// Host schoolbook product of small naturals (normalised result).
natural host_mul(const natural& a, const natural& b) {
  natural d;
  d.resize(a.size + b.size);
  std::memset(d.data, 0, 8 * d.size);
  for (u64 i = 0; i < a.size; ++i) {
    unsigned __int128 c = 0;
    const u64 x = a[i];
    if (!x) continue;
    for (u64 j = 0; j < b.size; ++j) {
      c += (unsigned __int128)x * b[j] + d[i + j];
      d[i + j] = (u64)c;
      c >>= 64;
    }
    d[i + b.size] = (u64)c;
  }
  return d.std();
}

template <class F>
void parallel_for(u64 n, F&& f) {
  const unsigned hw = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  if (n < 256 || hw == 1) {
    for (u64 i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> ts;
  for (unsigned t = 0; t < hw; ++t)
    ts.emplace_back([&, t] {
      for (u64 i = t; i < n; i += hw) f(i);
    });
  for (auto& th : ts) th.join();
}

struct Products {
  std::vector<const natural*> a, b;
  std::vector<natural*> out;
  void add(natural* o, const natural* x, const natural* y) {
    a.push_back(x);
    b.push_back(y);
    out.push_back(o);
  }
};

struct Stats {
  double gpu_s = 0, host_s = 0;
  u64 gpu_products = 0, host_products = 0, batches = 0;
};

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string("natural_gb300: ") + what + ": " + cudaGetErrorString(e));
}

// Computes every product of P: small ones on host threads, the rest as one GPU batch.
void run_products(nn_context* c, Products& P, u64 host_below, Stats& S) {
  std::vector<u64> host, gpu;
  for (u64 k = 0; k < P.out.size(); ++k)
    (std::min(P.a[k]->size, P.b[k]->size) < host_below ? host : gpu).push_back(k);
  auto t0 = Clock::now();
  parallel_for(host.size(), [&](u64 i) {
    const u64 k = host[i];
    natural r = host_mul(*P.a[k], *P.b[k]);
    *P.out[k] = std::move(r);
  });
  auto t1 = Clock::now();
  S.host_s += std::chrono::duration<double>(t1 - t0).count();
  S.host_products += host.size();
  if (gpu.empty()) return;
  // pack operands, run one batch, unpack
  std::vector<u64> na(gpu.size()), nb(gpu.size()), oa(gpu.size()), ob(gpu.size()), oo(gpu.size());
  u64 tin = 0, tout = 0;
  for (u64 i = 0; i < gpu.size(); ++i) {
    const u64 k = gpu[i];
    na[i] = P.a[k]->size;
    nb[i] = P.b[k]->size;
    oa[i] = tin;
    tin += na[i];
    ob[i] = tin;
    tin += nb[i];
    oo[i] = tout;
    tout += na[i] + nb[i];
  }
  std::vector<u64> hin(tin), hout(tout);
  parallel_for(gpu.size(), [&](u64 i) {
    const u64 k = gpu[i];
    std::memcpy(hin.data() + oa[i], P.a[k]->data, 8 * na[i]);
    std::memcpy(hin.data() + ob[i], P.b[k]->data, 8 * nb[i]);
  });
  cudaStream_t st = (cudaStream_t)nn_context_stream(c);
  u64 *din = nullptr, *dout = nullptr;
  check_cuda(cudaMallocAsync((void**)&din, 8 * tin, st), "batch operands");
  check_cuda(cudaMallocAsync((void**)&dout, 8 * tout, st), "batch products");
  check_cuda(cudaMemcpyAsync(din, hin.data(), 8 * tin, cudaMemcpyHostToDevice, st), "upload");
  std::vector<nn_mul_job> jobs(gpu.size());
  for (u64 i = 0; i < gpu.size(); ++i) jobs[i] = nn_mul_job{din + oa[i], na[i], din + ob[i], nb[i], dout + oo[i]};
  nn_batch* B = nullptr;
  nn_status s = nn_batch_create(c, na.data(), nb.data(), nullptr, gpu.size(), &B);
  if (s == NN_OK) s = nn_batch_launch(c, B, jobs.data());
  if (s == NN_OK) check_cuda(cudaMemcpyAsync(hout.data(), dout, 8 * tout, cudaMemcpyDeviceToHost, st), "download");
  if (B) nn_batch_destroy(c, B);
  cudaFreeAsync(din, st);
  cudaFreeAsync(dout, st);
  nn_gb300::check(s == NN_OK ? nn_context_synchronize(c) : s, "batched products");
  parallel_for(gpu.size(), [&](u64 i) {
    const u64 k = gpu[i];
    natural r;
    r.resize(na[i] + nb[i]);
    std::memcpy(r.data, hout.data() + oo[i], 8 * r.size);
    r.std();
    *P.out[k] = std::move(r);
  });
  S.gpu_s += std::chrono::duration<double>(Clock::now() - t1).count();
  S.gpu_products += gpu.size();
  S.batches += 1;
}

struct PiNode {
  natural num, den, numc;
};

// calc_pi(num, den, numc, 1, terms + 1) (natural.h:874-902) for terms a power of two.
void calc_pi_levels(nn_context* c, u64 terms, natural& num, natural& den, natural& numc, u64 host_below, Stats& S) {
  std::vector<PiNode> lv(terms);
  parallel_for(terms, [&](u64 i) {  // leaves (natural.h:875-884)
    const u64 b = i + 1;
    PiNode& n = lv[i];
    n.den = host_mul(host_mul(host_mul(natural(b), natural(b)), natural(b)), natural(0x26dd041d878000ull));
    n.numc = host_mul(host_mul(natural(2 * b - 1), natural(6 * b - 1)), natural(6 * b - 5));
    n.num = host_mul(host_mul(natural(0x207e2da6ull), natural(b)) + natural(0xcf6371), n.numc);
  });
  bool pair_level = true;  // end - begin == 2 (natural.h:888-893)
  while (lv.size() > 1) {
    const u64 m = lv.size() / 2;
    std::vector<PiNode> up(m);
    std::vector<natural> t1(m), t2(m);
    Products P;
    for (u64 j = 0; j < m; ++j) {
      PiNode &L = lv[2 * j], &R = lv[2 * j + 1];
      if (pair_level) {
        P.add(&t1[j], &L.numc, &R.num);  // numc * num1
        P.add(&t2[j], &L.num, &R.den);   // num * den1
      } else {
        P.add(&t1[j], &R.den, &L.num);    // num = den1 * num
        P.add(&t2[j], &L.numc, &R.num);   // num1 = numc * num1
      }
      P.add(&up[j].den, &R.den, &L.den);      // den = den1 * den
      P.add(&up[j].numc, &L.numc, &R.numc);   // numc = numc * numc1
    }
    run_products(c, P, host_below, S);
    parallel_for(m, [&](u64 j) {
      up[j].num = pair_level ? t1[j] - t2[j] : t1[j] + t2[j];  // |a - b| as natural::operator-
    });
    lv.swap(up);
    pair_level = false;
  }
  num = std::move(lv[0].num);
  den = std::move(lv[0].den);
  numc = std::move(lv[0].numc);
}

struct ENode {
  natural num, den;
};

// calc_e(num, den, 0, terms) (natural.h:841-857) for terms a power of two >= 2.
void calc_e_levels(nn_context* c, u64 terms, natural& num, natural& den, u64 host_below, Stats& S) {
  std::vector<ENode> lv(terms / 2);
  parallel_for(lv.size(), [&](u64 i) {  // leaves [begin, begin + 2)
    const u64 b = 2 * i;
    lv[i].num = natural(b + 2);
    lv[i].den = b ? host_mul(natural(b + 1), natural(b)) : natural(b + 1);
  });
  while (lv.size() > 1) {
    const u64 m = lv.size() / 2;
    std::vector<ENode> up(m);
    std::vector<natural> t(m);
    Products P;
    for (u64 j = 0; j < m; ++j) {
      ENode &L = lv[2 * j], &R = lv[2 * j + 1];
      P.add(&t[j], &R.den, &L.num);       // num = den1 * num
      P.add(&up[j].den, &R.den, &L.den);  // den = den1 * den
    }
    run_products(c, P, host_below, S);
    parallel_for(m, [&](u64 j) { up[j].num = t[j] + lv[2 * j + 1].num; });
    lv.swap(up);
  }
  num = std::move(lv[0].num);
  den = std::move(lv[0].den);
}

// Decimal digits (std::formatter<natural>, natural.h:1089-1091) with the
// split tree of _format_dec (natural.h:994-1011) evaluated level by level.
std::string to_dec_levels(nn_context* c, const natural& x, u64 host_below, Stats& S) {
  using namespace nn_gb300;
  const int top = dec_init(x);
  if (top < 0) return std::to_string(x[0]);
  DecCache& C = dec_cache();
  struct Node {
    natural v;
    bool first;
  };
  std::vector<Node> lv;
  lv.push_back(Node{x, true});
  for (int i = top; i >= 1; --i) {
    const natural& base = C.base[i];
    const natural& base_r = C.base_r[i];
    const unsigned n_shl = (unsigned)(std::countl_zero(base[base.size - 1]) + 1) & 63;
    const u64 n = lv.size();
    std::vector<natural> y(n), hi(n), lo(n), p(n);
    parallel_for(n, [&](u64 k) { y[k] = lv[k].v >> ((base.size - 1) << 6); });
    Products P1;
    for (u64 k = 0; k < n; ++k) P1.add(&hi[k], &base_r, &y[k]);  // mul_load(hi, base_r, x >> .., ni)
    run_products(c, P1, host_below, S);
    parallel_for(n, [&](u64 k) { hi[k] >>= ((base.size + 2) << 6) - n_shl; });
    Products P2;
    for (u64 k = 0; k < n; ++k) P2.add(&p[k], &base, &hi[k]);  // mul_load(lo, base, hi, ni)
    run_products(c, P2, host_below, S);
    parallel_for(n, [&](u64 k) {
      lo[k] = lv[k].v - p[k];
      while (lo[k] >= base) {  // natural.h:962-965
        hi[k] += 1;
        lo[k] -= base;
      }
    });
    std::vector<Node> next;
    next.reserve(2 * n);
    for (u64 k = 0; k < n; ++k) {
      if (lv[k].first && hi[k] == 0) {
        next.push_back(Node{std::move(lo[k]), true});
      } else {
        next.push_back(Node{std::move(hi[k]), lv[k].first});
        next.push_back(Node{std::move(lo[k]), false});
      }
    }
    lv.swap(next);
  }
  // level 0: div_base by 10^18 (natural.h:954-955), then the 18-digit leaves
  std::vector<std::string> parts(lv.size());
  parallel_for(lv.size(), [&](u64 k) {
    natural q;
    const u64 r = div_base(lv[k].v, dec_base_0, q);
    char buf[48];
    if (lv[k].first && q == 0)
      std::snprintf(buf, sizeof buf, "%llu", (unsigned long long)r);
    else if (lv[k].first)
      std::snprintf(buf, sizeof buf, "%llu%018llu", (unsigned long long)q[0], (unsigned long long)r);
    else
      std::snprintf(buf, sizeof buf, "%018llu%018llu", (unsigned long long)q[0], (unsigned long long)r);
    parts[k] = buf;
  });
  std::string out;
  out.reserve(parts.size() * 36);
  for (auto& s : parts) out += s;
  return out;
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

void fill_timing(double* t, const double* v, int k) {
  if (t)
    for (int i = 0; i < k; ++i) t[i] = v[i];
}

double since(Clock::time_point t) { return std::chrono::duration<double>(Clock::now() - t).count(); }

}  // namespace

extern "C" {

nn_status nn_pi_dec_levels(nn_context* c, uint64_t terms, uint64_t acc, uint64_t digits, uint64_t host_below,
                           char** out, uint64_t* len, double* timing) {
  if (!c || !out || !len || terms < 2 || (terms & (terms - 1))) return NN_ERR_INVALID;
  nn_gb300::ScopedContext scope(c);
  try {
    Stats S;
    auto t0 = Clock::now();
    natural num, den, numc, denc;
    calc_pi_levels(c, terms, num, den, numc, host_below, S);  // test.cpp:22-32 recipe
    const double t_tree = since(t0);
    sqrt_10005(numc, denc, acc);
    num = 0xcf6371 * den - num;
    den *= 0x68380 * numc * pow(natural(10), digits);
    num *= denc;
    den /= num;
    const double t_div = since(t0) - t_tree;
    std::string s = to_dec_levels(c, den, host_below, S);
    const double t_all = since(t0);
    const double tv[8] = {t_all, t_tree, t_div, t_all - t_tree - t_div, S.gpu_s, S.host_s, (double)S.gpu_products,
                          (double)S.host_products};
    fill_timing(timing, tv, 8);
    *out = export_str(s, len);
    return NN_OK;
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
    auto t0 = Clock::now();
    natural num, den;
    calc_e_levels(c, terms, num, den, host_below, S);  // test.cpp:12-19 recipe
    const double t_tree = since(t0);
    num *= pow(natural(10), digits);
    num /= den;
    const double t_div = since(t0) - t_tree;
    std::string s = to_dec_levels(c, num, host_below, S);
    const double t_all = since(t0);
    const double tv[8] = {t_all, t_tree, t_div, t_all - t_tree - t_div, S.gpu_s, S.host_s, (double)S.gpu_products,
                          (double)S.host_products};
    fill_timing(timing, tv, 8);
    *out = export_str(s, len);
    return NN_OK;
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
    natural x;
    x.resize(na);
    std::memcpy(x.data, a, 8 * na);
    x.std();
    Stats S;
    *out = export_str(to_dec_levels(c, x, host_below, S), len);
    return NN_OK;
  } catch (const std::bad_alloc&) {
    return NN_ERR_OOM;
  } catch (const std::exception&) {
    return NN_ERR_CUDA;
  }
}

}  // extern "C"

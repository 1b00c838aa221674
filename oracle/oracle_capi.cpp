// oracle_capi.cpp — TEST INFRASTRUCTURE ONLY.
// C entry points over the oracle (nn_oracle.hpp) for the test-suite and the
// bench's CPU-baseline leg.  Results are malloc'd; release with nno_free.
// oracle/ref_shim.cpp exports the same entry points (prefix ref_) over the
// reference compiled from its own sources, so both can be driven by one
// Python wrapper (oracle/__init__.py).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "nn_oracle.hpp"

using nno::Nat;
using nno::u64;

namespace {
u64* export_limbs(const nno::Limbs& x, u64* n) {
  *n = x.n;
  u64* p = (u64*)std::malloc(sizeof(u64) * (x.n ? x.n : 1));
  std::memcpy(p, x.data(), sizeof(u64) * x.n);
  return p;
}
char* export_str(const std::string& s, u64* n) {
  *n = s.size();
  char* p = (char*)std::malloc(s.size() + 1);
  std::memcpy(p, s.data(), s.size());
  p[s.size()] = 0;
  return p;
}
Nat make(const u64* a, u64 n) { return Nat(a, n); }

std::string pi_digits(u64 terms, u64 acc, u64 digits) {  // test.cpp:22-32 recipe
  Nat num, den, numc, denc;
  nno::calc_pi(num, den, numc, 1, terms | 1);
  nno::sqrt_10005(numc, denc, acc);
  num = nno::subn(nno::mul(Nat(0xcf6371), den), num);
  den = nno::mul(den, nno::mul(nno::mul(Nat(0x68380), numc), nno::pow(Nat(10), digits)));
  num = nno::mul(num, denc);
  Nat r;
  den = nno::divmod(den, num, r);
  return nno::to_dec(den);
}

std::string e_digits(u64 terms, u64 digits) {  // test.cpp:12-19 recipe
  Nat num, den;
  nno::calc_e(num, den, 0, terms);
  num = nno::mul(num, nno::pow(Nat(10), digits));
  Nat r;
  num = nno::divmod(num, den, r);
  return nno::to_dec(num);
}
}  // namespace

extern "C" {

void nno_free(void* p) { std::free(p); }

unsigned long long nno_div_fallbacks(void) { return nno::fallback_count(); }

u64* nno_mul(const u64* a, u64 na, const u64* b, u64 nb, u64* out_n) {
  return export_limbs(nno::mul(make(a, na), make(b, nb)), out_n);
}

u64* nno_sqr(const u64* a, u64 na, u64* out_n) { return export_limbs(nno::sqr(make(a, na)), out_n); }

u64* nno_mul_base(const u64* a, u64 na, const u64* b, u64 nb, u64* out_n) {
  return export_limbs(nno::mul_base_nat(make(a, na), make(b, nb)), out_n);
}

u64* nno_ntt_mul_raw(const u64* a, u64 na, const u64* b, u64 nb, int s, u64 size, u64* out_n) {
  return export_limbs(nno::ntt_mul_raw(a, na, b, nb, s, size), out_n);
}

u64* nno_ntt_sqr_raw(const u64* a, u64 na, int s, u64 size, u64* out_n) {
  nno::Xform x;
  x.load(a, na, s);
  x.ntt();
  x.mul(x, x);
  x.intt();
  nno::Limbs out;
  x.save(out, size);
  return export_limbs(out, out_n);
}

// load + forward NTT: 3 * 2^s words, prime-major, raw (values in [0, 2p)).
void nno_ntt_forward(const u64* a, u64 na, int s, u64* out) {
  nno::Xform x;
  x.load(a, na, s);
  x.ntt();
  const u64 L = 1ull << s;
  for (int i = 0; i < 3; ++i) std::memcpy(out + i * L, x.info[i].data(), sizeof(u64) * L);
}

// Twiddle table root (inverse=0) or iroot (inverse=1) for scale s: 2^(s-1) words.
void nno_root_table(int s, int prime, int inverse, u64* out) {
  nno::tables().init(s);
  const auto& t = inverse ? nno::tables().iroot[prime] : nno::tables().root[prime];
  std::memcpy(out, t.data(), sizeof(u64) * (1ull << (s - 1)));
}

u64* nno_div(const u64* a, u64 na, const u64* b, u64 nb, u64* qn, u64** r, u64* rn) {
  Nat rr;
  Nat q = nno::divmod(make(a, na), make(b, nb), rr);
  *r = export_limbs(rr, rn);
  return export_limbs(q, qn);
}

u64* nno_pow(const u64* b, u64 nb, u64 e, u64* out_n) { return export_limbs(nno::pow(make(b, nb), e), out_n); }

u64* nno_reciprocal2(const u64* d, u64 nd, u64 divd_size, u64* out_n) {
  return export_limbs(nno::reciprocal2(make(d, nd), divd_size), out_n);
}

u64* nno_reciprocal3(const u64* d, u64 nd, u64 divd_size, u64* out_n) {
  nno::Xform x;
  return export_limbs(nno::reciprocal3(make(d, nd), divd_size, x), out_n);
}

char* nno_to_dec(const u64* a, u64 na, u64* len) { return export_str(nno::to_dec(make(a, na)), len); }

char* nno_pi_dec(u64 terms, u64 acc, u64 digits, u64* len) { return export_str(pi_digits(terms, acc, digits), len); }

char* nno_e_dec(u64 terms, u64 digits, u64* len) { return export_str(e_digits(terms, digits), len); }

// Times `reps` products of the given operands; returns seconds per product.
double nno_time_mul(const u64* a, u64 na, const u64* b, u64 nb, int reps) {
  Nat x = make(a, na), y = make(b, nb);
  (void)nno::mul(x, y);  // grow the twiddle tables outside the timed loop
  auto t0 = std::chrono::steady_clock::now();
  u64 sink = 0;
  for (int i = 0; i < reps; ++i) sink ^= nno::mul(x, y)[0];
  auto t1 = std::chrono::steady_clock::now();
  if (sink == 0x5eed) std::fputc(' ', stderr);
  return std::chrono::duration<double>(t1 - t0).count() / reps;
}

double nno_time_sqr(const u64* a, u64 na, int reps) {
  Nat x = make(a, na);
  (void)nno::sqr(x);
  auto t0 = std::chrono::steady_clock::now();
  u64 sink = 0;
  for (int i = 0; i < reps; ++i) sink ^= nno::sqr(x)[0];
  auto t1 = std::chrono::steady_clock::now();
  if (sink == 0x5eed) std::fputc(' ', stderr);
  return std::chrono::duration<double>(t1 - t0).count() / reps;
}

}  // extern "C"

// ref_shim.cpp — TEST INFRASTRUCTURE ONLY.
// Glue that exposes the reference library itself (compiled from its own
// headers and its assembly, see oracle/build_ref.sh) through the same entry
// points as oracle/oracle_capi.cpp, prefixed ref_.  Used only to pin the
// oracle and to generate the golden fixtures under tests/golden/.
#include <utility>
#include <iostream>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <string>

#include "natural.h"  // resolved with -I<reference dir>

using u64 = std::uint64_t;

namespace {
u64* export_limbs(const basic_natural& x, u64* n) {
  *n = x.size;
  u64* p = (u64*)std::malloc(sizeof(u64) * (x.size ? x.size : 1));
  std::memcpy(p, x.data, sizeof(u64) * x.size);
  return p;
}
char* export_str(const std::string& s, u64* n) {
  *n = s.size();
  char* p = (char*)std::malloc(s.size() + 1);
  std::memcpy(p, s.data(), s.size());
  p[s.size()] = 0;
  return p;
}
natural make(const u64* a, u64 n) {
  natural x;
  x.resize(n);
  std::memcpy(x.data, a, n * sizeof(u64));
  return x;
}
}  // namespace

extern "C" {

void ref_free(void* p) { std::free(p); }

u64* ref_mul(const u64* a, u64 na, const u64* b, u64 nb, u64* out_n) {
  return export_limbs(make(a, na) * make(b, nb), out_n);
}

u64* ref_sqr(const u64* a, u64 na, u64* out_n) { return export_limbs(sqr(make(a, na)), out_n); }

u64* ref_mul_base(const u64* a, u64 na, const u64* b, u64 nb, u64* out_n) {
  natural x = make(a, na), y = make(b, nb), d;
  d._mul_base(&x, &y);
  return export_limbs(d, out_n);
}

u64* ref_ntt_mul_raw(const u64* a, u64 na, const u64* b, u64 nb, int s, u64 size, u64* out_n) {
  NTT_info xa(a, na, s), xb(b, nb, s);
  xa.NTT();
  xb.NTT();
  xa.mul(xa, xb);
  xa.INTT();
  basic_natural out;
  xa.save(out, size);
  return export_limbs(out, out_n);
}

u64* ref_ntt_sqr_raw(const u64* a, u64 na, int s, u64 size, u64* out_n) {
  NTT_info x(a, na, s);
  x.NTT();
  x.mul(x, x);
  x.INTT();
  basic_natural out;
  x.save(out, size);
  return export_limbs(out, out_n);
}

void ref_ntt_forward(const u64* a, u64 na, int s, u64* out) {
  NTT_info x(a, na, s);
  x.NTT();
  const u64 L = 1ull << s;
  for (int i = 0; i < 3; ++i) std::memcpy(out + i * L, x.info[i].data, sizeof(u64) * L);
}

void ref_root_table(int s, int prime, int inverse, u64* out) {
  NTT_info::init(s);
  const basic_natural& t = inverse ? NTT_info::iroot[prime] : NTT_info::root[prime];
  std::memcpy(out, t.data, sizeof(u64) * (1ull << (s - 1)));
}

u64* ref_div(const u64* a, u64 na, const u64* b, u64 nb, u64* qn, u64** r, u64* rn) {
  natural x = make(a, na), y = make(b, nb), q, rr;
  q._div(&x, &y, &rr);
  *r = export_limbs(rr, rn);
  return export_limbs(q, qn);
}

u64* ref_pow(const u64* b, u64 nb, u64 e, u64* out_n) { return export_limbs(pow(make(b, nb), e), out_n); }

u64* ref_reciprocal2(const u64* d, u64 nd, u64 divd_size, u64* out_n) {
  return export_limbs(reciprocal(make(d, nd), divd_size), out_n);
}

u64* ref_reciprocal3(const u64* d, u64 nd, u64 divd_size, u64* out_n) {
  NTT_info x;
  return export_limbs(reciprocal(make(d, nd), divd_size, x), out_n);
}

char* ref_to_dec(const u64* a, u64 na, u64* len) { return export_str(std::format("{}", make(a, na)), len); }

char* ref_pi_dec(u64 terms, u64 acc, u64 digits, u64* len) {  // test.cpp:22-32
  natural num, den, numc, denc;
  calc_pi(num, den, numc, 1, terms | 1);
  sqrt_10005(numc, denc, acc);
  num = 0xcf6371 * den - num;
  den *= 0x68380 * numc * pow(natural(10), digits);
  num *= denc;
  den /= num;
  return export_str(std::format("{}", den), len);
}

char* ref_e_dec(u64 terms, u64 digits, u64* len) {  // test.cpp:12-19
  natural num, den;
  calc_e(num, den, 0, terms);
  num *= pow(natural(10), digits);
  num /= den;
  return export_str(std::format("{}", num), len);
}

double ref_time_mul(const u64* a, u64 na, const u64* b, u64 nb, int reps) {
  natural x = make(a, na), y = make(b, nb);
  (void)(x * y);
  auto t0 = std::chrono::steady_clock::now();
  u64 sink = 0;
  for (int i = 0; i < reps; ++i) sink ^= (x * y)[0];
  auto t1 = std::chrono::steady_clock::now();
  if (sink == 0x5eed) std::cerr << ' ';
  return std::chrono::duration<double>(t1 - t0).count() / reps;
}

double ref_time_sqr(const u64* a, u64 na, int reps) {
  natural x = make(a, na);
  (void)sqr(x);
  auto t0 = std::chrono::steady_clock::now();
  u64 sink = 0;
  for (int i = 0; i < reps; ++i) sink ^= sqr(x)[0];
  auto t1 = std::chrono::steady_clock::now();
  if (sink == 0x5eed) std::cerr << ' ';
  return std::chrono::duration<double>(t1 - t0).count() / reps;
}

}  // extern "C"

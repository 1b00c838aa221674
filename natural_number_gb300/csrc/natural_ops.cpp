// natural_ops.cpp — C entry points for the natural-level algorithms of
// include/natural_gb300.hpp (division, power, reciprocals, decimal output,
// pi/e), so that C and Python callers reach the same code as C++ callers.
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>

#include "../../include/natural_gb300.hpp"

namespace {

uint64_t* export_limbs(const basic_natural& x, uint64_t* n) {
  *n = x.size;
  uint64_t* p = (uint64_t*)std::malloc(8 * (x.size ? x.size : 1));
  if (p) std::memcpy(p, x.data, 8 * x.size);
  return p;
}
char* export_str(const std::string& s, uint64_t* n) {
  *n = s.size();
  char* p = (char*)std::malloc(s.size() + 1);
  if (p) {
    std::memcpy(p, s.data(), s.size());
    p[s.size()] = 0;
  }
  return p;
}
natural make(const uint64_t* a, uint64_t n) {
  natural x;
  x.resize(n);
  std::memcpy(x.data, a, 8 * n);
  return x;
}

template <class F>
nn_status guarded(nn_context* c, F&& f) {
  if (!c) return NN_ERR_INVALID;
  nn_gb300::ScopedContext scope(c);
  try {
    f();
    return NN_OK;
  } catch (const std::bad_alloc&) {
    return NN_ERR_OOM;
  } catch (const std::exception& e) {
    std::string m = e.what();
    if (m.find("budget") != std::string::npos) return NN_ERR_BUDGET;
    if (m.find("timed out") != std::string::npos) return NN_ERR_TIMEOUT;
    return NN_ERR_CUDA;
  }
}

}  // namespace

extern "C" {

void nn_free(void* p) { std::free(p); }

nn_status nn_div_host(nn_context* c, const uint64_t* a, uint64_t na, const uint64_t* b, uint64_t nb, uint64_t** q,
                      uint64_t* qn, uint64_t** r, uint64_t* rn) {
  if (!a || !b || !na || !nb || !q || !r || !qn || !rn) return NN_ERR_INVALID;
  return guarded(c, [&] {
    natural x = make(a, na), y = make(b, nb), rr;
    natural qq = x;
    qq._div(&x, &y, &rr);
    *q = export_limbs(qq, qn);
    *r = export_limbs(rr, rn);
  });
}

nn_status nn_pow_host(nn_context* c, const uint64_t* b, uint64_t nb, uint64_t e, uint64_t** out, uint64_t* out_n) {
  if (!b || !nb || !out || !out_n) return NN_ERR_INVALID;
  return guarded(c, [&] { *out = export_limbs(pow(make(b, nb), e), out_n); });
}

nn_status nn_reciprocal_host(nn_context* c, const uint64_t* d, uint64_t nd, uint64_t divd_size, int variant,
                             uint64_t** out, uint64_t* out_n) {
  if (!d || nd < 2 || d[nd - 1] != 1 || !out || !out_n || divd_size + 1 < nd) return NN_ERR_INVALID;
  return guarded(c, [&] {
    if (variant == 2) {
      *out = export_limbs(reciprocal(make(d, nd), divd_size), out_n);
    } else {
      NTT_info ni;
      *out = export_limbs(reciprocal(make(d, nd), divd_size, ni), out_n);
    }
  });
}

nn_status nn_to_dec_host(nn_context* c, const uint64_t* a, uint64_t na, char** out, uint64_t* len) {
  if (!a || !na || !out || !len) return NN_ERR_INVALID;
  return guarded(c, [&] { *out = export_str(to_dec_string(make(a, na)), len); });
}

nn_status nn_pi_dec_host(nn_context* c, uint64_t terms, uint64_t acc, uint64_t digits, char** out, uint64_t* len) {
  if (!out || !len || terms < 1) return NN_ERR_INVALID;
  return guarded(c, [&] {  // test.cpp:22-32
    natural num, den, numc, denc;
    calc_pi(num, den, numc, 1, terms | 1);
    sqrt_10005(numc, denc, acc);
    num = 0xcf6371 * den - num;
    den *= 0x68380 * numc * pow(natural(10), digits);
    num *= denc;
    den /= num;
    *out = export_str(to_dec_string(den), len);
  });
}

nn_status nn_e_dec_host(nn_context* c, uint64_t terms, uint64_t digits, char** out, uint64_t* len) {
  if (!out || !len || terms < 2 || (terms & (terms - 1))) return NN_ERR_INVALID;
  return guarded(c, [&] {  // test.cpp:12-19
    natural num, den;
    calc_e(num, den, 0, terms);
    num *= pow(natural(10), digits);
    num /= den;
    *out = export_str(to_dec_string(num), len);
  });
}

}  // extern "C"

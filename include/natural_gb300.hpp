// natural_gb300.hpp — drop-in `natural` for the GB300 multiply path.
//
// The operator surface of Natural_Number's `natural` (natural.h:16-80,
// 537-564, 771-793, 1020-1093) and its engine object `NTT_info`
// (ntt_info.h:10-67), header-only C++20 like the original.  Every product,
// square and NTT transform goes through the C ABI in natural_gb300.h to the
// sm_103a kernels; the host keeps only O(n) glue (shifts, adds, subtractions,
// comparisons, the limb-by-limb complements of the Newton steps) and the
// one-limb division div_base.  The division, pi/e and decimal algorithms are
// the reference's, step for step, so intermediate values (wrapped products,
// reciprocal approximations) equal the reference's as well as the results.
//
// Differences from the reference:
//  - errors throw std::runtime_error (the reference exits on allocation failure);
//  - NTT_info holds a device-resident transform and is move-only; load() runs
//    the load and the forward transform together (NTT() is then a no-op);
//  - all calls use nn_default_context(): one CUDA device, one host thread.
#pragma once

#include <algorithm>
#include <bit>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <format>
#include <initializer_list>
#include <iostream>
#include <queue>
#include <stdexcept>
#include <string>
#include <string_view>
#include <utility>
#include <vector>

#include "natural_gb300.h"

namespace nn_gb300 {

// Context used by the calls below: a scoped override (ScopedContext), else the
// process-wide default context.
inline nn_context*& ctx_override() {
  static thread_local nn_context* c = nullptr;
  return c;
}
struct ScopedContext {
  nn_context* prev;
  explicit ScopedContext(nn_context* c) : prev(ctx_override()) { ctx_override() = c; }
  ~ScopedContext() { ctx_override() = prev; }
};

inline nn_context* ctx() {
  if (nn_context* o = ctx_override()) return o;
  nn_context* c = nn_default_context();
  if (!c) throw std::runtime_error("natural_gb300: no CUDA device");
  return c;
}

inline void check(nn_status st, const char* what) {
  if (st != NN_OK)
    throw std::runtime_error(std::string("natural_gb300: ") + what + ": " + nn_status_string(st) + ": " +
                             nn_last_error(ctx()));
}

// ---- host limb glue (the carry/borrow chains of asm.h:7-30) ---------------
// From 2^16 limbs up these run on all host cores in the library
// (nn_host_add_n and friends), with the same results.
constexpr uint64_t kParallelLimbs = 1u << 16;
inline void copy_n(uint64_t* d, const uint64_t* s, uint64_t n) {
  if (n >= kParallelLimbs)
    nn_host_copy(d, s, n);
  else
    std::memmove(d, s, n * 8);
}
inline int add_n(uint64_t n, uint64_t* d, const uint64_t* a, const uint64_t* b) {
  if (n >= kParallelLimbs) return nn_host_add_n(n, d, a, b);
  uint64_t c = 0;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t s = a[i] + c;
    uint64_t c1 = s < c;
    uint64_t t = s + b[i];
    d[i] = t;
    c = c1 | (t < s);
  }
  return (int)c;
}
inline int add_1(uint64_t n, const uint64_t* s, uint64_t* d, int cf) {
  uint64_t i = 0;
  for (; i < n && cf; ++i) {
    d[i] = s[i] + 1;
    cf = d[i] == 0;
  }
  if (i < n && d != s) copy_n(d + i, s + i, n - i);
  return cf;
}
inline int sub_n(uint64_t n, uint64_t* d, const uint64_t* a, const uint64_t* b) {
  if (n >= kParallelLimbs) return nn_host_sub_n(n, d, a, b);
  uint64_t br = 0;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t x = a[i], y = b[i];
    uint64_t t = x - y;
    uint64_t r = t - br;
    br = (x < y) | (t < br);
    d[i] = r;
  }
  return (int)br;
}
inline int sub_1(uint64_t n, const uint64_t* s, uint64_t* d, int cf) {
  uint64_t i = 0;
  for (; i < n && cf; ++i) {
    uint64_t v = s[i];
    d[i] = v - 1;
    cf = v == 0;
  }
  if (i < n && d != s) copy_n(d + i, s + i, n - i);
  return cf;
}
// base.h:7-16
inline int add(uint64_t* d, const uint64_t* a, uint64_t n1, const uint64_t* b, uint64_t n2) {
  return add_1(n1 - n2, a + n2, d + n2, add_n(n2, d, a, b));
}
inline int sub(uint64_t* d, const uint64_t* a, uint64_t n1, const uint64_t* b, uint64_t n2) {
  return sub_1(n1 - n2, a + n2, d + n2, sub_n(n2, d, a, b));
}
inline void shl_n(unsigned cl, uint64_t n, const uint64_t* s, uint64_t* d) {  // asmShl semantics
  if (n >= kParallelLimbs) return nn_host_shl_n(cl, n, s, d);
  uint64_t carry = 0;
  for (uint64_t i = n; i-- > 0;) {
    uint64_t x = s[i];
    d[i + 1] = (carry << cl) | (x >> (64 - cl));
    carry = x;
  }
  d[0] = carry << cl;
}
inline void shr_n(unsigned cl, uint64_t n, const uint64_t* s, uint64_t* d) {  // asmShr semantics
  if (n >= kParallelLimbs) return nn_host_shr_n(cl, n, s, d);
  uint64_t cur = s[0];
  for (uint64_t i = 0; i + 1 < n; ++i) {
    uint64_t nx = s[i + 1];
    d[i] = (cur >> cl) | (nx << (64 - cl));
    cur = nx;
  }
  d[n - 1] = cur >> cl;
}
inline uint64_t div_128(uint64_t lo, uint64_t hi, uint64_t d, uint64_t* rem = nullptr) {  // asmDiv/asmDivMod
  unsigned __int128 n = ((unsigned __int128)hi << 64) | lo;
  uint64_t q = (uint64_t)(n / d);
  if (rem) *rem = (uint64_t)(n - (unsigned __int128)q * d);
  return q;
}

// Thrown where the reference's Newton division would break one of its own
// size preconditions (the reference then reads or copies out of bounds and
// aborts, e.g. for some 2n-by-n-limb divisions); _div then takes the exact
// Newton division below instead.
struct precondition_broken {};

constexpr uint64_t NTTmul_threshold = 384;  // ntt_info.h:6
constexpr uint64_t NTTdiv_threshold = 256;  // ntt_info.h:7
constexpr int NTTscale_threshold = 10;      // ntt_info.h:8

}  // namespace nn_gb300

// ---------------------------------------------------------------------------
// basic_natural (basic_natural.h:9-97): limbs with capacity = bit_ceil(size).
// Buffers of 64 KiB and more come from the library's page-locked host pool,
// so the copies to and from the GPU around every product run at the host
// link's speed; smaller ones are malloc'd as in the reference.  Which
// allocator a buffer came from follows from its capacity alone.
// ---------------------------------------------------------------------------
namespace nn_gb300 {
constexpr uint64_t kPinnedLimbs = 1u << 13;
inline uint64_t* limb_alloc(uint64_t cap) {
  void* p = cap >= kPinnedLimbs ? nn_host_alloc(cap * 8) : std::malloc(cap * 8);
  if (!p) throw std::bad_alloc();
  return static_cast<uint64_t*>(p);
}
inline void limb_free(uint64_t* p, uint64_t cap) {
  if (!p) return;
  if (cap >= kPinnedLimbs)
    nn_host_free(p, cap * 8);
  else
    std::free(p);
}
}  // namespace nn_gb300

struct basic_natural {
  uint64_t* data;
  uint64_t size;
  uint64_t capacity;

  basic_natural() : data(nn_gb300::limb_alloc(1)), size(1), capacity(1) {}
  basic_natural(std::initializer_list<uint64_t> n) : size(n.size()), capacity(std::bit_ceil(n.size())) {
    data = nn_gb300::limb_alloc(capacity);
    std::memcpy(data, n.begin(), size * 8);
  }
  basic_natural(const basic_natural& n) : size(n.size), capacity(std::bit_ceil(n.size)) {
    data = nn_gb300::limb_alloc(capacity);
    nn_gb300::copy_n(data, n.data, size);
  }
  basic_natural(basic_natural&& n) noexcept : data(n.data), size(n.size), capacity(n.capacity) { n.data = nullptr; }
  ~basic_natural() { nn_gb300::limb_free(data, capacity); }
  basic_natural& operator=(const basic_natural& n) {
    if (this != &n) {
      resize(n.size);
      nn_gb300::copy_n(data, n.data, size);
    }
    return *this;
  }
  basic_natural& operator=(basic_natural&& n) noexcept {
    if (this != &n) {
      nn_gb300::limb_free(data, capacity);
      data = n.data;
      size = n.size;
      capacity = n.capacity;
      n.data = nullptr;
    }
    return *this;
  }
  void resize(uint64_t s) {
    size = s;
    if (capacity < s) {
      const uint64_t cap = std::bit_ceil(s);
      uint64_t* p = nn_gb300::limb_alloc(cap);
      if (data) nn_gb300::copy_n(p, data, capacity);  // what realloc would keep
      nn_gb300::limb_free(data, capacity);
      data = p;
      capacity = cap;
    }
  }
  uint64_t& operator[](uint64_t i) { return data[i]; }
  const uint64_t& operator[](uint64_t i) const { return data[i]; }
};

// ---------------------------------------------------------------------------
// NTT_info (ntt_info.h:10-67): a device-resident three-prime transform.
// ---------------------------------------------------------------------------
struct NTT_info {
  nn_transform* t = nullptr;
  int NTT_scale;

  NTT_info(int scale = 0) : NTT_scale(scale) {}
  NTT_info(const basic_natural& n, int scale) : NTT_scale(scale) { load(n, scale); }
  NTT_info(const uint64_t* src, uint64_t n, int scale) : NTT_scale(scale) { load(src, n, scale); }
  NTT_info(const NTT_info&) = delete;
  NTT_info& operator=(const NTT_info&) = delete;
  NTT_info(NTT_info&& o) noexcept : t(o.t), NTT_scale(o.NTT_scale) { o.t = nullptr; }
  NTT_info& operator=(NTT_info&& o) noexcept {
    std::swap(t, o.t);
    NTT_scale = o.NTT_scale;
    return *this;
  }
  ~NTT_info() {
    if (t) nn_transform_destroy(nn_gb300::ctx(), t);
  }
  void ensure() {
    if (!t) nn_gb300::check(nn_transform_create(nn_gb300::ctx(), &t), "transform_create");
  }
  // ntt_info.h:147-177, fused with NTT() (ntt_info.h:180-198).
  void load(const uint64_t* src, uint64_t n, int scale) {
    ensure();
    NTT_scale = scale;
    nn_gb300::check(nn_transform_forward_host(nn_gb300::ctx(), t, src, n, scale), "load/NTT");
  }
  void load(const basic_natural& n, int scale) { load(n.data, n.size, scale); }
  void NTT() {}  // the forward transform ran in load()
  // ntt_info.h:224-231
  void mul(const NTT_info& a, const NTT_info& b) {
    ensure();
    NTT_scale = a.NTT_scale;
    nn_gb300::check(nn_transform_pointwise(nn_gb300::ctx(), t, a.t, b.t), "pointwise");
  }
  // INTT (ntt_info.h:200-221) + save (ntt_info.h:237-248) into n.
  void save(basic_natural& n, uint64_t size) {
    const uint64_t L = 1ull << NTT_scale;
    n.resize(std::max(size, L));
    uint64_t w = 0;
    nn_gb300::check(nn_transform_inverse_save_host(nn_gb300::ctx(), t, n.data, size, &w), "INTT/save");
    n.size = w;
  }
};

// ---------------------------------------------------------------------------
// natural (natural.h:16-80)
// ---------------------------------------------------------------------------
struct natural : basic_natural {
  natural(uint64_t n = 0) { data[0] = n; }
  natural(std::string_view sv) { *this = sv; }
  natural(const natural& n) : basic_natural(n) {}
  natural(std::initializer_list<uint64_t> n) : basic_natural(n) {}
  natural(natural&& n) noexcept : basic_natural(std::move(n)) {}

  natural& std() {  // natural.h:82-93
    if (!size) {
      size = 1;
      data[0] = 0;
      return *this;
    }
    while (--size)
      if (data[size]) break;
    ++size;
    return *this;
  }
  natural& operator=(uint64_t n) {
    size = 1;
    data[0] = n;
    return *this;
  }
  natural& operator=(std::string_view sv) {
    if (sv.size() > 1 && sv[0] == '0' && (sv[1] == 'x' || sv[1] == 'X')) {
      sv.remove_prefix(2);
      hex(sv);
    } else {
      dec(sv);
    }
    return *this;
  }
  natural& operator=(const natural& n) {
    basic_natural::operator=(n);
    return *this;
  }
  natural& operator=(natural&& n) noexcept {
    basic_natural::operator=(std::move(n));
    return *this;
  }
  natural& hex(std::string_view sv);
  natural& dec(std::string_view sv);
  natural& _shl(const natural* ap, uint64_t b);
  natural& _shr(const natural* ap, uint64_t b);
  natural& _add(const natural* ap, const natural* bp);
  natural& _sub(const natural* ap, const natural* bp);
  natural& _mul_base(const natural* ap, const natural* bp);
  natural& _sqr_base(const natural* p);
  natural& _mul(const natural* ap, const natural* bp);
  natural& _sqr(const natural* p);
  natural& _div(const natural* ap, const natural* bp, natural* r);
  void _dec_split(int i, natural& hi, natural& lo) const;
  void _format_dec(std::string& out, int i, bool first) const;
};

inline bool operator<(const natural& a, const natural& b) {  // natural.h:145-153
  if (a.size != b.size) return a.size < b.size;
  for (uint64_t i = a.size; i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i];
  return false;
}
inline bool operator>(const natural& a, const natural& b) { return b < a; }
inline bool operator<=(const natural& a, const natural& b) { return !(b < a); }
inline bool operator>=(const natural& a, const natural& b) { return !(a < b); }
inline bool operator==(const natural& a, const natural& b) {
  if (a.size != b.size) return false;
  return std::memcmp(a.data, b.data, a.size * 8) == 0;
}
inline bool operator!=(const natural& a, const natural& b) { return !(a == b); }

// natural.h:181-242
inline natural operator|(const natural& x, const natural& y) {
  const natural *a = &x, *b = &y;
  if (a->size < b->size) std::swap(a, b);
  natural d;
  d.resize(a->size);
  for (uint64_t i = 0; i < b->size; ++i) d[i] = (*a)[i] | (*b)[i];
  std::memcpy(d.data + b->size, a->data + b->size, (a->size - b->size) * 8);
  return d;
}
inline natural operator^(const natural& x, const natural& y) {
  const natural *a = &x, *b = &y;
  if (a->size < b->size) std::swap(a, b);
  natural d;
  d.resize(a->size);
  for (uint64_t i = 0; i < b->size; ++i) d[i] = (*a)[i] ^ (*b)[i];
  std::memcpy(d.data + b->size, a->data + b->size, (a->size - b->size) * 8);
  return d.std();
}
inline natural operator&(const natural& x, const natural& y) {
  uint64_t s = std::min(x.size, y.size);
  natural d;
  d.resize(s);
  for (uint64_t i = 0; i < s; ++i) d[i] = x[i] & y[i];
  return d.std();
}
inline natural& operator|=(natural& a, const natural& b) { return a = a | b; }
inline natural& operator^=(natural& a, const natural& b) { return a = a ^ b; }
inline natural& operator&=(natural& a, const natural& b) { return a = a & b; }

inline natural& natural::_shl(const natural* ap, uint64_t b) {  // natural.h:244-262
  if (ap->size == 1 && (*ap)[0] == 0) {
    *this = 0;
    return *this;
  }
  uint64_t as = ap->size, n = b >> 6;
  b &= 63;
  if (b == 0) {
    resize(as + n);
    nn_gb300::copy_n(data + n, ap->data, as);
    std::memset(data, 0, n * 8);
    return *this;
  }
  resize(as + n + 1);
  nn_gb300::shl_n((unsigned)b, as, ap->data, data + n);
  std::memset(data, 0, n * 8);
  return std();
}
inline natural& natural::_shr(const natural* ap, uint64_t b) {  // natural.h:275-290
  uint64_t as = ap->size, n = b >> 6;
  if (as <= n) {
    *this = 0;
    return *this;
  }
  b &= 63;
  resize(as - n);
  if (b == 0) {
    nn_gb300::copy_n(data, ap->data + n, as - n);
    return *this;
  }
  nn_gb300::shr_n((unsigned)b, as - n, ap->data + n, data);
  return std();
}
inline natural& operator<<=(natural& a, uint64_t b) { return a._shl(&a, b); }
inline natural operator<<(const natural& a, uint64_t b) {
  natural d;
  d._shl(&a, b);
  return d;
}
inline natural& operator>>=(natural& a, uint64_t b) { return a._shr(&a, b); }
inline natural operator>>(const natural& a, uint64_t b) {
  natural d;
  d._shr(&a, b);
  return d;
}

inline natural& natural::_add(const natural* ap, const natural* bp) {  // natural.h:303-311
  if (ap->size < bp->size) std::swap(ap, bp);
  uint64_t as = ap->size, bs = bp->size;
  if (this == bp && this != ap) {
    natural t(*bp);
    return _add(ap, &t);
  }
  resize(as + 1);
  data[as] = nn_gb300::add(data, ap->data, as, bp->data, bs);
  return std();
}
inline natural& operator+=(natural& a, const natural& b) { return a._add(&a, &b); }
inline natural operator+(const natural& a, const natural& b) {
  natural d;
  d._add(&a, &b);
  return d;
}

inline natural& natural::_sub(const natural* ap, const natural* bp) {  // natural.h:324-343: |a - b|
  if (ap->size < bp->size) std::swap(ap, bp);
  uint64_t as = ap->size, bs = bp->size;
  if (this == bp && this != ap) {
    natural t(*bp);
    return _sub(ap, &t);
  }
  if (as == bs) {
    while (--bs)
      if ((*ap)[bs] != (*bp)[bs]) break;
    if ((*ap)[bs] < (*bp)[bs]) std::swap(ap, bp);
    if (this == bp) {
      natural t(*bp);
      return _sub(ap, &t);
    }
    resize(++bs);
    nn_gb300::sub_n(bs, data, ap->data, bp->data);
  } else {
    resize(as);
    nn_gb300::sub(data, ap->data, as, bp->data, bs);
  }
  return std();
}
inline natural& operator-=(natural& a, const natural& b) { return a._sub(&a, &b); }
inline natural operator-(const natural& a, const natural& b) {
  natural d;
  d._sub(&a, &b);
  return d;
}

// natural.h:356-369 -> GPU schoolbook
inline natural& natural::_mul_base(const natural* ap, const natural* bp) {
  natural ans;
  ans.resize(ap->size + bp->size);
  nn_gb300::check(nn_mul_base_host(nn_gb300::ctx(), ans.data, ap->data, ap->size, bp->data, bp->size), "mul_base");
  *this = std::move(ans);
  return std();
}
inline natural& natural::_sqr_base(const natural* p) { return _mul_base(p, p); }

inline int get_NTT_scale(uint64_t n1, uint64_t n2) { return 64 - std::countl_zero(n1 + n2 - 2); }  // natural.h:384

// natural.h:444-450 (with _mul_NTT's split, natural.h:391-419, inside nn_mul)
inline natural& natural::_mul(const natural* ap, const natural* bp) {
  natural ans;
  ans.resize(ap->size + bp->size);
  uint64_t n = 0;
  nn_gb300::check(nn_mul_host(nn_gb300::ctx(), ans.data, &n, ap->data, ap->size, bp->data, bp->size), "mul");
  ans.size = n;
  *this = std::move(ans);
  return *this;
}
// natural.h:529-535
inline natural& natural::_sqr(const natural* p) {
  natural ans;
  ans.resize(p->size * 2);
  uint64_t n = 0;
  nn_gb300::check(nn_sqr_host(nn_gb300::ctx(), ans.data, &n, p->data, p->size), "sqr");
  ans.size = n;
  *this = std::move(ans);
  return *this;
}
inline natural& operator*=(natural& a, const natural& b) { return a._mul(&a, &b); }
inline natural operator*(const natural& a, const natural& b) {
  natural d;
  d._mul(&a, &b);
  return d;
}
inline natural sqr(const natural& a) {
  natural d;
  d._sqr(&a);
  return d;
}
inline natural pow(const natural& b, uint64_t e) {  // natural.h:554-564
  if (e == 0) return 1;
  if (e == 1 || b < 2) return b;
  natural p = pow(b, e >> 1);
  p._sqr(&p);
  if (e & 1) p *= b;
  return p;
}

// Cached-transform products (natural.h:452-527).
inline void mul_save_NTT_info(natural& d, const natural& a, const natural& b, NTT_info& ni_a) {
  if (ni_a.NTT_scale < nn_gb300::NTTscale_threshold) {
    d._mul_base(&a, &b);
    ni_a.NTT_scale = 0;
    return;
  }
  const uint64_t size = a.size + b.size;
  ni_a.load(a, ni_a.NTT_scale);
  NTT_info ni_b(b, ni_a.NTT_scale);
  ni_b.mul(ni_a, ni_b);
  ni_b.save(d, size);
  d.std();
}
inline void mul_save_NTT_info(natural& d, const natural& a, const natural& b, NTT_info& ni_a, NTT_info& ni_b) {
  if (ni_a.NTT_scale < nn_gb300::NTTscale_threshold) {
    d._mul_base(&a, &b);
    ni_a.NTT_scale = 0;
    ni_b.NTT_scale = 0;
    return;
  }
  const uint64_t size = a.size + b.size;
  ni_a.load(a, ni_a.NTT_scale);
  ni_b.load(b, ni_a.NTT_scale);
  NTT_info ni;
  ni.mul(ni_a, ni_b);
  ni.save(d, size);
  d.std();
}
inline void sqr_save_NTT_info(natural& d, const natural& a, NTT_info& ni_a) {
  if (ni_a.NTT_scale < nn_gb300::NTTscale_threshold) {
    d._sqr_base(&a);
    ni_a.NTT_scale = 0;
    return;
  }
  const uint64_t size = a.size * 2;
  ni_a.load(a, ni_a.NTT_scale);
  NTT_info ni_b;
  ni_b.mul(ni_a, ni_a);
  ni_b.save(d, size);
  d.std();
}
inline void mul_load_NTT_info(natural& d, const natural& a, const natural& b, const NTT_info& ni_a) {
  if (ni_a.NTT_scale == 0) {
    d._mul_base(&a, &b);
    return;
  }
  const uint64_t size = a.size + b.size;
  NTT_info ni_b(b, ni_a.NTT_scale);
  ni_b.mul(ni_a, ni_b);
  ni_b.save(d, size);
  d.std();
}
inline void mul_load_NTT_info(natural& d, const natural& a, const natural& b, const NTT_info& ni_a,
                              const NTT_info& ni_b) {
  if (ni_a.NTT_scale == 0) {
    d._mul_base(&a, &b);
    return;
  }
  const uint64_t size = a.size + b.size;
  NTT_info ni;
  ni.mul(ni_a, ni_b);
  ni.save(d, size);
  d.std();
}

// natural.h:566-573 — serial 128/64 division by a one-limb divisor (host glue).
inline uint64_t div_base(const natural& a, uint64_t b, natural& q) {
  natural t;
  t.resize(a.size);
  uint64_t r = 0;
  for (uint64_t i = a.size; i-- > 0;) t[i] = nn_gb300::div_128(a[i], r, b, &r);
  q = std::move(t);
  q.std();
  return r;
}

// Newton reciprocal for decimal output; divs has top limb 1 (natural.h:575-617).
inline natural reciprocal(const natural& divs, uint64_t divd_size) {
  using namespace nn_gb300;
  const uint64_t expected_acc = divd_size + 1 - divs.size;
  natural ans = ((1ull << 63) | (divs[divs.size - 2] >> 1)) + 1;  // uint64_t arithmetic, may wrap to 0
  ans[0] = ans[0] == 0 ? 1ull << 63 : div_128(0, 1ull << 63, ans[0]);
  while (true) {
    uint64_t nxt_acc = 0, cur_acc = ans.size;
    if (cur_acc >= expected_acc + 1) {
      ans >>= (cur_acc - expected_acc) << 6;
      return ans;
    }
    natural tmp;
    if (divs.size > 2 * cur_acc + 1)
      tmp._shr(&divs, (divs.size - 2 * cur_acc - 1) << 6);
    else
      tmp._shl(&divs, (2 * cur_acc + 1 - divs.size) << 6);
    NTT_info ni_ans(get_NTT_scale(tmp.size, 1));
    mul_save_NTT_info(tmp, ans, tmp, ni_ans);
    tmp.size -= cur_acc;
    for (uint64_t i = 0; i < tmp.size; ++i) tmp[i] = ~tmp[i + cur_acc];
    tmp.std();
    const int l_zero = std::countl_zero(tmp[tmp.size - 1]);
    nxt_acc = std::min(2 * cur_acc, (2 * cur_acc - tmp.size) * 2 + ((uint64_t)(l_zero + 31) >> 5));
    if (nxt_acc == NTTdiv_threshold) nxt_acc = NTTdiv_threshold - 1;
    tmp >>= (2 * cur_acc - nxt_acc) << 6;
    if (tmp == 0) tmp = 1;
    if (nxt_acc < cur_acc) throw precondition_broken();  // natural.h:614 would shift by a negative count
    mul_load_NTT_info(tmp, ans, tmp, ni_ans);
    ans <<= (nxt_acc - cur_acc) << 6;
    if (tmp.size < cur_acc || tmp.size - cur_acc > ans.size) throw precondition_broken();  // natural.h:615
    add(ans.data, ans.data, ans.size, tmp.data + cur_acc, tmp.size - cur_acc);
  }
}

// Newton reciprocal for division; divisor has top limb 1; leaves the last
// divisor transform in ni_divisor (natural.h:619-687).
inline natural reciprocal(const natural& divisor, uint64_t dividend_size, NTT_info& ni_divisor) {
  using namespace nn_gb300;
  const uint64_t expected_acc = dividend_size + 1 - divisor.size;
  natural ans = ((1ull << 63) | (divisor[divisor.size - 2] >> 1)) + 1;  // uint64_t arithmetic
  ans[0] = ans[0] ? div_128(0, 1ull << 63, ans[0]) : 1ull << 63;
  for (uint64_t i = 1; i < divisor.size; i *= 2) {
    const uint64_t prev_acc = ans.size;
    uint64_t seg = 2 * prev_acc + 1;
    if (2 * i >= divisor.size) seg = divisor.size;
    const uint64_t* dseg = divisor.data + divisor.size - seg;
    natural tmp;
    NTT_info ni_ans;
    if (2 * i <= NTTdiv_threshold) {
      tmp.resize(seg + prev_acc);
      check(nn_mul_base_host(ctx(), tmp.data, dseg, seg, ans.data, prev_acc), "mul_base");
      tmp.std();
    } else {
      const int s = get_NTT_scale(i, i);
      ni_ans.load(ans, s);
      ni_divisor.load(dseg, seg, s);
      NTT_info ni_tmp;
      ni_tmp.mul(ni_ans, ni_divisor);
      ni_tmp.save(tmp, seg + prev_acc);
      tmp.std();
    }
    uint64_t n_shl = seg - 1 - prev_acc;
    while (tmp.size > n_shl + 1 && ~tmp[tmp.size - 1] == 0) tmp.size -= 1;
    const int l_zero = std::countl_zero(~tmp[tmp.size - 1]);
    uint64_t cur_acc = std::min(2 * prev_acc, (2 * prev_acc - tmp.size + n_shl) * 2 + ((uint64_t)(l_zero + 31) >> 5));
    if (cur_acc == NTTdiv_threshold) cur_acc -= 1;
    n_shl += 2 * prev_acc - cur_acc;
    if (tmp.size <= n_shl) {
      tmp = 1;
    } else {
      tmp.size -= n_shl;
      for (uint64_t k = 0; k < tmp.size; ++k) tmp[k] = ~tmp[k + n_shl];
      tmp.std();
    }
    mul_load_NTT_info(tmp, ans, tmp, ni_ans);
    tmp >>= prev_acc << 6;
    if (cur_acc < prev_acc) throw precondition_broken();  // natural.h:670-672: negative memset length
    const uint64_t inc_acc = cur_acc - prev_acc;
    if (inc_acc < tmp.size && tmp.size - inc_acc > prev_acc) throw precondition_broken();  // natural.h:676
    const uint64_t have = tmp.size;
    tmp.resize(std::max(cur_acc, have));
    tmp.size = have;
    if (inc_acc >= tmp.size) {
      std::memset(tmp.data + tmp.size, 0, 8 * (inc_acc - tmp.size));
      std::memcpy(tmp.data + inc_acc, ans.data, 8 * prev_acc);
    } else {
      add(tmp.data + inc_acc, ans.data, prev_acc, tmp.data + inc_acc, tmp.size - inc_acc);
    }
    tmp.resize(cur_acc);
    ans = std::move(tmp);
    if (cur_acc >= expected_acc + 1) {
      ans >>= (cur_acc - expected_acc) << 6;
      return ans;
    }
  }
  ans >>= 64;
  return ans;
}

// Block division with a wrapped b*q product and fix-up (natural.h:689-747).
inline void div_iterative(const natural& divd, const natural& divs, natural& q, natural& r) {
  using namespace nn_gb300;
  const unsigned n_shl = (unsigned)(std::countl_zero(divs[divs.size - 1]) + 1) & 63;
  natural b = divs << n_shl;
  r = divd << n_shl;
  NTT_info ni_b;
  natural rec = reciprocal(b, r.size, ni_b);
  NTT_info ni_rec(get_NTT_scale(rec.size, rec.size));
  const int NTT_scale_b = get_NTT_scale(b.size, 1);
  const uint64_t NTT_size_b = 1ull << NTT_scale_b;
  if (ni_b.NTT_scale != NTT_scale_b && NTT_scale_b >= NTTscale_threshold - 1) ni_b.load(b, NTT_scale_b);
  q.resize(r.size - b.size + 1);
  std::memset(q.data, 0, 8 * q.size);
  natural tmp;
  bool first = true;
  while (true) {
    uint64_t idx = 0;
    if (r.size > rec.size + b.size - 1) idx = r.size - rec.size - b.size + 1;
    if (first)
      mul_save_NTT_info(tmp, rec, r >> ((idx + b.size - 1) << 6), ni_rec);
    else
      mul_load_NTT_info(tmp, rec, r >> ((idx + b.size - 1) << 6), ni_rec);
    first = false;
    tmp >>= rec.size << 6;
    add(q.data + idx, q.data + idx, q.size - idx, tmp.data, tmp.size);
    mul_load_NTT_info(tmp, b, tmp, ni_b);
    if (r.size < idx || r.size - idx < tmp.size) throw precondition_broken();  // natural.h:724
    sub(r.data + idx, r.data + idx, r.size - idx, tmp.data, tmp.size);
    r.std();
    if (ni_b.NTT_scale) {
      if (r.size - idx > NTT_size_b) {
        int cf = add(r.data + idx, r.data + idx, NTT_size_b, r.data + idx + NTT_size_b, r.size - idx - NTT_size_b);
        add_1(NTT_size_b, r.data + idx, r.data + idx, cf);
        r.resize(idx + NTT_size_b);
      }
      if (r.size == idx + NTT_size_b && r[r.size - 1] >> 63) r.resize(idx);
      r.std();
    }
    if (idx == 0) break;
  }
  for (int guard = 0; r >= b; ++guard) {
    if (guard > 64) throw precondition_broken();  // block estimates are meant to be within a few units
    q += 1;
    r -= b;
  }
  r >>= n_shl;
}

// Exact Newton division (no counterpart in the reference), for the inputs on
// which the reference's own division breaks.  With the divisor normalised
// (top bit set, n limbs), R_k = floor(B^(n+k) / d) is built by recursive
// doubling: from X = R_h, h = ceil(k/2), and eps = B^(n+h) - d X (< d),
//   Z = X B^(k-h) + floor(eps X / B^(n+2h-k))
// underestimates R_k by less than 2, and exact checks against d Z finish it.
// Then q' = floor(a R_k / B^(n+k)) with k = m - n + 1 is q or q - 1.
// Every product runs on the GPU; the host adds, shifts and compares.
namespace nn_gb300 {
inline natural power_of_B(uint64_t e) {
  natural p;
  p.resize(e + 1);
  std::memset(p.data, 0, 8 * e);
  p[e] = 1;
  return p;
}
// floor(B^(n+k) / d) for normalised d of n >= 2 limbs.
inline natural recip_floor(const natural& d, uint64_t k) {
  const uint64_t n = d.size;
  if (k == 0) {  // B^n / d lies in (1, 2]
    natural half = power_of_B(n - 1) << 63;
    return natural(d == half ? 2 : 1);
  }
  if (k == 1) {  // B + floor(B E / d), E = B^n - d < d
    natural E = power_of_B(n) - d;
    uint64_t e_hi = E.size == n ? E[n - 1] : 0, e_lo = E.size >= n - 1 ? E[n - 2] : 0;
    if (E.size < n - 1) e_lo = 0;
    unsigned __int128 num = ((unsigned __int128)e_hi << 64) | e_lo;
    uint64_t t = (uint64_t)(num / ((unsigned __int128)d[n - 1] + 1));  // underestimate
    natural S = (E << 64) - d * natural(t);
    for (int g = 0; S >= d; ++g) {
      if (g > 8) throw std::runtime_error("natural_gb300: reciprocal base case did not converge");
      t += 1;
      S -= d;
    }
    natural Y = power_of_B(1);
    Y += natural(t);
    return Y;
  }
  const uint64_t h = (k + 1) / 2;
  natural X = recip_floor(d, h);
  natural eps = power_of_B(n + h) - d * X;
  natural Z = (X << (64 * (k - h))) + ((eps * X) >> (64 * (n + 2 * h - k)));
  natural T = d * Z;
  const natural top = power_of_B(n + k);
  for (int g = 0; T > top; ++g) {  // cannot happen: Z underestimates
    if (g > 8) throw std::runtime_error("natural_gb300: reciprocal overshoot");
    Z -= 1;
    T -= d;
  }
  natural E = top - T;
  for (int g = 0; E >= d; ++g) {
    if (g > 8) throw std::runtime_error("natural_gb300: reciprocal did not converge");
    Z += 1;
    E -= d;
  }
  return Z;
}
// q = floor(a / b), r = a mod b for b of at least two limbs.
inline void div_newton_exact(const natural& a, const natural& b, natural& q, natural& r) {
  const unsigned sh = (unsigned)std::countl_zero(b[b.size - 1]);
  natural d = b << sh, x = a << sh;
  if (x < d) {
    q = 0;
    r = a;
    return;
  }
  const uint64_t n = d.size, k = x.size - n + 1;
  natural R = recip_floor(d, k);
  q = (x * R) >> (64 * (n + k));
  natural rr = x - q * d;  // q <= true quotient, so this is x - q d itself
  for (int g = 0; rr >= d; ++g) {
    if (g > 8) throw std::runtime_error("natural_gb300: quotient correction did not converge");
    q += 1;
    rr -= d;
  }
  r = rr >> sh;
}
}  // namespace nn_gb300

inline natural& natural::_div(const natural* ap, const natural* bp, natural* r) {  // natural.h:749-769
  if (*bp == 0) {
    *this = *ap == 0 ? 1ull : 0ull;
    *r = 0;
    return *this;
  }
  if (*ap < *bp) {
    *r = *ap;
    *this = 0;
    return *this;
  }
  if (bp->size == 1) {
    uint64_t b0 = (*bp)[0];
    natural q;
    *r = div_base(*ap, b0, q);
    *this = std::move(q);
    return *this;
  }
  natural a(*ap), b(*bp), q, rr;
  try {
    div_iterative(a, b, q, rr);
  } catch (const nn_gb300::precondition_broken&) {
    nn_gb300::div_newton_exact(a, b, q, rr);
  }
  *this = std::move(q);
  *r = std::move(rr);
  return *this;
}
inline natural& operator/=(natural& a, const natural& b) {
  natural r;
  return a._div(&a, &b, &r);
}
inline natural operator/(const natural& a, const natural& b) {
  natural q, r;
  q._div(&a, &b, &r);
  return q;
}
inline natural& operator%=(natural& a, const natural& b) {
  natural q;
  q._div(&a, &b, &a);
  return a;
}
inline natural operator%(const natural& a, const natural& b) {
  natural q, r;
  q._div(&a, &b, &r);
  return r;
}

// natural.h:795-839.  n! = 2^e2 * prod over odd primes p of p^e_p, built by
// Horner's rule over the bits of the exponents: at bit i, ans = ans^2 times
// the product of the primes whose exponent has bit i set (a balanced product
// through a min-queue).  Where no odd prime's exponent has bit i set (n = 9:
// 3^4 5 7) the reference reads the top of an empty queue; here that factor is
// 1, the value the formula means.
inline natural factorial(uint64_t n) {
  if (n <= 1) return 1;
  if (n == 2) return 2;
  std::vector<char> is_prime(n + 1, 1);
  std::vector<uint64_t> prime, prime_exp;
  for (uint64_t i = 2; i <= n; ++i) {
    if (is_prime[i]) {
      prime.push_back(i);
      uint64_t e = 0, m = n;
      while (m) e += m /= i;
      prime_exp.push_back(e);
    }
    for (uint64_t j = 0; j < prime.size() && i * prime[j] <= n; ++j) {
      is_prime[i * prime[j]] = 0;
      if (i % prime[j] == 0) break;
    }
  }
  natural ans = 1;
  for (int i = 63 - std::countl_zero(prime_exp[1]); i >= 0; --i) {
    std::priority_queue<natural, std::vector<natural>, std::greater<natural>> pq;
    for (uint64_t j = 1; j < prime.size(); ++j) {
      if (prime_exp[j] < (1ull << i)) break;
      if (prime_exp[j] & (1ull << i)) pq.push(prime[j]);
    }
    while (pq.size() > 1) {
      natural n1 = pq.top();
      pq.pop();
      natural n2 = pq.top();
      pq.pop();
      pq.push(n1 * n2);
    }
    ans = sqr(ans);
    if (!pq.empty()) ans *= pq.top();
  }
  ans <<= prime_exp[0];
  return ans;
}

// Binary splitting for e (natural.h:841-857).
inline void calc_e(natural& num, natural& den, uint64_t begin, uint64_t end) {
  if (end - begin == 2) {
    num = end;
    den = begin + 1;
    if (begin) den *= begin;
    return;
  }
  natural num1, den1;
  calc_e(num, den, begin, (begin + end) >> 1);
  calc_e(num1, den1, (begin + end) >> 1, end);
  NTT_info ni_den1;
  ni_den1.NTT_scale = get_NTT_scale(std::max(den.size, num.size), den1.size);
  mul_save_NTT_info(num, den1, num, ni_den1);
  mul_load_NTT_info(den, den1, den, ni_den1);
  num += num1;
}

// Newton iteration for sqrt(10005) as a fraction (natural.h:859-872).
inline void sqrt_10005(natural& num, natural& den, uint64_t acc) {
  num = 4001;
  den = 40;
  natural cache1, cache2;
  while (num.size + den.size - 2 < acc) {
    NTT_info ni_num, ni_den;
    ni_num.NTT_scale = ni_den.NTT_scale = get_NTT_scale(num.size, num.size);
    sqr_save_NTT_info(cache1, den, ni_den);
    sqr_save_NTT_info(cache2, num, ni_num);
    mul_load_NTT_info(den, num, den, ni_num, ni_den);
    den <<= 1;
    num = cache1 * 10005 + cache2;
  }
}

// Chudnovsky binary splitting (natural.h:874-902).
inline void calc_pi(natural& num, natural& den, natural& numc, uint64_t begin, uint64_t end) {
  if (end - begin == 1) {
    den = begin;
    den = den * den * den * 0x26dd041d878000ull;
    numc = 2 * begin - 1;
    numc *= 6 * begin - 1;
    numc *= 6 * begin - 5;
    num = begin;
    num = (natural(0x207e2da6ull) * num + 0xcf6371) * numc;
    return;
  }
  natural num1, den1, numc1;
  calc_pi(num, den, numc, begin, (begin + end) >> 1);
  calc_pi(num1, den1, numc1, (begin + end) >> 1, end);
  if (end - begin == 2) {
    num = numc * num1 - num * den1;
    den = den * den1;
    numc = numc * numc1;
    return;
  }
  NTT_info ni_den1, ni_numc;
  ni_den1.NTT_scale = get_NTT_scale(std::max(den.size, num.size), den1.size);
  mul_save_NTT_info(num, den1, num, ni_den1);
  mul_load_NTT_info(den, den1, den, ni_den1);
  ni_numc.NTT_scale = get_NTT_scale(std::max(numc1.size, num1.size), numc.size);
  mul_save_NTT_info(num1, numc, num1, ni_numc);
  mul_load_NTT_info(numc, numc, numc1, ni_numc);
  num = num + num1;
}

// ---------------------------------------------------------------------------
// Decimal I/O (natural.h:904-1093)
// ---------------------------------------------------------------------------
namespace nn_gb300 {
constexpr uint64_t dec_length = 18, dec_base_0 = 1000000000000000000ull;
struct DecCache {  // natural.h:905-906 (globals there)
  natural base[64], base_r[64];
  NTT_info ni_base[64], ni_base_r[64];
  DecCache() {
    base[0] = dec_base_0;
    for (int i = 1; i < 64; ++i) base[i] = 0;
  }
};
// One cache per context (its transforms live on that context's device);
// caches are never destroyed, so they outlive every caller.
inline DecCache& dec_cache() {
  static std::vector<std::pair<nn_context*, DecCache*>> caches;
  nn_context* c = ctx();
  for (auto& e : caches)
    if (e.first == c) return *e.second;
  caches.emplace_back(c, new DecCache);
  return *caches.back().second;
}
// natural.h:909-923
inline void calc_dec_base(int i) {
  DecCache& C = dec_cache();
  if (!(C.base[i + 1] == 0)) return;
  C.ni_base[i].NTT_scale = get_NTT_scale(C.base[i].size, C.base[i].size);
  sqr_save_NTT_info(C.base[i + 1], C.base[i], C.ni_base[i]);
  const unsigned n_shl = (unsigned)(std::countl_zero(C.base[i][C.base[i].size - 1]) + 1) & 63;
  C.base_r[i] = reciprocal(C.base[i] << n_shl, C.base[i].size * 2 + 1);
  C.ni_base_r[i].NTT_scale = get_NTT_scale(C.base_r[i].size, C.base[i].size + 2);
  if (C.ni_base_r[i].NTT_scale < NTTscale_threshold)
    C.ni_base_r[i].NTT_scale = 0;
  else
    C.ni_base_r[i].load(C.base_r[i], C.ni_base_r[i].NTT_scale);
}
inline int dec_init(const natural& n) {  // natural.h:1013-1018
  int i = 0;
  for (; n >= dec_cache().base[i]; ++i) calc_dec_base(i);
  return i - 1;
}
}  // namespace nn_gb300

inline natural& natural::hex(std::string_view sv) {  // natural.h:121-143
  if (sv.empty()) {
    *this = 0;
    return *this;
  }
  resize((sv.size() + 15) >> 4);
  uint64_t j = size;
  std::size_t pos = sv.size();
  for (uint64_t k = 0; k < j; ++k) {
    uint64_t x = 0;
    std::size_t lo = pos >= 16 ? pos - 16 : 0;
    for (std::size_t t = lo; t < pos; ++t) {
      char c = sv[t];
      unsigned v = c <= '9' ? c - '0' : (c | 32) - 'a' + 10;
      x = x << 4 | v;
    }
    data[k] = x;
    pos = lo;
  }
  return std();
}
inline natural& natural::dec(std::string_view sv) {  // natural.h:925-941
  using namespace nn_gb300;
  if (sv.empty()) {  // the reference's index arithmetic below underflows (i = 63) on ""
    *this = 0;
    return *this;
  }
  int i = 63 - std::countl_zero((uint64_t)((sv.size() + dec_length - 1) / dec_length - 1));
  if (i == -1) {
    *this = 0;
    for (char c : sv) data[0] = data[0] * 10 + (c - '0');
    return *this;
  }
  if (dec_cache().base[i] == 0)
    for (int j = 0; j < i; ++j) calc_dec_base(j);
  natural hi, lo;
  hi.dec(sv.substr(0, sv.size() - (dec_length << i)));
  lo.dec(sv.substr(sv.size() - (dec_length << i)));
  *this = hi * dec_cache().base[i] + lo;
  return *this;
}
// natural.h:953-967
inline void natural::_dec_split(int i, natural& hi, natural& lo) const {
  using namespace nn_gb300;
  DecCache& C = dec_cache();
  if (i == 0) {
    lo = div_base(*this, dec_base_0, hi);
    return;
  }
  const unsigned n_shl = (unsigned)(std::countl_zero(C.base[i][C.base[i].size - 1]) + 1) & 63;
  mul_load_NTT_info(hi, C.base_r[i], *this >> ((C.base[i].size - 1) << 6), C.ni_base_r[i]);
  hi >>= ((C.base[i].size + 2) << 6) - n_shl;
  mul_load_NTT_info(lo, C.base[i], hi, C.ni_base[i]);
  lo = *this - lo;
  while (lo >= C.base[i]) {
    hi += 1;
    lo -= C.base[i];
  }
}
// natural.h:994-1011 (into a string)
inline void natural::_format_dec(std::string& out, int i, bool first) const {
  if (i == -1) {
    char buf[32];
    std::snprintf(buf, sizeof buf, first ? "%llu" : "%018llu", (unsigned long long)data[0]);
    out += buf;
    return;
  }
  natural hi, lo;
  _dec_split(i, hi, lo);
  if (first && hi == 0) {
    lo._format_dec(out, i - 1, true);
    return;
  }
  hi._format_dec(out, i - 1, first);
  lo._format_dec(out, i - 1, false);
}
inline std::string to_dec_string(const natural& n) {
  std::string s;
  n._format_dec(s, nn_gb300::dec_init(n), true);
  return s;
}
inline std::string to_hex_string(const natural& n, bool upper = false) {
  std::string s;
  char buf[24];
  uint64_t i = n.size - 1;
  std::snprintf(buf, sizeof buf, upper ? "%llX" : "%llx", (unsigned long long)n[i]);
  s += buf;
  while (i--) {
    std::snprintf(buf, sizeof buf, upper ? "%016llX" : "%016llx", (unsigned long long)n[i]);
    s += buf;
  }
  return s;
}

inline std::ostream& operator<<(std::ostream& os, const natural& n) {  // natural.h:1020-1039
  if (os.flags() & std::ios::hex)
    os << to_hex_string(n, (os.flags() & std::ios::uppercase) != 0);
  else
    os << to_dec_string(n);
  return os;
}
inline std::istream& operator>>(std::istream& is, natural& n) {  // natural.h:943-951
  std::string s;
  is >> s;
  if (is.flags() & std::ios::hex)
    n.hex(s);
  else
    n.dec(s);
  return is;
}

template <>
struct std::formatter<natural> {  // natural.h:1041-1093
  bool prefix = false, upper = false;
  char base = 'd';
  constexpr auto parse(std::format_parse_context& ctx) {
    auto it = ctx.begin();
    if (it == ctx.end() || *it == '}') return it;
    if (*it == '#') {
      prefix = true;
      ++it;
    }
    if (*it == '}') return it;
    upper = *it >= 'A' && *it <= 'Z';
    base = (char)(*it | 32);
    if (base != 'd' && base != 'x') throw std::format_error("Invalid format specifier for natural.");
    ++it;
    if (*it != '}') throw std::format_error("Invalid format specifier for natural.");
    return it;
  }
  auto format(const natural& n, std::format_context& ctx) const {
    std::string s = base == 'x' ? (prefix ? (upper ? "0X" : "0x") : "") + to_hex_string(n, upper) : to_dec_string(n);
    return std::copy(s.begin(), s.end(), ctx.out());
  }
};

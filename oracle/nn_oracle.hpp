// nn_oracle.hpp — TEST INFRASTRUCTURE ONLY (the oracle).
//
// A portable, single-threaded CPU restatement of Natural_Number's big-number
// multiply path: limb primitives (asm.h), the schoolbook/Karatsuba base case
// (base.h), the three-prime NTT engine (ntt_info.h), and the natural-level
// dispatch, Newton-reciprocal division, pi/e binary splitting and decimal
// output (natural.h).  Every function names the reference file:line whose
// behaviour it restates.  The reference's x86-64 assembly kernels are
// restated with `unsigned __int128` so this builds on aarch64 and x86-64 alike.
//
// Only the test-suite, the smoke check and the bench's CPU-baseline leg may
// link this; the GPU product never calls it.
//
// Parity pin: outputs are checked against fixtures produced by the reference
// itself (tests/golden/, generated by tests/golden/make_golden.py from the
// reference compiled by oracle/build_ref.sh).
#pragma once

#include <algorithm>
#include <bit>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <queue>
#include <string>
#include <vector>

namespace nno {

using u64 = std::uint64_t;
using i64 = std::int64_t;
using u128 = unsigned __int128;

static inline u64 hi64(u128 x) { return (u64)(x >> 64); }

// Thrown where the reference's Newton division would break one of its own
// size preconditions (it then reads or copies out of bounds).
struct PreconditionBroken {};
inline unsigned long long& fallback_count() {
  static unsigned long long n = 0;
  return n;
}

// ---------------------------------------------------------------------------
// Limb primitives (asm.h:7-61; asmLinux.asm:7-344, 720-751)
// ---------------------------------------------------------------------------

// d = a + b over n limbs, returns carry (asmAdd0, asmLinux.asm:7-28).
static inline int add_n(u64 n, u64* d, const u64* a, const u64* b) {
  u64 c = 0;
  for (u64 i = 0; i < n; ++i) {
    u128 s = (u128)a[i] + b[i] + c;
    d[i] = (u64)s;
    c = (u64)(s >> 64);
  }
  return (int)c;
}

// d = s + cf over n limbs; once the carry dies the rest is copied
// (asmAdd1, asmLinux.asm:30-62).
static inline int add_1(u64 n, const u64* s, u64* d, int cf) {
  u64 i = 0;
  for (; i < n && cf; ++i) {
    d[i] = s[i] + 1;
    cf = d[i] == 0;
  }
  if (i < n && d != s) std::memmove(d + i, s + i, (n - i) * sizeof(u64));
  return cf;
}

// d = a - b over n limbs, returns borrow (asmSub0, asmLinux.asm:64-85).
static inline int sub_n(u64 n, u64* d, const u64* a, const u64* b) {
  u64 br = 0;
  for (u64 i = 0; i < n; ++i) {
    u64 x = a[i], y = b[i];
    u64 t = x - y;
    u64 b1 = x < y;
    u64 r = t - br;
    u64 b2 = t < br;
    d[i] = r;
    br = b1 | b2;
  }
  return (int)br;
}

// d = s - cf (asmSub1, asmLinux.asm:87-119).
static inline int sub_1(u64 n, const u64* s, u64* d, int cf) {
  u64 i = 0;
  for (; i < n && cf; ++i) {
    u64 v = s[i];
    d[i] = v - 1;
    cf = v == 0;
  }
  if (i < n && d != s) std::memmove(d + i, s + i, (n - i) * sizeof(u64));
  return cf;
}

// d[0..n] = s << cl, 1 <= cl <= 63, top-down so d >= s may overlap
// (asmShl, asmLinux.asm:121-139).
static inline void shl_n(unsigned cl, u64 n, const u64* s, u64* d) {
  u64 carry = 0;
  for (u64 i = n; i-- > 0;) {
    u64 x = s[i];
    d[i + 1] = (carry << cl) | (x >> (64 - cl));
    carry = x;
  }
  d[0] = carry << cl;
}

// d[0..n-1] = s >> cl, bottom-up so d <= s may overlap (asmShr, asmLinux.asm:141-164).
static inline void shr_n(unsigned cl, u64 n, const u64* s, u64* d) {
  u64 cur = s[0];
  for (u64 i = 0; i + 1 < n; ++i) {
    u64 nx = s[i + 1];
    d[i] = (cur >> cl) | (nx << (64 - cl));
    cur = nx;
  }
  d[n - 1] = cur >> cl;
}

// d[0..n] = s * m (asmMul0, asmLinux.asm:166-186).
static inline void mul_1(u64 n, u64 m, const u64* s, u64* d) {
  u64 c = 0;
  for (u64 i = 0; i < n; ++i) {
    u128 t = (u128)s[i] * m + c;
    d[i] = (u64)t;
    c = hi64(t);
  }
  d[n] = c;
}

// d[0..n1+n2) = s1 * s2, n1 <= n2, column-wise with a 192-bit accumulator
// (asmMul1, asmLinux.asm:188-278).
static inline void mul_school(u64 n1, u64 n2, const u64* s1, const u64* s2, u64* d) {
  u64 a0 = 0, a1 = 0, a2 = 0;
  for (u64 k = 0; k + 1 < n1 + n2; ++k) {
    u64 lo = k >= n2 ? k - n2 + 1 : 0;
    u64 hi = std::min(k, n1 - 1);
    for (u64 i = lo; i <= hi; ++i) {
      u128 p = (u128)s1[i] * s2[k - i];
      u128 s = (u128)a0 + (u64)p;
      a0 = (u64)s;
      u128 t = (u128)a1 + hi64(p) + hi64(s);
      a1 = (u64)t;
      a2 += hi64(t);
    }
    d[k] = a0;
    a0 = a1;
    a1 = a2;
    a2 = 0;
  }
  d[n1 + n2 - 1] = a0;
}

// d[0..2n) = s^2 with doubled cross products (asmSqr, asmLinux.asm:280-344).
static inline void sqr_school(u64 n, u64* d, const u64* s) {
  u64 c0 = 0, c1 = 0;  // running carry (2 words)
  for (u64 k = 0; k + 1 < 2 * n; ++k) {
    u64 a0 = 0, a1 = 0, a2 = 0;
    u64 lo = k >= n ? k - n + 1 : 0;
    u64 i = lo, j = k - lo;
    for (; i < j; ++i, --j) {
      u128 p = (u128)s[i] * s[j];
      u128 t = (u128)a0 + (u64)p;
      a0 = (u64)t;
      u128 t2 = (u128)a1 + hi64(p) + hi64(t);
      a1 = (u64)t2;
      a2 += hi64(t2);
    }
    // double
    a2 = (a2 << 1) | (a1 >> 63);
    a1 = (a1 << 1) | (a0 >> 63);
    a0 <<= 1;
    if (i == j) {
      u128 p = (u128)s[i] * s[i];
      u128 t = (u128)a0 + (u64)p;
      a0 = (u64)t;
      u128 t2 = (u128)a1 + hi64(p) + hi64(t);
      a1 = (u64)t2;
      a2 += hi64(t2);
    }
    u128 t = (u128)a0 + c0;
    a0 = (u64)t;
    u128 t2 = (u128)a1 + c1 + hi64(t);
    a1 = (u64)t2;
    a2 += hi64(t2);
    d[k] = a0;
    c0 = a1;
    c1 = a2;
  }
  d[2 * n - 1] = c0;
}

// 128/64 divide, quotient must fit 64 bits (asmDiv / asmDivMod, asmLinux.asm:720-737).
static inline u64 div_128(u64 lo, u64 hi, u64 d, u64* rem = nullptr) {
  u128 n = ((u128)hi << 64) | lo;
  u64 q = (u64)(n / d);
  if (rem) *rem = (u64)(n - (u128)q * d);
  return q;
}

// ---------------------------------------------------------------------------
// Base case (base.h:7-90)
// ---------------------------------------------------------------------------

// base.h:7-10 — _Size1 >= _Size2.
static inline int add(u64* d, const u64* a, u64 n1, const u64* b, u64 n2) {
  int cf = add_n(n2, d, a, b);
  return add_1(n1 - n2, a + n2, d + n2, cf);
}

// base.h:13-16 — a >= b.
static inline int sub(u64* d, const u64* a, u64 n1, const u64* b, u64 n2) {
  int cf = sub_n(n2, d, a, b);
  return sub_1(n1 - n2, a + n2, d + n2, cf);
}

constexpr u64 kToom22MulThreshold = 32;  // base.h:18
constexpr u64 kToom22SqrThreshold = 48;  // base.h:37

// Karatsuba on equal lengths (base.h:21-35).
static void toom22_mul(u64* d, const u64* a, const u64* b, u64 s) {
  if (s < kToom22MulThreshold) {
    mul_school(s, s, a, b, d);
    return;
  }
  u64 s0 = (s + 1) >> 1, s1 = s - s0;
  toom22_mul(d, a, b, s0);
  toom22_mul(d + 2 * s0, a + s0, b + s0, s1);
  std::vector<u64> a1(s0 + 1), b1(s0 + 1), d1(2 * (s0 + 1));
  a1[s0] = add(a1.data(), a, s0, a + s0, s1);
  b1[s0] = add(b1.data(), b, s0, b + s0, s1);
  toom22_mul(d1.data(), a1.data(), b1.data(), s0 + 1);
  sub(d1.data(), d1.data(), 2 * (s0 + 1), d, 2 * s0);
  sub(d1.data(), d1.data(), 2 * (s0 + 1), d + 2 * s0, 2 * s1);
  add(d + s0, d + s0, s + s1, d1.data(), 2 * (s0 + 1));
}

// Karatsuba square (base.h:40-53).
static void toom22_sqr(u64* d, const u64* a, u64 s) {
  if (s < kToom22SqrThreshold) {
    sqr_school(s, d, a);
    return;
  }
  u64 s0 = (s + 1) >> 1, s1 = s - s0;
  toom22_sqr(d, a, s0);
  toom22_sqr(d + 2 * s0, a + s0, s1);
  std::vector<u64> a1(s0 + 1), d1(2 * (s0 + 1));
  a1[s0] = add(a1.data(), a, s0, a + s0, s1);
  toom22_sqr(d1.data(), a1.data(), s0 + 1);
  sub(d1.data(), d1.data(), 2 * (s0 + 1), d, 2 * s0);
  sub(d1.data(), d1.data(), 2 * (s0 + 1), d + 2 * s0, 2 * s1);
  add(d + s0, d + s0, s + s1, d1.data(), 2 * (s0 + 1));
}

// Unbalanced product in chunks of n2 (base.h:56-81); n1 >= n2, d has n1+n2 limbs.
static void mul_base(u64* d, const u64* a, u64 n1, const u64* b, u64 n2) {
  if (n2 <= 1) {
    mul_1(n1, *b, a, d);
  } else if (n2 < kToom22MulThreshold) {
    mul_school(n2, n1, b, a, d);
  } else {
    toom22_mul(d, a, b, n2);
    a += n2;
    d += n2;
    n1 -= n2;
    std::memset(d + n2, 0, sizeof(u64) * n1);
    std::vector<u64> t(2 * n2);
    while (n1 >= n2) {
      toom22_mul(t.data(), a, b, n2);
      add(d, d, 2 * n2, t.data(), 2 * n2);
      a += n2;
      d += n2;
      n1 -= n2;
    }
    if (n1 > 0) {
      mul_base(t.data(), b, n2, a, n1);
      add(d, d, n1 + n2, t.data(), n1 + n2);
    }
  }
}

// base.h:84-90.
static void sqr_base(u64* d, const u64* a, u64 n) {
  if (n <= 1)
    mul_1(n, *a, a, d);
  else if (n < kToom22MulThreshold)
    sqr_school(n, d, a);
  else
    toom22_sqr(d, a, n);
}

// ---------------------------------------------------------------------------
// Limb buffer (basic_natural.h:9-97): size + grow-only capacity (bit_ceil).
// Limbs past `n` keep their contents, as the reference relies on.
// ---------------------------------------------------------------------------
struct Limbs {
  std::vector<u64> buf;
  u64 n = 0;
  Limbs() : buf(1, 0), n(1) {}
  explicit Limbs(u64 v) : buf(1, v), n(1) {}
  Limbs(const u64* p, u64 k) : buf(std::bit_ceil(std::max<u64>(k, 1))), n(k) {
    if (k) std::memcpy(buf.data(), p, k * sizeof(u64));
  }
  u64* data() { return buf.data(); }
  const u64* data() const { return buf.data(); }
  u64& operator[](u64 i) { return buf[i]; }
  const u64& operator[](u64 i) const { return buf[i]; }
  void resize(u64 s) {  // basic_natural.h:81-89
    n = s;
    if (buf.size() < s) buf.resize(std::bit_ceil(s));
  }
  void reserve(u64 s) {
    if (buf.size() < s) buf.resize(std::bit_ceil(s));
  }
};

// ---------------------------------------------------------------------------
// Three-prime NTT engine (ntt_info.h)
// ---------------------------------------------------------------------------
constexpr u64 kNttMulThreshold = 384;  // ntt_info.h:6
constexpr u64 kNttDivThreshold = 256;  // ntt_info.h:7
constexpr int kNttScaleThreshold = 10;  // ntt_info.h:8
constexpr int kNttL3Threshold = 20;     // ntt_info.h:179

// p_i = c_i * 2^56 + 1 (ntt_info.h:69-73).
constexpr u64 kMod[3] = {27ull << 56 | 1, 58ull << 56 | 1, 87ull << 56 | 1};

static inline u64 mulmod_exact(u64 a, u64 b, u64 p) { return (u64)(((u128)a * b) % p); }

static inline u64 powmod(u64 b, u64 e, u64 p) {
  u64 r = 1;
  for (; e; e >>= 1, b = mulmod_exact(b, b, p))
    if (e & 1) r = mulmod_exact(r, b, p);
  return r;
}

// Root chain per prime (ntt_info.h:81-139): root_base[i][j] has order 2^(j+1)
// and equals g_i^(2^(55-j)) for the primitive 2^56-th roots g = 11, 2, 310;
// iroot_base holds the inverses.  Derived here instead of tabulated.
struct RootChain {
  u64 fwd[3][56], inv[3][56];
  RootChain() {
    const u64 g[3] = {11, 2, 310};
    for (int i = 0; i < 3; ++i) {
      u64 pm = (i == 0 ? 27ull : i == 1 ? 58ull : 87ull) << 56 | 1;
      u64 x = g[i];
      for (int j = 55; j >= 0; --j) {
        fwd[i][j] = x;
        inv[i][j] = powmod(x, pm - 2, pm);
        x = mulmod_exact(x, x, pm);
      }
    }
  }
};
inline const RootChain& root_chain() {
  static RootChain c;
  return c;
}

// Shoup companion floor(w * 2^64 / p) + 1 (ntt_info.h:31, 37).
static inline u64 shoup_companion(u64 w, u64 p) { return div_128(0, w, p) + 1; }

// w * y mod p in [0,p) from a Shoup pair (w, wp); y < 2^64 (asmLinux.asm:414-426).
static inline u64 shoup_mul(u64 y, u64 w, u64 wp, u64 p) {
  u64 q = hi64((u128)y * wp);
  i64 r = (i64)(y * w - q * p);
  return r < 0 ? (u64)(r + (i64)p) : (u64)r;
}

// x in [0,2p) -> [0,p) (the sub/cmovs idiom of asmLinux.asm:370-372).
static inline u64 reduce2p(u64 x, u64 p) {
  u64 t = x - p;
  return (i64)t < 0 ? x : t;
}

struct Tables {
  std::vector<u64> root[3], iroot[3];
  int scale = 1;  // NTT_info::root_scale (ntt_info.h:145)
  Tables() {       // ntt_info.h:141-143
    const u64 c0[3] = {10, 5, 3};
    for (int i = 0; i < 3; ++i) {
      root[i] = {1, c0[i]};
      iroot[i] = {1, c0[i]};
    }
  }
  // ntt_info.h:22-41 — grow-only.
  void init(int s) {
    s -= 1;
    if (s <= scale) return;
    for (int i = 0; i < 3; ++i) {
      root[i].resize(1ull << s);
      iroot[i].resize(1ull << s);
      for (int j = scale; j < s; ++j)
        for (u64 k = 0, n = 1ull << j; k < n; k += 2) {
          root[i][n + k] = mulmod_exact(root[i][k], root_chain().fwd[i][j], kMod[i]);
          root[i][n + k + 1] = shoup_companion(root[i][n + k], kMod[i]);
          iroot[i][n + k] = mulmod_exact(iroot[i][k], root_chain().inv[i][j], kMod[i]);
          iroot[i][n + k + 1] = shoup_companion(iroot[i][n + k], kMod[i]);
        }
    }
    scale = s;
  }
};

inline Tables& tables() {
  static Tables t;
  return t;
}

// One forward stage of half-width j over [d, d+len): block b uses root[2b]
// (asmNtt / asmNtt2, asmLinux.asm:346-534).  Outputs are in [0, 2p).
static void ntt_stage(u64 j, u64 p, u64* d, const u64* root, u64 len) {
  for (u64 b = 0, off = 0; off < len; ++b, off += 2 * j) {
    u64 w = root[2 * b], wp = root[2 * b + 1];
    u64* x = d + off;
    u64* y = x + j;
    for (u64 i = 0; i < j; ++i) {
      u64 t = shoup_mul(y[i], w, wp, p);
      u64 xr = reduce2p(x[i], p);
      x[i] = xr + t;
      y[i] = xr + p - t;
    }
  }
}

// One inverse stage of half-width j: (x, y) -> (x + y, (x - y) * iw)
// (asmINtt / asmINtt2, asmLinux.asm:536-718).  Inputs and outputs in [0,p).
static void intt_stage(u64 j, u64 p, u64* d, const u64* iroot, u64 len) {
  for (u64 b = 0, off = 0; off < len; ++b, off += 2 * j) {
    u64 w = iroot[2 * b], wp = iroot[2 * b + 1];
    u64* x = d + off;
    u64* y = x + j;
    for (u64 i = 0; i < j; ++i) {
      u64 s = reduce2p(x[i] + y[i], p);
      u64 t = shoup_mul(x[i] - y[i] + p, w, wp, p);
      x[i] = s;
      y[i] = t;
    }
  }
}

// v * 2^-cl mod p for v in [0,p) using p = c*2^56 + 1 (asmLinux.asm:821-859).
static inline u64 div_pow2(u64 v, unsigned cl, u64 p) {
  u64 mask = (1ull << cl) - 1;
  i64 t = (i64)v - 1;
  u64 lo = (~(u64)t) & mask;
  return (u64)((t >> cl) + 1) + lo * (p >> cl);
}

// Last inverse stage (twiddle 1) fused with the scale by 2^-(s-1)
// (asmINttShr, asmLinux.asm:776-875).
static void intt_last(int s, u64 p, u64* d) {
  unsigned cl = (unsigned)(s - 1);
  u64 half = 1ull << cl;
  for (u64 i = 0; i < half; ++i) {
    u64 x = d[i], y = d[i + half];
    u64 a = reduce2p(x + y, p);
    u64 b = x >= y ? x - y : x - y + p;
    d[i] = div_pow2(a, cl, p);
    d[i + half] = div_pow2(b, cl, p);
  }
}

// Barrett reduction of the 128-bit pointwise sums (asmLinux.asm:947-960);
// the correction loop makes it exact for any input below 4p^2.
static inline u64 barrett128(u128 t, int i) {
  static const u64 mu[3] = {(u64)(((u128)1 << 124) / kMod[0]), (u64)(((u128)1 << 125) / kMod[1]),
                            (u64)(((u128)1 << 126) / kMod[2])};
  u64 p = kMod[i];
  u64 top = (u64)(t >> (60 + i));
  u64 q = hi64((u128)top * mu[i]);
  u64 r = (u64)t - q * p;
  while (r >= p) r -= p;
  return r;
}

// x mod p via q = hi(x * ceil(2^64/p)) (asmLoad / asmMod, asmLinux.asm:739-751, 891-904).
static inline u64 limb_mod(u64 x, int i) {
  static const u64 m64[3] = {10, 5, 3};  // ceil(2^64 / p_i) (ntt_info.h:148)
  u64 q = hi64((u128)x * m64[i]);
  i64 r = (i64)(x - q * kMod[i]);
  return r < 0 ? (u64)(r + (i64)kMod[i]) : (u64)r;
}

struct Xform {  // struct NTT_info (ntt_info.h:10-67)
  Limbs info[3];
  int scale = 0;
  Xform(int s = 0) : scale(s) {}

  // ntt_info.h:147-173.
  void load(const u64* src, u64 n, int s) {
    const u64 N = 1ull << (s - 1);
    scale = s;
    for (int i = 0; i < 3; ++i) info[i].resize(2 * N);
    for (int i = 0; i < 3; ++i) {
      u64 p = kMod[i];
      u64* d = info[i].data();
      if (n <= N) {
        for (u64 j = 0; j < n; ++j) d[j] = d[j + N] = limb_mod(src[j], i);
        std::memset(d + n, 0, sizeof(u64) * (N - n));
        std::memset(d + N + n, 0, sizeof(u64) * (N - n));
      } else {
        u64 j = 0;
        for (; j < n - N; ++j) {
          u64 a = limb_mod(src[j], i), b = limb_mod(src[j + N], i);
          d[j] = a + b;
          d[j + N] = a - b + p;
        }
        for (; j < N; ++j) d[j] = d[j + N] = limb_mod(src[j], i);
      }
    }
    tables().init(scale);
  }
  void load(const Limbs& x, int s) { load(x.data(), x.n, s); }

  // ntt_info.h:180-198.
  void ntt() {
    Tables& T = tables();
    for (int i = 0; i < 3; ++i) {
      u64* d = info[i].data();
      u64 len = info[i].n;
      const u64* root = T.root[i].data();
      if (scale <= kNttL3Threshold) {
        for (u64 j = 1ull << (scale - 2); j > 1; j >>= 1) ntt_stage(j, kMod[i], d, root, len);
        continue;
      }
      for (u64 j = 1ull << (scale - 2); j >= (1ull << kNttL3Threshold); j >>= 1)
        ntt_stage(j, kMod[i], d, root, len);
      const u64 chunk = 1ull << kNttL3Threshold;
      for (u64 k = 0; k < (len >> kNttL3Threshold); ++k)
        for (int j = kNttL3Threshold - 1; j > 0; --j)
          ntt_stage(1ull << j, kMod[i], d + k * chunk, root + (k << (kNttL3Threshold - j)), chunk);
    }
  }

  // ntt_info.h:200-221.
  void intt() {
    Tables& T = tables();
    for (int i = 0; i < 3; ++i) {
      u64* d = info[i].data();
      u64 len = info[i].n;
      const u64* iroot = T.iroot[i].data();
      if (scale <= kNttL3Threshold) {
        for (u64 j = 2; j < (1ull << (scale - 1)); j <<= 1) intt_stage(j, kMod[i], d, iroot, len);
      } else {
        const u64 chunk = 1ull << kNttL3Threshold;
        for (u64 k = 0; k < (len >> kNttL3Threshold); ++k)
          for (int j = 1; j < kNttL3Threshold; ++j)
            intt_stage(1ull << j, kMod[i], d + k * chunk, iroot + (k << (kNttL3Threshold - j)), chunk);
        for (u64 j = chunk; j < (1ull << (scale - 1)); j <<= 1) intt_stage(j, kMod[i], d, iroot, len);
      }
      intt_last(scale, kMod[i], d);
    }
  }

  // Pointwise product of degree-1 residues mod (x^2 - w) and (x^2 + w)
  // (ntt_info.h:224-231; asmNttMul0/1/2, asmLinux.asm:910-1367).
  void mul(const Xform& A, const Xform& B) {
    scale = A.scale;
    const u64 L = 1ull << scale;
    Tables& T = tables();
    for (int i = 0; i < 3; ++i) {
      const u64 p = kMod[i];
      info[i].resize(A.info[i].n);
      const u64* a = A.info[i].data();
      const u64* b = B.info[i].data();
      u64* d = info[i].data();
      const u64* root = T.root[i].data();
      for (u64 g = 0; g < L / 4; ++g) {
        u64 w = root[2 * g], wp = root[2 * g + 1];
        u64 a0 = reduce2p(a[4 * g], p), a1 = reduce2p(a[4 * g + 1], p);
        u64 a2 = reduce2p(a[4 * g + 2], p), a3 = reduce2p(a[4 * g + 3], p);
        u64 b0 = reduce2p(b[4 * g], p), b1 = reduce2p(b[4 * g + 1], p);
        u64 b2 = reduce2p(b[4 * g + 2], p), b3 = reduce2p(b[4 * g + 3], p);
        u64 wb1 = shoup_mul(b1, w, wp, p);
        u64 wb3 = shoup_mul(b3, w, wp, p);
        u64 nwb3 = wb3 ? p - wb3 : 0;
        u64 r1 = barrett128((u128)a0 * b1 + (u128)a1 * b0, i);
        u64 r0 = barrett128((u128)a0 * b0 + (u128)a1 * wb1, i);
        u64 r2 = barrett128((u128)a2 * b2 + (u128)a3 * nwb3, i);
        u64 r3 = barrett128((u128)a2 * b3 + (u128)a3 * b2, i);
        d[4 * g] = r0;
        d[4 * g + 1] = r1;
        d[4 * g + 2] = r2;
        d[4 * g + 3] = r3;
      }
    }
  }

  // Garner recombination + carry over `count` coefficients; low limbs go to
  // info[0], the two carry words to info[1][0..1]; returns the low carry word
  // (ntt_info.h:233-235; asmCRT, asmLinux.asm:1369-1450).
  u64 crt(u64 count) {
    const u64 p0 = kMod[0], p1 = kMod[1], p2 = kMod[2];
    static const u64 inv_p0_m1 = inv_mod(p0 % p1, p1);
    static const u64 inv_p0_m2 = inv_mod(p0 % p2, p2);
    static const u64 inv_p1_m2 = inv_mod(p1 % p2, p2);
    static const u64 s01 = shoup_companion(inv_p0_m1, p1);
    static const u64 s02 = shoup_companion(inv_p0_m2, p2);
    static const u64 s12 = shoup_companion(inv_p1_m2, p2);
    static const u128 p0p1 = (u128)p0 * p1;
    u64* r0 = info[0].data();
    const u64* r1 = info[1].data();
    const u64* r2 = info[2].data();
    u64 c0 = 0, c1 = 0;
    for (u64 k = 0; k < count; ++k) {
      u64 x0 = r0[k], x1 = r1[k], x2 = r2[k];
      // u1 = (x1 - x0) / p0 mod p1
      u64 d1 = x1 >= x0 ? x1 - x0 : x1 + p1 - x0;
      u64 u1 = shoup_mul(d1, inv_p0_m1, s01, p1);
      // v = ((x2 - x0) / p0 - u1) / p1 mod p2
      u64 d2 = x2 >= x0 ? x2 - x0 : x2 + p2 - x0;
      u64 t2 = shoup_mul(d2, inv_p0_m2, s02, p2);
      u64 e2 = t2 >= u1 ? t2 - u1 : t2 + p2 - u1;
      u64 v = shoup_mul(e2, inv_p1_m2, s12, p2);
      // x = x0 + p0*u1 + p0*p1*v  (< 2^186)
      u128 lo = (u128)p0 * u1 + x0;
      u128 m = (u128)(u64)p0p1 * v;
      u128 h = (u128)(u64)(p0p1 >> 64) * v;
      u128 w0 = (u128)(u64)lo + (u64)m;
      u128 w1 = (u128)hi64(lo) + hi64(m) + (u64)h + hi64(w0);
      u64 w2 = hi64(h) + hi64(w1);
      // add the running two-word carry
      u128 s0 = (u128)(u64)w0 + c0;
      u128 s1 = (u128)(u64)w1 + c1 + hi64(s0);
      r0[k] = (u64)s0;
      c0 = (u64)s1;
      c1 = w2 + hi64(s1);
    }
    info[1][0] = c0;
    info[1][1] = c1;
    return c0;
  }

  // ntt_info.h:237-248 — normal mode writes `size` limbs; wrap mode (size-1 > L)
  // folds the carry back in and returns the product mod B^L - 1 in L limbs.
  void save(Limbs& out, u64 size) {
    const u64 L = 1ull << scale;
    if (size - 1 > L) {
      crt(L);
      int cf = add(info[0].data(), info[0].data(), info[0].n, info[1].data(), 2);
      add_1(info[0].n, info[0].data(), info[0].data(), cf);
    } else {
      info[0].resize(size);
      info[0][size - 1] = crt(size - 1);
    }
    out = std::move(info[0]);
  }

  static u64 inv_mod(u64 a, u64 m) {  // extended Euclid
    i64 t = 0, nt = 1;
    u64 r = m, nr = a;
    while (nr) {
      u64 q = r / nr;
      i64 tmp = t - (i64)q * nt;
      t = nt;
      nt = tmp;
      u64 tr = r - q * nr;
      r = nr;
      nr = tr;
    }
    return t < 0 ? (u64)(t + (i64)m) : (u64)t;
  }
};

// ---------------------------------------------------------------------------
// natural (natural.h:16-1093)
// ---------------------------------------------------------------------------
struct Nat : Limbs {
  Nat() : Limbs() {}
  Nat(u64 v) : Limbs(v) {}
  Nat(const u64* p, u64 k) : Limbs(p, k) {}

  Nat& norm() {  // natural::std (natural.h:82-93)
    if (!n) {
      n = 1;
      buf[0] = 0;
      return *this;
    }
    while (--n)
      if (buf[n]) break;
    ++n;
    return *this;
  }
  bool is_zero() const { return n == 1 && buf[0] == 0; }
};

inline bool operator<(const Nat& a, const Nat& b) {  // natural.h:145-153
  if (a.n != b.n) return a.n < b.n;
  for (u64 i = a.n; i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i];
  return false;
}
inline bool operator==(const Nat& a, const Nat& b) {  // natural.h:167-175
  if (a.n != b.n) return false;
  for (u64 i = a.n; i-- > 0;)
    if (a[i] != b[i]) return false;
  return true;
}
inline bool operator>=(const Nat& a, const Nat& b) { return !(a < b); }
inline bool operator!=(const Nat& a, const Nat& b) { return !(a == b); }

// natural.h:244-262 (note: the whole-limb case does not normalise).
inline Nat shl(const Nat& a, u64 bits) {
  Nat d;
  if (a.is_zero()) return Nat(0);
  u64 as = a.n, n = bits >> 6;
  unsigned b = bits & 63;
  if (b == 0) {
    d.resize(as + n);
    std::memmove(d.data() + n, a.data(), as * sizeof(u64));
    std::memset(d.data(), 0, n * sizeof(u64));
    return d;
  }
  d.resize(as + n + 1);
  shl_n(b, as, a.data(), d.data() + n);
  std::memset(d.data(), 0, n * sizeof(u64));
  d.norm();
  return d;
}

// natural.h:275-290 (the whole-limb case does not normalise).
inline Nat shr(const Nat& a, u64 bits) {
  u64 as = a.n, n = bits >> 6;
  if (as <= n) return Nat(0);
  unsigned b = bits & 63;
  Nat d;
  d.resize(as - n);
  if (b == 0) {
    std::memmove(d.data(), a.data() + n, (as - n) * sizeof(u64));
    return d;
  }
  shr_n(b, as - n, a.data() + n, d.data());
  d.norm();
  return d;
}

// In-place right shift keeping the buffer (natural.h:275-290 with this == ap).
inline void shr_inplace(Nat& a, u64 bits) {
  u64 as = a.n, n = bits >> 6;
  if (as <= n) {
    a.n = 1;
    a[0] = 0;
    return;
  }
  unsigned b = bits & 63;
  a.n = as - n;
  if (b == 0) {
    std::memmove(a.data(), a.data() + n, (as - n) * sizeof(u64));
    return;
  }
  shr_n(b, as - n, a.data() + n, a.data());
  a.norm();
}

inline Nat addn(const Nat& x, const Nat& y) {  // natural.h:303-311
  const Nat* a = &x;
  const Nat* b = &y;
  if (a->n < b->n) std::swap(a, b);
  Nat d;
  d.resize(a->n + 1);
  d[a->n] = add(d.data(), a->data(), a->n, b->data(), b->n);
  d.norm();
  return d;
}

inline Nat subn(const Nat& x, const Nat& y) {  // natural.h:324-343, |x - y|
  const Nat* a = &x;
  const Nat* b = &y;
  if (a->n < b->n) std::swap(a, b);
  u64 as = a->n, bs = b->n;
  Nat d;
  if (as == bs) {
    while (--bs)
      if ((*a)[bs] != (*b)[bs]) break;
    if ((*a)[bs] < (*b)[bs]) std::swap(a, b);
    d.resize(++bs);
    sub_n(bs, d.data(), a->data(), b->data());
  } else {
    d.resize(as);
    sub(d.data(), a->data(), as, b->data(), bs);
  }
  d.norm();
  return d;
}

inline Nat mul_base_nat(const Nat& x, const Nat& y) {  // natural.h:356-369
  const Nat* a = &x;
  const Nat* b = &y;
  if (a->n < b->n) std::swap(a, b);
  Nat d;
  d.resize(a->n + b->n);
  mul_base(d.data(), a->data(), a->n, b->data(), b->n);
  d.norm();
  return d;
}

inline Nat sqr_base_nat(const Nat& a) {  // natural.h:371-382
  Nat d;
  d.resize(a.n << 1);
  sqr_base(d.data(), a.data(), a.n);
  d.norm();
  return d;
}

inline int ntt_scale(u64 n1, u64 n2) {  // natural.h:384-386
  u64 v = n1 + n2 - 2;
  return 64 - std::countl_zero(v);
}

// Raw transform product at a fixed scale (the load/NTT/mul/INTT/save pipeline
// of natural.h:399-405), wrap mode included.
inline Nat ntt_mul_raw(const u64* a, u64 na, const u64* b, u64 nb, int s, u64 size) {
  Xform xa, xb;
  xa.load(a, na, s);
  xb.load(b, nb, s);
  xa.ntt();
  xb.ntt();
  xa.mul(xa, xb);
  xa.intt();
  Limbs out;
  xa.save(out, size);
  Nat r;
  static_cast<Limbs&>(r) = std::move(out);
  return r;
}

inline Nat from_limbs(Limbs&& l) {
  Nat r;
  static_cast<Limbs&>(r) = std::move(l);
  return r;
}

// natural.h:452-467
inline void mul_save(Nat& d, const Nat& a, const Nat& b, Xform& xa) {
  if (xa.scale < kNttScaleThreshold) {
    d = mul_base_nat(a, b);
    xa.scale = 0;
    return;
  }
  xa.load(a, xa.scale);
  Xform xb;
  xb.load(b, xa.scale);
  u64 size = a.n + b.n;
  xa.ntt();
  xb.ntt();
  xb.mul(xa, xb);
  xb.intt();
  Limbs out;
  xb.save(out, size);
  d = from_limbs(std::move(out));
  d.norm();
}

// natural.h:469-486
inline void mul_save2(Nat& d, const Nat& a, const Nat& b, Xform& xa, Xform& xb) {
  if (xa.scale < kNttScaleThreshold) {
    d = mul_base_nat(a, b);
    xa.scale = 0;
    xb.scale = 0;
    return;
  }
  xa.load(a, xa.scale);
  xb.load(b, xa.scale);
  u64 size = a.n + b.n;
  xa.ntt();
  xb.ntt();
  Xform x;
  x.mul(xa, xb);
  x.intt();
  Limbs out;
  x.save(out, size);
  d = from_limbs(std::move(out));
  d.norm();
}

// natural.h:488-502
inline void sqr_save(Nat& d, const Nat& a, Xform& xa) {
  if (xa.scale < kNttScaleThreshold) {
    d = sqr_base_nat(a);
    xa.scale = 0;
    return;
  }
  xa.load(a, xa.scale);
  u64 size = a.n * 2;
  Xform x;
  xa.ntt();
  x.mul(xa, xa);
  x.intt();
  Limbs out;
  x.save(out, size);
  d = from_limbs(std::move(out));
  d.norm();
}

// natural.h:504-515
inline void mul_load(Nat& d, const Nat& a, const Nat& b, const Xform& xa) {
  if (xa.scale == 0) {
    d = mul_base_nat(a, b);
    return;
  }
  Xform xb;
  xb.load(b, xa.scale);
  u64 size = a.n + b.n;
  xb.ntt();
  xb.mul(xa, xb);
  xb.intt();
  Limbs out;
  xb.save(out, size);
  d = from_limbs(std::move(out));
  d.norm();
}

// natural.h:517-527
inline void mul_load2(Nat& d, const Nat& a, const Nat& b, const Xform& xa, const Xform& xb) {
  if (xa.scale == 0) {
    d = mul_base_nat(a, b);
    return;
  }
  u64 size = a.n + b.n;
  Xform x;
  x.mul(xa, xb);
  x.intt();
  Limbs out;
  x.save(out, size);
  d = from_limbs(std::move(out));
  d.norm();
}

// natural.h:391-419
inline Nat mul_ntt(const Nat& x, const Nat& y) {
  const Nat* a = &x;
  const Nat* b = &y;
  if (a->n < b->n) std::swap(a, b);
  u64 a0_size = (a->n + 1) >> 1;
  int s = ntt_scale(a->n, b->n);
  int s_opt = ntt_scale(a0_size, b->n);
  if (s == s_opt) {
    Nat d = ntt_mul_raw(a->data(), a->n, b->data(), b->n, s, a->n + b->n);
    d.norm();
    return d;
  }
  Nat a0(a->data(), a0_size), a1(a->data() + a0_size, a->n - a0_size);
  Xform xb(s_opt);
  mul_save(a0, *b, a0, xb);
  mul_load(a1, *b, a1, xb);
  return addn(shl(a1, a0_size << 6), a0);
}

// natural.h:433-442
inline Nat sqr_ntt(const Nat& a) {
  int s = ntt_scale(a.n, a.n);
  Xform x;
  x.load(a, s);
  x.ntt();
  x.mul(x, x);
  x.intt();
  Limbs out;
  x.save(out, a.n * 2);
  Nat d = from_limbs(std::move(out));
  d.norm();
  return d;
}

inline Nat mul(const Nat& a, const Nat& b) {  // natural.h:444-450
  if (std::min(a.n, b.n) < kNttMulThreshold) return mul_base_nat(a, b);
  return mul_ntt(a, b);
}

inline Nat sqr(const Nat& a) {  // natural.h:529-535
  if (a.n < kNttMulThreshold) return sqr_base_nat(a);
  return sqr_ntt(a);
}

inline Nat pow(const Nat& b, u64 e) {  // natural.h:554-564
  if (e == 0) return Nat(1);
  if (e == 1 || b < Nat(2)) return b;
  Nat p = pow(b, e >> 1);
  p = sqr(p);
  if (e & 1) p = mul(p, b);
  return p;
}

// natural.h:566-573
inline u64 div_base(const Nat& a, u64 b, Nat& q) {
  q.resize(a.n);
  u64 r = 0;
  for (u64 i = a.n; i-- > 0;) q[i] = div_128(a[i], r, b, &r);
  q.norm();
  return r;
}

// Newton reciprocal used by decimal output; divs's top limb is 1
// (natural.h:575-617).
inline Nat reciprocal2(const Nat& divs, u64 divd_size) {
  u64 expected_acc = divd_size + 1 - divs.n;
  // u64 arithmetic: wraps to 0 when divs[n-2] >= 2^64 - 2 (natural.h:578)
  Nat ans(((1ull << 63) | (divs[divs.n - 2] >> 1)) + 1);
  if (ans[0] == 0)
    ans[0] = 1ull << 63;
  else
    ans[0] = div_128(0, 1ull << 63, ans[0]);
  while (true) {
    u64 nxt_acc = 0, cur_acc = ans.n;
    if (cur_acc >= expected_acc + 1) {
      shr_inplace(ans, (cur_acc - expected_acc) << 6);
      return ans;
    }
    Nat tmp;
    if (divs.n > 2 * cur_acc + 1)
      tmp = shr(divs, (divs.n - 2 * cur_acc - 1) << 6);
    else
      tmp = shl(divs, (2 * cur_acc + 1 - divs.n) << 6);
    Xform xans(ntt_scale(tmp.n, 1));
    mul_save(tmp, ans, tmp, xans);
    tmp.n = tmp.n - cur_acc;
    for (u64 i = 0; i < tmp.n; ++i) tmp[i] = ~tmp[i + cur_acc];
    tmp.norm();
    int l_zero = std::countl_zero(tmp[tmp.n - 1]);
    nxt_acc = std::min<u64>(2 * cur_acc, (2 * cur_acc - tmp.n) * 2 + ((u64)(l_zero + 31) >> 5));
    if (nxt_acc == kNttDivThreshold) nxt_acc = kNttDivThreshold - 1;
    shr_inplace(tmp, (2 * cur_acc - nxt_acc) << 6);
    if (tmp.is_zero()) tmp = Nat(1);
    if (nxt_acc < cur_acc) throw PreconditionBroken();  // natural.h:614 would shift by a negative count
    mul_load(tmp, ans, tmp, xans);
    ans = shl(ans, (nxt_acc - cur_acc) << 6);
    if (tmp.n < cur_acc || tmp.n - cur_acc > ans.n) throw PreconditionBroken();  // natural.h:615 add() needs it
    add(ans.data(), ans.data(), ans.n, tmp.data() + cur_acc, tmp.n - cur_acc);
  }
}

// Newton reciprocal used by division; divisor's top limb is 1 and its
// transform is left in xdiv (natural.h:619-687).
inline Nat reciprocal3(const Nat& divisor, u64 dividend_size, Xform& xdiv) {
  u64 expected_acc = dividend_size + 1 - divisor.n;
  // u64 arithmetic: wraps to 0 when divisor[n-2] >= 2^64 - 2 (natural.h:622)
  Nat ans(((1ull << 63) | (divisor[divisor.n - 2] >> 1)) + 1);
  ans[0] = ans[0] ? div_128(0, 1ull << 63, ans[0]) : 1ull << 63;
  for (u64 i = 1; i < divisor.n; i *= 2) {
    u64 prev_acc = ans.n, seg = 2 * prev_acc + 1;
    if (2 * i >= divisor.n) seg = divisor.n;
    const u64* dseg = divisor.data() + divisor.n - seg;
    Nat tmp;
    Xform xans;
    if (2 * i <= kNttDivThreshold) {
      tmp.resize(seg + prev_acc);
      mul_base(tmp.data(), dseg, seg, ans.data(), prev_acc);
      tmp.norm();
    } else {
      int s = ntt_scale(i, i);
      xans.load(ans, s);
      xdiv.load(dseg, seg, s);
      xans.ntt();
      xdiv.ntt();
      Xform xt;
      xt.mul(xans, xdiv);
      xt.intt();
      Limbs out;
      xt.save(out, seg + prev_acc);
      tmp = from_limbs(std::move(out));
      tmp.norm();
    }
    u64 n_shl = seg - 1 - prev_acc;
    while (tmp.n > n_shl + 1 && ~tmp[tmp.n - 1] == 0) tmp.n -= 1;
    int l_zero = std::countl_zero(~tmp[tmp.n - 1]);
    u64 cur_acc = std::min<u64>(2 * prev_acc, (2 * prev_acc - tmp.n + n_shl) * 2 + ((u64)(l_zero + 31) >> 5));
    if (cur_acc == kNttDivThreshold) cur_acc -= 1;
    n_shl += 2 * prev_acc - cur_acc;
    if (tmp.n <= n_shl)
      tmp = Nat(1);
    else {
      tmp.n = tmp.n - n_shl;
      for (u64 k = 0; k < tmp.n; ++k) tmp[k] = ~tmp[k + n_shl];
      tmp.norm();
    }
    mul_load(tmp, ans, tmp, xans);
    shr_inplace(tmp, prev_acc << 6);
    if (cur_acc < prev_acc) throw PreconditionBroken();  // natural.h:670-672 would memset a negative length
    u64 inc_acc = cur_acc - prev_acc;
    if (inc_acc < tmp.n && tmp.n - inc_acc > prev_acc) throw PreconditionBroken();  // natural.h:676 add() needs it
    tmp.reserve(cur_acc);
    if (inc_acc >= tmp.n) {
      std::memset(tmp.data() + tmp.n, 0, sizeof(u64) * (inc_acc - tmp.n));
      std::memcpy(tmp.data() + inc_acc, ans.data(), sizeof(u64) * prev_acc);
    } else {
      add(tmp.data() + inc_acc, ans.data(), prev_acc, tmp.data() + inc_acc, tmp.n - inc_acc);
    }
    tmp.resize(cur_acc);
    ans = std::move(tmp);
    if (cur_acc >= expected_acc + 1) {
      shr_inplace(ans, (cur_acc - expected_acc) << 6);
      return ans;
    }
  }
  shr_inplace(ans, 64);
  return ans;
}

// Block division with a wrapped b*q product and fix-up (natural.h:689-747).
inline void div_iterative(const Nat& divd, const Nat& divs, Nat& q, Nat& r) {
  unsigned n_shl = (unsigned)(std::countl_zero(divs[divs.n - 1]) + 1) & 63;
  Nat b = shl(divs, n_shl);
  r = shl(divd, n_shl);
  Xform xb;
  Nat rec = reciprocal3(b, r.n, xb);
  Xform xrec(ntt_scale(rec.n, rec.n));
  int s_b = ntt_scale(b.n, 1);
  u64 L_b = 1ull << s_b;
  if (xb.scale != s_b && s_b >= kNttScaleThreshold - 1) {
    xb.load(b, s_b);
    xb.ntt();
  }
  q.resize(r.n - b.n + 1);
  std::memset(q.data(), 0, sizeof(u64) * q.n);
  Nat tmp;
  bool first = true;
  while (true) {
    u64 idx = 0;
    if (r.n > rec.n + b.n - 1) idx = r.n - rec.n - b.n + 1;
    Nat rs = shr(r, (idx + b.n - 1) << 6);
    if (first)
      mul_save(tmp, rec, rs, xrec);
    else
      mul_load(tmp, rec, rs, xrec);
    first = false;
    shr_inplace(tmp, rec.n << 6);
    add(q.data() + idx, q.data() + idx, q.n - idx, tmp.data(), tmp.n);
    mul_load(tmp, b, tmp, xb);
    if (r.n < idx || r.n - idx < tmp.n) throw PreconditionBroken();  // natural.h:724 sub() needs it
    sub(r.data() + idx, r.data() + idx, r.n - idx, tmp.data(), tmp.n);
    r.norm();
    if (xb.scale) {
      if (r.n - idx > L_b) {
        int cf = add(r.data() + idx, r.data() + idx, L_b, r.data() + idx + L_b, r.n - idx - L_b);
        add_1(L_b, r.data() + idx, r.data() + idx, cf);
        r.resize(idx + L_b);
      }
      if (r.n == idx + L_b && r[r.n - 1] >> 63) r.resize(idx);
      r.norm();
    }
    if (idx == 0) break;
  }
  for (int guard = 0; r >= b; ++guard) {
    if (guard > 64) throw PreconditionBroken();  // the block estimates were meant to be within a few units
    q = addn(q, Nat(1));
    r = subn(r, b);
  }
  shr_inplace(r, n_shl);
}

// Knuth's algorithm D (TAOCP vol. 2, 4.3.1): exact long division, used where
// the reference's Newton division breaks its own preconditions (on such
// inputs the reference itself reads or copies out of bounds and aborts).
inline void div_knuth(const Nat& a, const Nat& b, Nat& q, Nat& r) {
  const u64 n = b.n, m = a.n - b.n;
  const unsigned sh = (unsigned)std::countl_zero(b[n - 1]);
  std::vector<u64> v(n), u(a.n + 1);
  for (u64 i = n; i-- > 0;) v[i] = (b[i] << sh) | (sh && i ? b[i - 1] >> (64 - sh) : 0);
  u[a.n] = sh ? a[a.n - 1] >> (64 - sh) : 0;
  for (u64 i = a.n; i-- > 0;) u[i] = (a[i] << sh) | (sh && i ? a[i - 1] >> (64 - sh) : 0);
  q.resize(m + 1);
  for (u64 j = m + 1; j-- > 0;) {
    u128 num = ((u128)u[j + n] << 64) | u[j + n - 1];
    u128 qh = num / v[n - 1], rh = num % v[n - 1];
    while (qh >> 64 || (n > 1 && qh * v[n - 2] > ((rh << 64) | u[j + n - 2]))) {
      --qh;
      rh += v[n - 1];
      if (rh >> 64) break;
    }
    u64 borrow = 0, carry = 0;
    for (u64 i = 0; i < n; ++i) {
      u128 p = (u128)(u64)qh * v[i] + carry;
      carry = hi64(p);
      u64 t = u[i + j] - (u64)p;
      u64 b1 = u[i + j] < (u64)p;
      u64 t2 = t - borrow;
      u64 b2 = t < borrow;
      u[i + j] = t2;
      borrow = b1 | b2;
    }
    u64 t = u[j + n] - carry;
    u64 b1 = u[j + n] < carry;
    u64 t2 = t - borrow;
    u64 b2 = t < borrow;
    u[j + n] = t2;
    if (b1 | b2) {  // added back: the estimate was one too large
      --qh;
      u64 c = 0;
      for (u64 i = 0; i < n; ++i) {
        u128 s2 = (u128)u[i + j] + v[i] + c;
        u[i + j] = (u64)s2;
        c = hi64(s2);
      }
      u[j + n] += c;
    }
    q[j] = (u64)qh;
  }
  q.norm();
  r.resize(n);
  for (u64 i = 0; i < n; ++i) r[i] = (u[i] >> sh) | (sh && i + 1 < n + 1 ? (u[i + 1] << (64 - sh)) : 0);
  r.norm();
}

// natural.h:749-769 — returns the quotient, writes the remainder.
inline Nat divmod(const Nat& a, const Nat& b, Nat& r) {
  Nat q;
  if (b.is_zero()) {
    q = Nat(a.is_zero() ? 1 : 0);
    r = Nat(0);
    return q;
  }
  if (a < b) {
    r = a;
    return Nat(0);
  }
  if (b.n == 1) {
    r = Nat(div_base(a, b[0], q));
    return q;
  }
  try {
    div_iterative(a, b, q, r);
  } catch (const PreconditionBroken&) {
    ++fallback_count();
    div_knuth(a, b, q, r);
  }
  return q;
}

// Binary-splitting series for e (natural.h:841-857).
inline void calc_e(Nat& num, Nat& den, u64 begin, u64 end) {
  if (end - begin == 2) {
    num = Nat(end);
    den = Nat(begin + 1);
    if (begin) den = mul(den, Nat(begin));
    return;
  }
  Nat num1, den1;
  calc_e(num, den, begin, (begin + end) >> 1);
  calc_e(num1, den1, (begin + end) >> 1, end);
  Xform x(ntt_scale(std::max(den.n, num.n), den1.n));
  mul_save(num, den1, num, x);
  mul_load(den, den1, den, x);
  num = addn(num, num1);
}

// Newton iteration for sqrt(10005) as a fraction (natural.h:859-872).
inline void sqrt_10005(Nat& num, Nat& den, u64 acc) {
  num = Nat(4001);
  den = Nat(40);
  Nat c1, c2;
  while (num.n + den.n - 2 < acc) {
    Xform xn, xd;
    xn.scale = xd.scale = ntt_scale(num.n, num.n);
    sqr_save(c1, den, xd);
    sqr_save(c2, num, xn);
    mul_load2(den, num, den, xn, xd);
    den = shl(den, 1);
    num = addn(mul(c1, Nat(10005)), c2);
  }
}

// Chudnovsky binary splitting (natural.h:874-902).
inline void calc_pi(Nat& num, Nat& den, Nat& numc, u64 begin, u64 end) {
  if (end - begin == 1) {
    den = Nat(begin);
    den = mul(mul(mul(den, den), den), Nat(0x26dd041d878000ull));
    numc = Nat(2 * begin - 1);
    numc = mul(numc, Nat(6 * begin - 1));
    numc = mul(numc, Nat(6 * begin - 5));
    num = Nat(begin);
    num = mul(addn(mul(Nat(0x207e2da6ull), num), Nat(0xcf6371)), numc);
    return;
  }
  Nat num1, den1, numc1;
  calc_pi(num, den, numc, begin, (begin + end) >> 1);
  calc_pi(num1, den1, numc1, (begin + end) >> 1, end);
  if (end - begin == 2) {
    num = subn(mul(numc, num1), mul(num, den1));
    den = mul(den, den1);
    numc = mul(numc, numc1);
    return;
  }
  Xform xd1, xnc;
  xd1.scale = ntt_scale(std::max(den.n, num.n), den1.n);
  mul_save(num, den1, num, xd1);
  mul_load(den, den1, den, xd1);
  xnc.scale = ntt_scale(std::max(numc1.n, num1.n), numc.n);
  mul_save(num1, numc, num1, xnc);
  mul_load(numc, numc, numc1, xnc);
  num = addn(num, num1);
}

// ---------------------------------------------------------------------------
// Decimal output (natural.h:904-1011)
// ---------------------------------------------------------------------------
constexpr u64 kDecLength = 18;
constexpr u64 kDecBase0 = 1000000000000000000ull;

struct DecCache {  // natural.h:904-906 (globals there)
  Nat base[64], base_r[64];
  Xform xbase[64], xbase_r[64];
  DecCache() { base[0] = Nat(kDecBase0); for (int i = 1; i < 64; ++i) base[i] = Nat(0); }
};
inline DecCache& dec_cache() {
  static DecCache c;
  return c;
}

// natural.h:909-923
inline void calc_dec_base(int i) {
  DecCache& C = dec_cache();
  if (!C.base[i + 1].is_zero()) return;
  C.xbase[i].scale = ntt_scale(C.base[i].n, C.base[i].n);
  sqr_save(C.base[i + 1], C.base[i], C.xbase[i]);
  unsigned n_shl = (unsigned)(std::countl_zero(C.base[i][C.base[i].n - 1]) + 1) & 63;
  C.base_r[i] = reciprocal2(shl(C.base[i], n_shl), C.base[i].n * 2 + 1);
  C.xbase_r[i].scale = ntt_scale(C.base_r[i].n, C.base[i].n + 2);
  if (C.xbase_r[i].scale < kNttScaleThreshold)
    C.xbase_r[i].scale = 0;
  else {
    C.xbase_r[i].load(C.base_r[i], C.xbase_r[i].scale);
    C.xbase_r[i].ntt();
  }
}

// natural.h:953-967
inline void dec_split(const Nat& x, int i, Nat& hi, Nat& lo) {
  DecCache& C = dec_cache();
  if (i == 0) {
    lo = Nat(div_base(x, kDecBase0, hi));
    return;
  }
  unsigned n_shl = (unsigned)(std::countl_zero(C.base[i][C.base[i].n - 1]) + 1) & 63;
  mul_load(hi, C.base_r[i], shr(x, (C.base[i].n - 1) << 6), C.xbase_r[i]);
  shr_inplace(hi, ((C.base[i].n + 2) << 6) - n_shl);
  mul_load(lo, C.base[i], hi, C.xbase[i]);
  lo = subn(x, lo);
  while (lo >= C.base[i]) {
    hi = addn(hi, Nat(1));
    lo = subn(lo, C.base[i]);
  }
}

inline void format_dec(const Nat& x, int i, bool first, std::string& out) {  // natural.h:994-1011
  if (i == -1) {
    char tmp[32];
    std::string s = std::to_string(x[0]);
    if (!first) {
      std::snprintf(tmp, sizeof tmp, "%018llu", (unsigned long long)x[0]);
      s = tmp;
    }
    out += s;
    return;
  }
  Nat hi, lo;
  dec_split(x, i, hi, lo);
  if (first && hi.is_zero()) {
    format_dec(lo, i - 1, true, out);
    return;
  }
  format_dec(hi, i - 1, first, out);
  format_dec(lo, i - 1, false, out);
}

inline int dec_init(const Nat& x) {  // natural.h:1013-1018
  DecCache& C = dec_cache();
  int i = 0;
  for (; x >= C.base[i]; ++i) calc_dec_base(i);
  return i - 1;
}

inline std::string to_dec(const Nat& x) {  // std::formatter<natural> 'd' (natural.h:1089-1091)
  std::string out;
  format_dec(x, dec_init(x), true, out);
  return out;
}

}  // namespace nno

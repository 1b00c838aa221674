// divide.cpp — quotient and remainder with every operand resident on the GPU.
//
// The reference divides (natural::_div, div_iterative and the Newton
// reciprocal, natural.h:620-769) on the host around its products; the
// drop-in header keeps that algorithm step for step.  Quotient and remainder
// are unique, so for long operands the C entry points here use a different
// division whose every step stays in HBM, and the results are the
// reference's:
//   1. normalise: D = b << cl (top bit set), A = a << cl (na + 1 limbs);
//   2. V ~ floor(B^(2t) / D_t) by Newton's method with precision doubling,
//      t = k + 1 for a quotient of k limbs, D_t the top t limbs of D (or D
//      padded with zero limbs below): X_t = X_h B^(t-h) + floor(X_h E / B^(2h))
//      with E = B^(t+h) - D_t X_h (signed, |E| < 2 B^t) and h = ceil(t/2) + 1
//      (one guard limb, so the Newton error squared is divided by B and V is
//      within one unit of the floor, never above it); t <= 32 is Knuth's
//      algorithm D on the host;
//   3. floor(A_top V / B^(2t)) is within one of q, so q' = that - 2 lies in
//      [q - 3, q - 1];
//   4. r = A - q' D, then at most a few steps r -= D, q' += 1 while r >= D;
//   5. r >>= cl.
// Every product is the engine's (natural::_mul dispatch); sums, differences
// and comparisons are carry scans (lin_combine); a comparison's outcome is one
// limb read back.
#include <cuda_runtime.h>

#include <algorithm>
#include <bit>
#include <cstring>
#include <vector>

#include "context_access.h"

namespace {

using nn::u64;
using u128 = unsigned __int128;

constexpr u64 kRecipBase = 32;  // limbs: reciprocals this short are computed on the host
constexpr int kMaxFixups = 8;   // correction steps allowed before giving up (at most 3 are needed)

// Device buffer counted against the context's budget.
struct Buf {
  nn_context* c;
  u64* p = nullptr;
  u64 n = 0;
  explicit Buf(nn_context* ctx) : c(ctx) {}
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  nn_status alloc(u64 words) {
    n = words;
    return nn::ctx_alloc(c, &p, words);
  }
  ~Buf() {
    if (p) nn::ctx_free(c, p, n);
  }
};

#define DV_CK(c, expr, what)                                   \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) return nn::ctx_fail((c), _e, what); \
  } while (0)
#define DV_ST(expr)                  \
  do {                               \
    nn_status _s = (expr);           \
    if (_s != NN_OK) return _s;      \
  } while (0)

// Page-locked staging for the division's small host<->device transfers (limbs
// read back for comparisons, constants, the base-case reciprocal): per host
// thread, grown on demand, never released.
u64* staging(u64 words) {
  static thread_local u64* buf = nullptr;
  static thread_local u64 cap = 0;
  if (cap < words) {
    if (buf) nn_host_free(buf, cap * 8);
    cap = std::max<u64>(words, 256);
    buf = static_cast<u64*>(nn_host_alloc(cap * 8));
    if (!buf) cap = 0;
  }
  return buf;
}

// A host buffer as the GPU copies see it: the buffer itself when it is
// page-locked, else a page-locked block from the library's pool, filled from
// (load) or emptied into (store) the caller's buffer on all host cores.
struct HostStage {
  u64* user;
  u64 n;
  u64* p;
  bool own = false;
  HostStage(const u64* buf, u64 words) : user(const_cast<u64*>(buf)), n(words), p(const_cast<u64*>(buf)) {
    cudaPointerAttributes at{};
    const bool locked = cudaPointerGetAttributes(&at, buf) == cudaSuccess && at.type == cudaMemoryTypeHost;
    cudaGetLastError();
    if (!locked) {
      p = static_cast<u64*>(nn_host_alloc(words * 8));
      own = true;
    }
  }
  HostStage(const HostStage&) = delete;
  HostStage& operator=(const HostStage&) = delete;
  bool ok() const { return p != nullptr; }
  void load() {
    if (own) nn_host_copy(p, user, n);
  }
  void store() {
    if (own) nn_host_copy(user, p, n);
  }
  ~HostStage() {
    if (own && p) nn_host_free(p, n * 8);
  }
};

nn_status read_limb(nn_context* c, const u64* p, u64* v) {
  cudaStream_t st = nn::ctx_stream(c);
  u64* h = staging(1);
  if (!h) return NN_ERR_OOM;
  DV_CK(c, cudaMemcpyAsync(h, p, 8, cudaMemcpyDeviceToHost, st), "read limb");
  DV_CK(c, cudaStreamSynchronize(st), "read limb");
  *v = h[0];
  return NN_OK;
}

// Copies n host limbs to the device through the staging buffer and waits.
nn_status put_limbs(nn_context* c, u64* d, const u64* h, u64 n) {
  cudaStream_t st = nn::ctx_stream(c);
  u64* s = staging(n);
  if (!s) return NN_ERR_OOM;
  std::memcpy(s, h, n * 8);
  DV_CK(c, cudaMemcpyAsync(d, s, n * 8, cudaMemcpyHostToDevice, st), "constants");
  DV_CK(c, cudaStreamSynchronize(st), "constants");
  return NN_OK;
}

// floor(B^(2t) / d) for normalised d (top bit set) of t limbs, by Knuth's
// algorithm D on the dividend B^(2t): q has t + 1 limbs.
void recip_base(const u64* d, u64 t, u64* q) {
  const u64 n = t, m = t + 1;
  std::vector<u64> u(2 * t + 2, 0);
  u[2 * t] = 1;
  for (u64 j = m; j-- > 0;) {
    const u128 num = ((u128)u[j + n] << 64) | u[j + n - 1];
    u128 qhat = num / d[n - 1];
    u128 rhat = num % d[n - 1];
    while ((qhat >> 64) || (n >= 2 && qhat * d[n - 2] > ((rhat << 64) | u[j + n - 2]))) {
      --qhat;
      rhat += d[n - 1];
      if (rhat >> 64) break;
    }
    u64 borrow = 0, carry = 0;
    for (u64 i = 0; i < n; ++i) {  // u[j..j+n] -= qhat * d
      const u128 p = qhat * d[i] + carry;
      carry = (u64)(p >> 64);
      const u64 lo = (u64)p, x = u[i + j];
      const u64 s1 = x - lo, b1 = x < lo;
      const u64 s2 = s1 - borrow, b2 = s1 < borrow;
      u[i + j] = s2;
      borrow = b1 + b2;
    }
    const u64 x = u[j + n];
    const u64 s1 = x - carry, b1 = x < carry;
    const u64 s2 = s1 - borrow, b2 = s1 < borrow;
    u[j + n] = s2;
    if (b1 + b2) {  // qhat was one too large: add d back
      --qhat;
      u64 c2 = 0;
      for (u64 i = 0; i < n; ++i) {
        const u128 s = (u128)u[i + j] + d[i] + c2;
        u[i + j] = (u64)s;
        c2 = (u64)(s >> 64);
      }
      u[j + n] += c2;
    }
    q[j] = (u64)qhat;
  }
}

// x[0..t+1) ~ floor(B^(2t) / d) for normalised d of t limbs on the device,
// within one unit below; x holds t + 2 limbs.
nn_status recip(nn_context* c, const u64* d, u64 t, u64* x) {
  cudaStream_t st = nn::ctx_stream(c);
  nn::Scan& sc = nn::ctx_scan(c);
  if (t <= kRecipBase) {
    std::vector<u64> hd(t), hx(t + 2, 0);
    u64* s = staging(t);
    if (!s) return NN_ERR_OOM;
    DV_CK(c, cudaMemcpyAsync(s, d, t * 8, cudaMemcpyDeviceToHost, st), "reciprocal base");
    DV_CK(c, cudaStreamSynchronize(st), "reciprocal base");
    std::memcpy(hd.data(), s, t * 8);
    recip_base(hd.data(), t, hx.data());
    return put_limbs(c, x, hx.data(), t + 2);
  }
  const u64 h = (t + 1) / 2 + 1;
  Buf xh(c), p(c), e(c), y(c);
  DV_ST(xh.alloc(h + 2));
  DV_ST(recip(c, d + (t - h), h, xh.p));  // the top h limbs of d
  DV_ST(p.alloc(t + h + 1));
  DV_ST(nn::ctx_mul(c, p.p, d, t, xh.p, h + 1));  // P = d X_h < 2 B^(t+h)
  // The sign of E = B^(t+h) - P is P's top limb (0: E > 0; 1: E <= 0), read
  // by the scans on the device, so the levels queue without a host round trip.
  const u64* top = p.p + t + h;
  // |E|: 0 - P modulo B^(t+h) when top = 0, else 0 + P; < 2 B^t, so its low
  // t + 1 limbs hold it
  DV_ST(e.alloc(t + h + 1));
  DV_CK(c, nn::lin_combine(e.p, t + h, nullptr, 0, 0, p.p, t + h, 0, true, 1, sc, st, top), "reciprocal residual");
  // Y = X_h |E|, used from limb 2h
  DV_ST(y.alloc(h + t + 2));
  DV_ST(nn::ctx_mul(c, y.p, xh.p, h + 1, e.p, t + 1));
  const u64* yt = y.p + 2 * h;
  const u64 nyt = t + 2 - h;
  // X = X_h B^(t-h) + floor(Y / B^(2h))   (top = 0)
  //   = X_h B^(t-h) - floor(Y / B^(2h)) - 1   (top = 1: the subtraction with cin = 0)
  DV_CK(c, nn::lin_combine(x, t + 1, xh.p, h + 1, t - h, yt, nyt, 0, false, 0, sc, st, top), "reciprocal step");
  return NN_OK;
}

// q[0..na-nb+1) and r[0..nb) (unnormalised) of a / b; na >= nb >= 1 and
// b[nb-1] != 0.  None of the pointers alias.
nn_status div_impl(nn_context* c, u64* q, u64* r, const u64* a, u64 na, const u64* b, u64 nb) {
  cudaStream_t st = nn::ctx_stream(c);
  nn::Scan& sc = nn::ctx_scan(c);
  u64 top = 0;
  DV_ST(read_limb(c, b + nb - 1, &top));
  if (top == 0) {
    nn::ctx_error(c, "division: the divisor's top limb is zero");
    return NN_ERR_INVALID;
  }
  const unsigned cl = (unsigned)std::countl_zero(top);
  const u64 ma = na + 1, k = ma - nb + 1, t = k + 1;
  Buf dn(c), an(c), dt(c), at(c), v(c), pq(c), q1(c), small(c), qd(c), rr(c), tt(c), qs(c);
  DV_ST(dn.alloc(nb + 1));
  DV_ST(an.alloc(na + 1));
  DV_CK(c, nn::shl_bits(dn.p, b, nb, cl, st), "normalise");
  DV_CK(c, nn::shl_bits(an.p, a, na, cl, st), "normalise");
  // D_t and A_top: the top t limbs (t <= nb), or padded below with t - nb zero limbs
  const u64* d_t = dn.p + (t <= nb ? nb - t : 0);
  const u64* a_t = an.p + (t <= nb ? nb - t : 0);
  const u64 lat = t <= nb ? ma - (nb - t) : ma + (t - nb);
  if (t > nb) {
    DV_ST(dt.alloc(t));
    DV_ST(at.alloc(lat));
    DV_CK(c, cudaMemsetAsync(dt.p, 0, (t - nb) * 8, st), "pad");
    DV_CK(c, cudaMemcpyAsync(dt.p + (t - nb), dn.p, nb * 8, cudaMemcpyDeviceToDevice, st), "pad");
    DV_CK(c, cudaMemsetAsync(at.p, 0, (t - nb) * 8, st), "pad");
    DV_CK(c, cudaMemcpyAsync(at.p + (t - nb), an.p, ma * 8, cudaMemcpyDeviceToDevice, st), "pad");
    d_t = dt.p;
    a_t = at.p;
  }
  DV_ST(v.alloc(t + 2));
  DV_ST(recip(c, d_t, t, v.p));
  // q' = floor(A_top V / B^(2t)): k limbs from limb 2t of the product
  DV_ST(pq.alloc(lat + t + 1));
  DV_ST(nn::ctx_mul(c, pq.p, a_t, lat, v.p, t + 1));
  const u64* qe = pq.p + 2 * t;
  // q1 = q' - 2 (0 when q' < 2): never above q
  DV_ST(small.alloc(2));
  const u64 consts[2] = {2, 0};
  DV_ST(put_limbs(c, small.p, consts, 2));
  DV_ST(q1.alloc(k + 1));
  DV_CK(c, nn::lin_combine(q1.p, k, qe, k, 0, small.p, 1, 0, true, 1, sc, st), "quotient estimate");
  u64 ge2 = 0;
  DV_ST(read_limb(c, q1.p + k, &ge2));
  if (!ge2) DV_CK(c, cudaMemsetAsync(q1.p, 0, k * 8, st), "quotient estimate");
  // r = A - q1 D  (>= 0, below 4 D: nb + 1 limbs)
  DV_ST(qd.alloc(k + nb));
  DV_ST(nn::ctx_mul(c, qd.p, q1.p, k, dn.p, nb));
  DV_ST(rr.alloc(ma + 1));
  DV_CK(c, nn::lin_combine(rr.p, ma, an.p, ma, 0, qd.p, ma, 0, true, 1, sc, st), "remainder");
  u64 no_borrow = 0;
  DV_ST(read_limb(c, rr.p + ma, &no_borrow));
  if (!no_borrow) {
    nn::ctx_error(c, "division: quotient estimate above the quotient");
    return NN_ERR_CUDA;
  }
  // while r >= D: r -= D, count += 1
  DV_ST(tt.alloc(nb + 2));
  u64* cur = rr.p;
  u64* nxt = tt.p;
  u64 count = 0;
  for (;; ++count) {
    if (count > (u64)kMaxFixups) {
      nn::ctx_error(c, "division: too many correction steps");
      return NN_ERR_CUDA;
    }
    DV_CK(c, nn::lin_combine(nxt, nb + 1, cur, nb + 1, 0, dn.p, nb, 0, true, 1, sc, st), "remainder correction");
    u64 ge = 0;
    DV_ST(read_limb(c, nxt + nb + 1, &ge));
    if (!ge) break;
    std::swap(cur, nxt);
  }
  // q = q1 + count: the quotient fits na - nb + 1 limbs
  const u64 cnt[2] = {count, 0};
  DV_ST(put_limbs(c, small.p, cnt, 2));
  DV_ST(qs.alloc(k + 1));
  DV_CK(c, nn::lin_combine(qs.p, k, q1.p, k, 0, small.p, 1, 0, false, 0, sc, st), "quotient");
  DV_CK(c, cudaMemcpyAsync(q, qs.p, (na - nb + 1) * 8, cudaMemcpyDeviceToDevice, st), "quotient");
  // r = (A - q D) >> cl  (below D: nb limbs)
  DV_CK(c, nn::shr_bits(r, cur, nb, cl, st), "remainder");
  return NN_OK;
}

}  // namespace

namespace nn {
nn_status device_divide(nn_context* c, u64* q, u64* r, const u64* a, u64 na, const u64* b, u64 nb) {
  return div_impl(c, q, r, a, na, b, nb);
}
}  // namespace nn

extern "C" {

nn_status nn_divmod_host(nn_context* c, uint64_t* q, uint64_t* r, const uint64_t* a, uint64_t n_a, const uint64_t* b,
                         uint64_t n_b) {
  if (!c || !q || !r || !a || !b || n_b == 0 || n_a < n_b || b[n_b - 1] == 0) return NN_ERR_INVALID;
  cudaStream_t st = nn::ctx_stream(c);
  u64 *da = nullptr, *db = nullptr;
  DV_ST(nn::ctx_scratch(c, 0, n_a, &da));
  DV_ST(nn::ctx_scratch(c, 1, n_b, &db));
  Buf dq(c), dr(c);
  DV_ST(dq.alloc(n_a - n_b + 1));
  DV_ST(dr.alloc(n_b));
  // Pageable host buffers move through page-locked staging blocks, page-locked
  // ones directly: after large pageable transfers elsewhere in the process the
  // driver's own staging of pageable copies was measured several times slower.
  HostStage sa(a, n_a), sb(b, n_b), sq(q, n_a - n_b + 1), sr(r, n_b);
  if (!sa.ok() || !sb.ok() || !sq.ok() || !sr.ok()) return NN_ERR_OOM;
  sa.load();
  sb.load();
  DV_CK(c, cudaMemcpyAsync(da, sa.p, n_a * 8, cudaMemcpyHostToDevice, st), "H2D");
  DV_CK(c, cudaMemcpyAsync(db, sb.p, n_b * 8, cudaMemcpyHostToDevice, st), "H2D");
  DV_ST(div_impl(c, dq.p, dr.p, da, n_a, db, n_b));
  DV_CK(c, cudaMemcpyAsync(sq.p, dq.p, (n_a - n_b + 1) * 8, cudaMemcpyDeviceToHost, st), "D2H");
  DV_CK(c, cudaMemcpyAsync(sr.p, dr.p, n_b * 8, cudaMemcpyDeviceToHost, st), "D2H");
  const nn_status status = nn_context_synchronize(c);
  if (status == NN_OK) {
    sq.store();
    sr.store();
  }
  return status;
}

nn_status nn_div(nn_context* c, uint64_t* d_q, uint64_t* d_r, const uint64_t* d_a, uint64_t n_a,
                 const uint64_t* d_b, uint64_t n_b) {
  if (!c || !d_q || !d_r || !d_a || !d_b || n_b == 0 || n_a < n_b) return NN_ERR_INVALID;
  return div_impl(c, d_q, d_r, d_a, n_a, d_b, n_b);
}

}  // extern "C"

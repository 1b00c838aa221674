// nn_device.cuh — modular arithmetic for the three NTT primes on sm_103a.
//
// The primes are p_i = c_i * 2^56 + 1 with c = 27, 58, 87 (ntt_info.h:69-73).
// All arithmetic is exact 64-bit integer work on the IMAD pipe; nothing here
// uses floating point or tensor cores.
#pragma once

#include <cstdint>

namespace nn {

typedef std::uint64_t u64;
typedef std::int64_t i64;
typedef unsigned int u32;

struct PrimeSet {
  u64 p[3];      // moduli
  u64 m64[3];    // ceil(2^64 / p) — limb reduction (ntt_info.h:148)
  u64 mu[3];     // floor(2^(124+i) / p_i) — Barrett for the pointwise sums (asmLinux.asm:926,1075,1236)
  u32 c_hi[3];   // c_i << 24: the high 32 bits of q*p are q_hi + q_lo*(c_i<<24)
  // Garner constants: x = r0 + p0*u + p0*p1*v
  u64 inv01, inv01s;  // p0^-1 mod p1 and its Shoup companion
  u64 inv02, inv02s;  // p0^-1 mod p2
  u64 inv12, inv12s;  // p1^-1 mod p2
  u64 p01_lo, p01_hi; // p0*p1 as two words
};

// One copy per translation unit (no relocatable device code); every unit
// that launches kernels exports an uploader and upload_primes() calls them all.
static __constant__ PrimeSet g_primes;
#define NN_DEFINE_PRIME_UPLOADER(name) \
  cudaError_t name(const PrimeSet& ps) { return cudaMemcpyToSymbol(g_primes, &ps, sizeof ps); }
cudaError_t upload_primes_ntt(const PrimeSet& ps);
cudaError_t upload_primes_carry(const PrimeSet& ps);
cudaError_t upload_primes_batch(const PrimeSet& ps);

__device__ __forceinline__ u64 mulhi(u64 a, u64 b) { return __umul64hi(a, b); }

// q * p mod 2^64 for p = c*2^56 + 1: the low word is q, the high word gains
// (q_lo * c) << 24 — one 32-bit IMAD instead of a 64x64 product.
__device__ __forceinline__ u64 mul_p(u64 q, u32 c_hi) {
  u32 lo = (u32)q, hi = (u32)(q >> 32);
  hi += lo * c_hi;
  return ((u64)hi << 32) | lo;
}

// Compile-time constants of p_i = c_i * 2^56 + 1 (ntt_info.h:69-73).
template <int PR>
struct PrimeC {
  static constexpr u64 c = PR == 0 ? 27 : PR == 1 ? 58 : 87;
  static constexpr u64 p = c << 56 | 1;
  static constexpr u64 np = 0ull - p;  // 2^64 - p
  static constexpr u32 c_hi = (u32)(c << 24);
  static constexpr u64 m64 = PR == 0 ? 10 : PR == 1 ? 5 : 3;  // ceil(2^64 / p)
  // floor(2^(124+i) / p_i): the reference's Barrett constants (asmLinux.asm:926, 1075, 1236)
  static constexpr u64 mu = PR == 0 ? 0x97b425ed097b4259ull : PR == 1 ? 0x8d3dcb08d3dcb08aull : 0xbc52640bc52640baull;
};

// Shoup's remainder y*w - q*p with q = hi(y * wp) for a pair (w, wp =
// floor(w*2^64/p)+1): q is floor(y*w/p) or one more for any y < 2^64, so the
// result lies in [-p, p) as a signed value.  Written y*w + q*(2^64 - p), so
// the whole remainder is multiply-adds on the IMAD pipe rather than a product
// and a subtraction on the integer ALU (5 % more butterflies per second
// measured on GB300 in a register-only loop).
template <int PR>
__device__ __forceinline__ u64 shoup_rem_c(u64 y, u64 w, u64 wp) {
  return y * w + mulhi(y, wp) * PrimeC<PR>::np;
}
// The same reduced to [0, p).
template <int PR>
__device__ __forceinline__ u64 shoup_mul_c(u64 y, u64 w, u64 wp) {
  const u64 r = shoup_rem_c<PR>(y, w, wp);
  return ((i64)r < 0) ? r + PrimeC<PR>::p : r;
}

// w*y mod p in [0,p) from a Shoup pair (w, wp = floor(w*2^64/p)+1), y < 2^64.
// q is floor(y*w/p) or one more, so the low-word difference lies in [-p, p).
__device__ __forceinline__ u64 shoup_mul(u64 y, u64 w, u64 wp, u64 p, u32 c_hi) {
  u64 q = mulhi(y, wp);
  u64 r = y * w - mul_p(q, c_hi);
  return ((i64)r < 0) ? r + p : r;
}

// [0,2p) -> [0,p)
__device__ __forceinline__ u64 reduce2p(u64 x, u64 p) {
  u64 t = x - p;
  return ((i64)t < 0) ? x : t;
}

// limb mod p via q = hi(x * ceil(2^64/p)) (asmLoad, asmLinux.asm:891-904).
__device__ __forceinline__ u64 limb_mod(u64 x, u64 m64, u64 p, u32 c_hi) {
  u64 q = mulhi(x, m64);
  u64 r = x - mul_p(q, c_hi);
  return ((i64)r < 0) ? r + p : r;
}

// Forward CRT-tree butterfly (asmLinux.asm:409-445): x,y in [0,2p) ->
// (x mod p) + (w*y mod p), (x mod p) + p - (w*y mod p), both in [0,2p).
__device__ __forceinline__ void fwd_bfly(u64& x, u64& y, u64 w, u64 wp, u64 p, u32 c_hi) {
  u64 t = shoup_mul(y, w, wp, p, c_hi);
  u64 xr = reduce2p(x, p);
  x = xr + t;
  y = xr + p - t;
}

// Inverse butterfly (asmLinux.asm:595-630): x,y in [0,p) ->
// (x+y) mod p, (x-y)*w mod p.
__device__ __forceinline__ void inv_bfly(u64& x, u64& y, u64 w, u64 wp, u64 p, u32 c_hi) {
  u64 s = reduce2p(x + y, p);
  u64 t = shoup_mul(x - y + p, w, wp, p, c_hi);
  x = s;
  y = t;
}

// v * 2^-cl mod p for v in [0,p), p = c*2^56+1, 1 <= cl <= 56:
// with t = v-1 = h*2^cl + l, the result is h + 1 + (2^cl-1-l)*(p>>cl)
// (the identity used by asmINttShr, asmLinux.asm:821-859).
__device__ __forceinline__ u64 div_pow2(u64 v, u32 cl, u64 p) {
  u64 mask = (1ull << cl) - 1;
  i64 t = (i64)v - 1;
  u64 lo = (~(u64)t) & mask;
  return (u64)((t >> cl) + 1) + lo * (p >> cl);
}

// 128-bit accumulate helpers
struct U128 {
  u64 lo, hi;
};
__device__ __forceinline__ U128 mul_wide(u64 a, u64 b) { return U128{a * b, mulhi(a, b)}; }
__device__ __forceinline__ U128 add128(U128 a, U128 b) {
  U128 r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo);
  return r;
}

// Exact reduction of T < 2p^2 (pointwise sums) with the reference's Barrett
// constant; two conditional subtractions cover the quotient deficit.
__device__ __forceinline__ u64 barrett(U128 t, int i) {
  const u64 p = g_primes.p[i];
  const int sh = 60 + i;
  u64 top = (t.hi << (64 - sh)) | (t.lo >> sh);
  u64 q = mulhi(top, g_primes.mu[i]);
  u64 r = t.lo - mul_p(q, g_primes.c_hi[i]);
  if (r >= p) r -= p;
  if (r >= p) r -= p;
  return r;
}

}  // namespace nn

// scan_tiles.cuh — tile-level device code of the multiword carry scan
// (decoupled lookback) and its value producers, shared by the per-call kernels
// (carry.cu) and the persistent batch kernel (batch.cu).  See carry.cu for the
// scheme.
#pragma once

#include "nn_device.cuh"
#include "nn_internal.h"

namespace nn {

constexpr u32 kFlagAggregate = 1, kFlagInclusive = 2;
constexpr int kSpinLimit = 1 << 22;

struct W3 {
  u64 w0, w1, w2;
};

// Multiword sums as carry chains (add.cc / addc, mad.lo.cc / madc): the carry
// travels in the condition code instead of a compare and a select per word.
// A chain lives inside one asm statement, the only place the code survives.

// a + b mod 2^192.
__device__ __forceinline__ W3 add_w3(W3 a, W3 b) {
  W3 r;
  asm("add.cc.u64 %0, %3, %6;\n\t"
      "addc.cc.u64 %1, %4, %7;\n\t"
      "addc.u64 %2, %5, %8;"
      : "=l"(r.w0), "=l"(r.w1), "=l"(r.w2)
      : "l"(a.w0), "l"(a.w1), "l"(a.w2), "l"(b.w0), "l"(b.w1), "l"(b.w2));
  return r;
}

// y[0..8) += a0 + a1 * 2^64 (a carry rippling through all eight words);
// returns the carry out of the top word.
__device__ __forceinline__ u64 add_ripple8(u64 (&y)[8], u64 a0, u64 a1) {
  u64 c;
  asm("add.cc.u64 %0, %0, %9;\n\t"
      "addc.cc.u64 %1, %1, %10;\n\t"
      "addc.cc.u64 %2, %2, 0;\n\t"
      "addc.cc.u64 %3, %3, 0;\n\t"
      "addc.cc.u64 %4, %4, 0;\n\t"
      "addc.cc.u64 %5, %5, 0;\n\t"
      "addc.cc.u64 %6, %6, 0;\n\t"
      "addc.cc.u64 %7, %7, 0;\n\t"
      "addc.u64 %8, 0, 0;"
      : "+l"(y[0]), "+l"(y[1]), "+l"(y[2]), "+l"(y[3]), "+l"(y[4]), "+l"(y[5]), "+l"(y[6]), "+l"(y[7]), "=l"(c)
      : "l"(a0), "l"(a1));
  return c;
}

// Garner: x = r0 + p0*u + p0*p1*v with u = (r1-r0)/p0 mod p1 and
// v = ((r2-r0)/p0 - u)/p1 mod p2; residues in [0,p) after the inverse.
template <bool CG>
struct CrtProducerT {
  const u64* res;
  u64 L;
  u64 count;
  static constexpr bool kBulk = true;
  __device__ __forceinline__ W3 operator()(u64 k) const {
    if (k >= count) return W3{0, 0, 0};
    u64 x0, x1, x2;
    if (CG) {
      x0 = __ldcg(res + k);
      x1 = __ldcg(res + L + k);
      x2 = __ldcg(res + 2 * L + k);
    } else {
      x0 = res[k];
      x1 = res[L + k];
      x2 = res[2 * L + k];
    }
    return garner(x0, x1, x2);
  }
  // Eight consecutive positions from k0 (a multiple of 8) with 16-byte loads.
  __device__ __forceinline__ void bulk(u64 k0, W3 (&x)[kScanE]) const {
    if (k0 + kScanE > count) {
#pragma unroll
      for (int e = 0; e < kScanE; ++e) x[e] = (*this)(k0 + e);
      return;
    }
    u64 r[3][kScanE];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int e = 0; e < kScanE; e += 2) {
        const ulonglong2* q = reinterpret_cast<const ulonglong2*>(res + (u64)i * L + k0 + e);
        const ulonglong2 v = CG ? __ldcg(q) : *q;
        r[i][e] = v.x;
        r[i][e + 1] = v.y;
      }
#pragma unroll
    for (int e = 0; e < kScanE; ++e) x[e] = garner(r[0][e], r[1][e], r[2][e]);
  }
  __device__ __forceinline__ W3 garner(u64 x0, u64 x1, u64 x2) const {
    const PrimeSet& P = g_primes;
    constexpr u64 p0 = PrimeC<0>::p, p1 = PrimeC<1>::p, p2 = PrimeC<2>::p;
    const u64 d1 = x1 >= x0 ? x1 - x0 : x1 + p1 - x0;
    const u64 u = shoup_mul_c<1>(d1, P.inv01, P.inv01s);
    const u64 d2 = x2 >= x0 ? x2 - x0 : x2 + p2 - x0;
    const u64 t2 = shoup_mul_c<2>(d2, P.inv02, P.inv02s);
    const u64 e2 = t2 >= u ? t2 - u : t2 + p2 - u;
    const u64 v = shoup_mul_c<2>(e2, P.inv12, P.inv12s);
    // x0 + p0*u + (p01_lo + p01_hi*2^64)*v as one carry chain
    W3 r;
    asm("mad.lo.cc.u64 %0, %3, %4, %5;\n\t"
        "madc.hi.u64 %1, %3, %4, 0;\n\t"
        "mad.lo.cc.u64 %0, %6, %8, %0;\n\t"
        "madc.hi.cc.u64 %1, %6, %8, %1;\n\t"
        "madc.hi.u64 %2, %7, %8, 0;\n\t"
        "mad.lo.cc.u64 %1, %7, %8, %1;\n\t"
        "addc.u64 %2, %2, 0;"
        : "=l"(r.w0), "=l"(r.w1), "=l"(r.w2)
        : "l"(p0), "l"(u), "l"(x0), "l"(P.p01_lo), "l"(P.p01_hi), "l"(v));
    return r;
  }
};

typedef CrtProducerT<false> CrtProducer;


// A product split into pieces: the longer operand x (nx limbs) cut into P
// pieces of k limbs (the last one shorter), each multiplied by the shorter
// operand y (ny <= k + 1 limbs) through its own transform of L words, laid
// out [P][3][L].  Product coefficient j is the sum of coefficient j - i*k of
// piece i = floor(j/k) (the last piece for j beyond it) and coefficient
// j - (i-1)*k of piece i-1 when that is below k + ny - 1: at most two terms
// (k >= ny - 1), each below 2^160, so the sum fits three limbs.  k is a
// multiple of 8, so eight positions starting at a multiple of 8 lie in one
// piece.  Batch work items read other CTAs' results: .cg loads.
struct PieceCrtProducer {
  const u64* res;
  u64 L, k, P, ny, count;
  static constexpr bool kBulk = true;
  __device__ __forceinline__ CrtProducerT<true> piece(u64 i) const { return {res + i * 3 * L, L, L}; }
  __device__ __forceinline__ u64 piece_of(u64 j) const {
    const u64 i = j / k;
    return i < P ? i : P - 1;
  }
  __device__ __forceinline__ W3 operator()(u64 j) const {
    if (j >= count) return W3{0, 0, 0};
    const u64 i = piece_of(j), r = j - i * k;
    W3 x = piece(i)(r);
    if (i > 0 && r + 1 < ny) x = add_w3(x, piece(i - 1)(r + k));
    return x;
  }
  __device__ __forceinline__ void bulk(u64 k0, W3 (&x)[kScanE]) const {
    if (k0 + kScanE > count) {
#pragma unroll
      for (int e = 0; e < kScanE; ++e) x[e] = (*this)(k0 + e);
      return;
    }
    // one piece lookup for the eight positions; scalar loads keep fewer
    // values live than two eight-position vector loads
    const u64 i = piece_of(k0), r = k0 - i * k;
    const CrtProducerT<true> cur = piece(i), prev = piece(i > 0 ? i - 1 : 0);
    const bool ov = i > 0;
#pragma unroll
    for (int e = 0; e < kScanE; ++e) {
      x[e] = cur(r + e);
      if (ov && r + e + 1 < ny) x[e] = add_w3(x[e], prev(r + e + k));
    }
  }
};

// Column sums of a schoolbook product (asmMul1's column order, asmLinux.asm:188-278).
struct ColumnProducer {
  static constexpr bool kBulk = false;
  __device__ __forceinline__ void bulk(u64, W3 (&)[kScanE]) const {}
  const u64* a;
  u64 na;
  const u64* b;
  u64 nb;
  __device__ __forceinline__ W3 operator()(u64 k) const {
    W3 r{0, 0, 0};
    if (k + 1 >= na + nb) return r;
    const u64 lo = k >= nb ? k - nb + 1 : 0;
    const u64 hi = k < na - 1 ? k : na - 1;
    for (u64 i = lo; i <= hi; ++i) {
      const u64 x = a[i], y = b[k - i];
      const u64 pl = x * y, ph = mulhi(x, y);
      r.w0 += pl;
      const u64 c = r.w0 < pl;
      const u64 t = r.w1 + ph;
      r.w2 += t < ph;
      r.w1 = t + c;
      r.w2 += r.w1 < c;
    }
    return r;
  }
};

// Three-word values stored as three arrays (word i of position k at
// s[i * total + k]): the column sums of a base-case product, computed before
// the scan by one thread a position.
struct SumsProducer {
  static constexpr bool kBulk = true;
  const u64* s;
  u64 total;
  __device__ __forceinline__ W3 operator()(u64 k) const {
    if (k >= total) return W3{0, 0, 0};
    return W3{s[k], s[total + k], s[2 * total + k]};
  }
  __device__ __forceinline__ void bulk(u64 k0, W3 (&x)[kScanE]) const {
#pragma unroll
    for (int e = 0; e < kScanE; ++e) x[e] = (*this)(k0 + e);
  }
};

// x[k] + y[k - shift] (two words).
struct AddProducer {
  static constexpr bool kBulk = false;
  __device__ __forceinline__ void bulk(u64, W3 (&)[kScanE]) const {}
  const u64* x;
  u64 nx;
  const u64* y;
  u64 ny;
  u64 shift;
  __device__ __forceinline__ W3 operator()(u64 k) const {
    const u64 a = k < nx ? x[k] : 0;
    const u64 b = (k >= shift && k - shift < ny) ? y[k - shift] : 0;
    const u64 s = a + b;
    return W3{s, (u64)(s < a), 0};
  }
};

// x*B^xs + y*B^ys (add) or, as x*B^xs + ~(y*B^ys) + cin over `count`
// positions (sub), x*B^xs - y*B^ys - (1 - cin): with the scan run over
// count + 1 positions, the extra limb receives the carry out, which for a
// subtraction is 1 exactly when no borrow occurred.  Zero beyond count.
// With `flip` set, a nonzero *flip (a limb in device memory, read by every
// thread) swaps add and subtract, so a sign known only on the device picks
// the operation without a round trip to the host.
struct LinProducer {
  static constexpr bool kBulk = false;
  __device__ __forceinline__ void bulk(u64, W3 (&)[kScanE]) const {}
  const u64* x;
  u64 nx, xs;
  const u64* y;
  u64 ny, ys;
  u64 count;
  int sub, cin;
  const u64* flip;
  __device__ __forceinline__ W3 operator()(u64 k) const {
    if (k >= count) return W3{0, 0, 0};
    const u64 a = (k >= xs && k - xs < nx) ? x[k - xs] : 0;
    u64 b = (k >= ys && k - ys < ny) ? y[k - ys] : 0;
    u64 c = 0;
    if (sub ^ (flip != nullptr && __ldcg(flip) != 0)) {
      b = ~b;
      c = k == 0 ? (u64)cin : 0;
    }
    const u64 s = a + b;
    const u64 c1 = s < a;
    const u64 s2 = s + c;
    const u64 c2 = s2 < s;
    return W3{s2, c1 + c2, 0};
  }
};

__device__ __forceinline__ u32 flag_load(const u32* f) {
  u32 v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
  return v;
}
__device__ __forceinline__ void flag_store(u32* f, u32 v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(f), "r"(v) : "memory");
}
// Polls *f until it is nonzero, at most `limit` times; 0 means the wait gave up.
__device__ __forceinline__ u32 wait_flag(const u32* f, int limit) {
  u32 v;
  int spins = 0;
  while ((v = flag_load(f)) == 0) {
    if (++spins > limit) break;
    __nanosleep(32);
  }
  return v;
}

// One tile of the scan over positions [0, total): limbs below out_limit go to
// out, the rest to side.
// LOOKBACK: the tile takes its carry-in from its predecessors' status words
// (decoupled lookback); tiles of one scan must then start in increasing order
// (their predecessors already running), which the callers guarantee.
// Without LOOKBACK the tile takes carry-in 0 and records in flags[tile] its
// carry out for carry-in 0 (bit 0, generate) and whether a carry-in would pass
// straight through (bit 1, propagate: every limb all ones); a later step
// resolves the one-bit carries between tiles (carry.cu).
// The scan's shared scratch: one block per kernel, whatever producers its
// scan_tile instances take (a function's __shared__ variables exist once per
// CTA, while each instance of a template would get its own).
struct ScanShared {
  u64 h0[kScanThreads], h1[kScanThreads];
  u32 wg[kScanThreads / 32], wp[kScanThreads / 32];
  u32 cin;
  u64 x[kScanE][3];
};
__device__ __forceinline__ ScanShared& scan_shared() {
  __shared__ ScanShared sh;
  return sh;
}

template <class Prod, bool LOOKBACK = true>
__device__ __forceinline__ void scan_tile(const Prod& prod, u64 tile, u64 total, u64* out, u64 out_limit, u64* side,
                                          u32* flags, u32* err) {
  constexpr int E = kScanE;
  ScanShared& sh = scan_shared();
  u64* const s_h0 = sh.h0;
  u64* const s_h1 = sh.h1;
  u32* const s_wg = sh.wg;
  u32* const s_wp = sh.wp;
  u32& s_cin = sh.cin;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const u64 k0 = tile * kScanTile + (u64)tid * E;

  u64 y[E];
  u64 c0 = 0, c1 = 0;
  W3 xs[E];
  if (Prod::kBulk && k0 + E <= total) {
    prod.bulk(k0, xs);
  } else {
#pragma unroll
    for (int e = 0; e < E; ++e) xs[e] = k0 + e < total ? prod(k0 + e) : W3{0, 0, 0};
  }
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const W3 t = add_w3(xs[e], W3{c0, c1, 0});
    y[e] = t.w0;
    c0 = t.w1;
    c1 = t.w2;
  }
  s_h0[tid] = c0;
  s_h1[tid] = c1;
  // Overflow of the E positions before this tile: lanes 0..E-1 of warp 0
  // produce one value each, thread 0 chains them.
  u64(&s_x)[E][3] = sh.x;
  if (warp == 0) {
    if (lane < E && tile != 0) {
      const W3 x = prod(tile * kScanTile - E + lane);
      s_x[lane][0] = x.w0;
      s_x[lane][1] = x.w1;
      s_x[lane][2] = x.w2;
    }
    __syncwarp();
  }
  u64 hp0 = 0, hp1 = 0;
  if (tid == 0 && tile != 0) {
    u64 d0 = 0, d1 = 0;
    for (int e = 0; e < E; ++e) {
      const W3 t = add_w3(W3{s_x[e][0], s_x[e][1], s_x[e][2]}, W3{d0, d1, 0});
      d0 = t.w1;
      d1 = t.w2;
    }
    hp0 = d0;
    hp1 = d1;
  }
  __syncthreads();
  if (tid > 0) {
    hp0 = s_h0[tid - 1];
    hp1 = s_h1[tid - 1];
  }
  // u_t = lo_t + H_{t-1}; the carry out is the generate bit
  static_assert(E == 8, "the carry chains take eight limbs a thread");
  const u32 g = (u32)add_ripple8(y, hp0, hp1);
  u64 all = y[0];
#pragma unroll
  for (int e = 1; e < E; ++e) all &= y[e];
  const u32 pr = (all == ~0ull) & !g;

  const u32 G = __ballot_sync(0xffffffffu, g);
  const u32 GP = __ballot_sync(0xffffffffu, g | pr);
  if (lane == 0) {
    const u64 s0 = (u64)G + GP, s1 = (u64)G + GP + 1;
    s_wg[warp] = (u32)(s0 >> 32);
    s_wp[warp] = (u32)(s1 >> 32) & ~(u32)(s0 >> 32);
  }
  __syncthreads();
  if (tid == 0) {
    u32 c_if0 = 0, c_if1 = 1;
    for (int w = 0; w < kScanThreads / 32; ++w) {
      c_if0 = s_wg[w] | (s_wp[w] & c_if0);
      c_if1 = s_wg[w] | (s_wp[w] & c_if1);
    }
    const u32 tg = c_if0, tp = c_if1 & !c_if0;
    u32 cin = 0;
    if (!LOOKBACK) {
      flags[tile] = tg | (tp << 1);
    } else if (tile > 0) {
      flag_store(&flags[tile], kFlagAggregate | (tg << 2) | (tp << 3));
      long long j = (long long)tile - 1;
      for (;;) {
        if (j < 0) {
          cin = 0;
          break;
        }
        const u32 f = wait_flag(&flags[j], kSpinLimit);
        if (f == 0) {
          atomicExch(err, 1u);
          cin = 0;
          break;
        }
        if (f & kFlagInclusive) {
          cin = (f >> 2) & 1;
          break;
        }
        if ((f >> 2) & 1) {  // predecessor generates
          cin = 1;
          break;
        }
        if (!((f >> 3) & 1)) {  // predecessor kills
          cin = 0;
          break;
        }
        --j;  // predecessor propagates: look further back
      }
    }
    if (LOOKBACK) flag_store(&flags[tile], kFlagInclusive | ((tg | (tp & cin)) << 2));
    s_cin = cin;
  }
  __syncthreads();
  u32 wc = s_cin;
  for (int w = 0; w < warp; ++w) wc = s_wg[w] | (s_wp[w] & wc);
  const u64 sum = (u64)G + GP + wc;
  const u32 cin_bits = (u32)sum ^ G ^ GP;
  add_ripple8(y, (cin_bits >> lane) & 1, 0);  // its carry out is the next thread's carry-in, counted above
  if (k0 + E <= out_limit && k0 + E <= total && !(reinterpret_cast<uintptr_t>(out) & 15)) {
#pragma unroll
    for (int e = 0; e < E; e += 2) *reinterpret_cast<ulonglong2*>(out + k0 + e) = make_ulonglong2(y[e], y[e + 1]);
    return;
  }
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const u64 k = k0 + e;
    if (k < out_limit)
      out[k] = y[e];
    else if (k < total)
      side[k - out_limit] = y[e];
  }
}

}  // namespace nn

// ntt_tiles.cuh — tile-level device code of the NTT passes and the pointwise
// product, shared by the per-call kernels (ntt.cu) and the persistent batch
// kernel (batch.cu).  See ntt.cu for the level/pass decomposition.
//
// Every routine is specialised per prime (template PR), so the modulus and
// its reduction constants are immediates.  In-tile indices are 32-bit.  The
// shared-memory tile is padded by two words per 32 words, which spreads the
// strided accesses of the deepest levels over the banks.
#pragma once

#include "nn_device.cuh"

namespace nn {

// Exact reduction of T < 2p^2 with the reference's Barrett constant and two
// conditional subtractions (see barrett() in nn_device.cuh).
template <int PR>
__device__ __forceinline__ u64 barrett_c(U128 t) {
  constexpr u64 p = PrimeC<PR>::p;
  constexpr int sh = 60 + PR;
  const u64 top = (t.hi << (64 - sh)) | (t.lo >> sh);
  const u64 q = mulhi(top, PrimeC<PR>::mu);
  u64 r = t.lo + q * PrimeC<PR>::np;
  if (r >= p) r -= p;
  if (r >= p) r -= p;
  return r;
}

// Butterflies with per-prime lazy ranges.  q = hi(y * wp) with the
// reference's companion wp = floor(w*2^64/p)+1 is floor(y*w/p) or one more for
// any y < 2^64, so r = y*w - q*p lies in [-p, p) as a signed value.
//  - p0, p1 (4p < 2^64): forward values live in [0, 4p) and inverse values in
//    [0, 2p); r + p enters the sums directly (one conditional per butterfly).
//  - p2 (4p > 2^64): forward values in [0, 2p), inverse values in [0, p), as
//    in the reference (asmLinux.asm:409-445, 595-630).
template <int PR>
__device__ __forceinline__ void fwd_bfly_c(u64& x, u64& y, u64 w, u64 wp) {
  constexpr u64 p = PrimeC<PR>::p;
  if constexpr (PR < 2) {
    const u64 r = shoup_rem_c<PR>(y, w, wp);        // signed, in [-p, p)
    const u64 xr = x >= 2 * p ? x - 2 * p : x;      // [0, 2p)
    x = xr + r + p;                                 // [0, 4p)
    y = xr - r + p;                                 // [0, 4p)
  } else {  // asmLinux.asm:409-445: x, y in [0, 2p)
    const u64 t = shoup_mul_c<PR>(y, w, wp);
    const u64 xr = reduce2p(x, p);
    x = xr + t;
    y = xr + p - t;
  }
}
template <int PR>
__device__ __forceinline__ void inv_bfly_c(u64& x, u64& y, u64 w, u64 wp) {
  constexpr u64 p = PrimeC<PR>::p;
  if constexpr (PR < 2) {
    const u64 d = x - y + 2 * p;                    // (0, 4p)
    const u64 sum = x + y;                          // [0, 4p)
    x = sum >= 2 * p ? sum - 2 * p : sum;           // [0, 2p)
    y = shoup_rem_c<PR>(d, w, wp) + p;              // r in [-p, p) as a signed value; y in [0, 2p)
  } else {  // asmLinux.asm:595-630: x, y in [0, p)
    const u64 s = reduce2p(x + y, p);
    const u64 t = shoup_mul_c<PR>(x - y + p, w, wp);
    x = s;
    y = t;
  }
}
// Any lazy value of prime PR to [0, p).
template <int PR>
__device__ __forceinline__ u64 canon_c(u64 x) {
  constexpr u64 p = PrimeC<PR>::p;
  if constexpr (PR < 2) x = x >= 2 * p ? x - 2 * p : x;
  return reduce2p(x, p);
}

// Shared-memory padding: two words per 32, so pairs of words stay 16-byte
// aligned (16-byte async copies) while strided accesses of the deep levels
// spread over the banks.
__device__ __forceinline__ u32 pad16(u32 x) { return x + ((x >> 5) << 1); }

template <bool CG>
__device__ __forceinline__ ulonglong2 ld2(const u64* p) {
  const ulonglong2* q = reinterpret_cast<const ulonglong2*>(p);
  if (CG) return __ldcg(q);
  return *q;
}
template <bool CG>
__device__ __forceinline__ void st2(u64* p, ulonglong2 v) {
  ulonglong2* q = reinterpret_cast<ulonglong2*>(p);
  if (CG)
    __stcg(q, v);
  else
    *q = v;
}

// 16-byte asynchronous global -> shared copies (L2 only, as .cg loads), so a
// thread's loads of a tile are all in flight before any of them is waited on.
__device__ __forceinline__ void cp_async16(u64* smem, const u64* gmem) {
  const u32 d = (u32)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Words of the padded tile, rounded up to an even count so that the twiddle
// pairs a row pass (C = 2) keeps after the tile start on a 16-byte boundary.
__device__ __forceinline__ u32 tile_words(u32 nel) { return (nel + nel / 16 + 3) & ~1u; }

// The twiddle pairs of one tile of a row pass, staged in shared memory: local
// level j (global level lambda0 + j) uses pairs ksb*2^j + r, r < 2^j, kept at
// [2^j - 1, 2^(j+1) - 1).  Every deep-level pair is used by one thread only,
// so staging turns one dependent load per butterfly group into a batch of
// asynchronous copies at the start of the tile.
__device__ __forceinline__ void stage_twiddles(u64* tws, const u64* tw, u64 ksb, int R) {
  const u32 npairs = (1u << R) - 1;
  for (u32 q = threadIdx.x; q < npairs; q += blockDim.x) {
    const u32 j = 31 - __clz(q + 1);
    const u32 r = q + 1 - (1u << j);
    cp_async16(tws + 2 * q, tw + 2 * ((ksb << j) + r));
  }
}

// K levels [l, l+K) of a tile held in shared memory: each thread takes units
// of 2^K rows of one column and runs the radix-2^K network in registers.  The
// unit's rows are S = C * 2^nsub words apart, and the padded index is linear
// in the row: pad16(x0 + m*S) = pad16(x0) + m*S + 2*floor(m*S/32) for every
// unit of every tile shape used here, so each row is one add from the first.
// SC (inverse only): the group also scales its outputs by 2^-sc_sh to [0, p).
template <int K, int C, bool INV, int PR, bool PAD = true, bool SC = false>
__device__ __forceinline__ void level_group(u64* sm, int l, int R, u64 ksb, const u64* __restrict__ tw,
                                            const u64* tws, u32 sc_sh = 0) {
  const int nsub = R - l - K;
  const u32 units = (u32)C << (R - K);
  const u32 tmask = (1u << nsub) - 1;
  const u32 S = (u32)C << nsub;
  auto off = [S](u32 m) { return PAD ? m * S + (((m * S) >> 5) << 1) : m * S; };
  const ulonglong2* twv = reinterpret_cast<const ulonglong2*>(tw);
  const ulonglong2* twsv = reinterpret_cast<const ulonglong2*>(tws);
  // twiddle pair g of local level l + lv for the unit of block rb
  auto twiddle = [&](u32 rb, u64 bidx, int lv, int g) -> ulonglong2 {
    if (C == 2) return twsv[(1u << (l + lv)) - 1 + (rb << lv) + g];
    return __ldg(twv + ((bidx << lv) + g));
  };
  for (u32 u = threadIdx.x; u < units; u += blockDim.x) {
    const u32 i = u & (C - 1);
    const u32 v = u / C;
    const u32 rb = v >> nsub;
    const u32 row0 = (rb << (R - l)) + (v & tmask);
    const u64 bidx = (ksb << l) + rb;
    u64* sp = sm + (PAD ? pad16(row0 * C + i) : row0 * C + i);
    u64 x[1 << K];
#pragma unroll
    for (int m = 0; m < (1 << K); ++m) x[m] = sp[off(m)];
    if (!INV) {
#pragma unroll
      for (int lv = 0; lv < K; ++lv) {
        const int half = (1 << K) >> (lv + 1);
#pragma unroll
        for (int g = 0; g < (1 << lv); ++g) {
          const ulonglong2 wv = twiddle(rb, bidx, lv, g);
#pragma unroll
          for (int m = 0; m < half; ++m) fwd_bfly_c<PR>(x[g * 2 * half + m], x[g * 2 * half + m + half], wv.x, wv.y);
        }
      }
    } else {
#pragma unroll
      for (int lv = K - 1; lv >= 0; --lv) {
        const int half = (1 << K) >> (lv + 1);
#pragma unroll
        for (int g = 0; g < (1 << lv); ++g) {
          const ulonglong2 wv = twiddle(rb, bidx, lv, g);
#pragma unroll
          for (int m = 0; m < half; ++m) inv_bfly_c<PR>(x[g * 2 * half + m], x[g * 2 * half + m + half], wv.x, wv.y);
        }
      }
      if constexpr (SC) {
#pragma unroll
        for (int m = 0; m < (1 << K); ++m) x[m] = div_pow2(canon_c<PR>(x[m]), sc_sh, PrimeC<PR>::p);
      }
    }
#pragma unroll
    for (int m = 0; m < (1 << K); ++m) sp[off(m)] = x[m];
  }
}

// Levels per register group: as even as possible, at most kMaxGroupLevels, and at most what
// keeps every thread of the CTA busy (units = C * 2^(R-K) >= blockDim).
// Radix-8 at most: radix-16 units need ~100 registers and halve occupancy,
// which costs more than the saved shared-memory round trips.
constexpr int kMaxGroupLevels = 3;

__device__ __forceinline__ int group_cap(int C, int R) {
  int k = R < kMaxGroupLevels ? R : kMaxGroupLevels;
  while (k > 1 && ((u32)C << (R - k)) < blockDim.x) --k;
  return k;
}

template <int C, bool INV, int PR, bool PAD = true>
__device__ __forceinline__ void run_group(u64* sm, int k, int l, int R, u64 ksb, const u64* tw, const u64* tws) {
  if (k == 3)
    level_group<3, C, INV, PR, PAD>(sm, l, R, ksb, tw, tws);
  else if (k == 2)
    level_group<2, C, INV, PR, PAD>(sm, l, R, ksb, tw, tws);
  else
    level_group<1, C, INV, PR, PAD>(sm, l, R, ksb, tw, tws);
}

// Forward levels [l0, R) of the tile in shared memory.
template <int C, int PR, bool PAD = true>
__device__ __forceinline__ void tile_forward(u64* sm, int R, u64 ksb, const u64* tw, const u64* tws, int l0 = 0) {
  const int cap = group_cap(C, R);
  const int n = (R - l0 + cap - 1) / cap;
  for (int g = 0, l = l0; g < n; ++g) {
    const int k = (R - l + (n - g) - 1) / (n - g);
    run_group<C, false, PR, PAD>(sm, k, l, R, ksb, tw, tws);
    __syncthreads();
    l += k;
  }
}

// The same with R and the first level known at compile time (256 threads):
// the group schedule unrolls by template recursion, so every group's size,
// stride, unit count and twiddle offsets are constants and the index
// arithmetic folds away.  MAXK = 4 (radix-16 units) where the kernel has the
// registers for 16 residues per thread: the fused pass, at 11 levels (4 + 4
// + 3, one unit per thread).
__host__ __device__ constexpr int group_cap_ct(int C, int R, int maxk) {
  int k = R < maxk ? R : maxk;
  while (k > 1 && (C << (R - k)) < 256) --k;
  return k;
}
template <int C, int PR, int R, int L, int N, int G, bool PAD = true>
__device__ __forceinline__ void fwd_groups_ct(u64* sm, u64 ksb, const u64* tw, const u64* tws) {
  if constexpr (G < N) {
    constexpr int K = (R - L + (N - G) - 1) / (N - G);
    level_group<K, C, false, PR, PAD>(sm, L, R, ksb, tw, tws);
    __syncthreads();
    fwd_groups_ct<C, PR, R, L + K, N, G + 1, PAD>(sm, ksb, tw, tws);
  }
}
template <int C, int PR, int R, int L0, int MAXK = 3, bool PAD = true>
__device__ __forceinline__ void tile_forward_ct(u64* sm, u64 ksb, const u64* tw, const u64* tws) {
  constexpr int cap = group_cap_ct(C, R, MAXK);
  fwd_groups_ct<C, PR, R, L0, (R - L0 + cap - 1) / cap, 0, PAD>(sm, ksb, tw, tws);
}

// Inverse levels R-1 .. l_stop of the tile in shared memory.
template <int C, int PR, bool PAD = true>
__device__ __forceinline__ void tile_inverse(u64* sm, int R, u64 ksb, const u64* tw, const u64* tws, int l_stop = 0) {
  const int cap = group_cap(C, R);
  const int n = (R - l_stop + cap - 1) / cap;
  for (int g = 0, l = R; g < n; ++g) {
    const int k = (l - l_stop + (n - g) - 1) / (n - g);
    l -= k;
    run_group<C, true, PR, PAD>(sm, k, l, R, ksb, tw, tws);
    __syncthreads();
  }
}
// Inverse groups from level L (exclusive) down to LSTOP.
// SC: the last group also applies the scale 2^-sc_sh.
template <int C, int PR, int R, int L, int LSTOP, int N, int G, bool PAD = true, bool SC = false>
__device__ __forceinline__ void inv_groups_ct(u64* sm, u64 ksb, const u64* tw, const u64* tws, u32 sc_sh) {
  if constexpr (G < N) {
    constexpr int K = (L - LSTOP + (N - G) - 1) / (N - G);
    level_group<K, C, true, PR, PAD, SC && G + 1 == N>(sm, L - K, R, ksb, tw, tws, sc_sh);
    __syncthreads();
    inv_groups_ct<C, PR, R, L - K, LSTOP, N, G + 1, PAD, SC>(sm, ksb, tw, tws, sc_sh);
  }
}
template <int C, int PR, int R, int LSTOP, int MAXK = 3, bool PAD = true, bool SC = false>
__device__ __forceinline__ void tile_inverse_ct(u64* sm, u64 ksb, const u64* tw, const u64* tws, u32 sc_sh = 0) {
  constexpr int cap = group_cap_ct(C, R, MAXK);
  inv_groups_ct<C, PR, R, R, LSTOP, (R - LSTOP + cap - 1) / cap, 0, PAD, SC>(sm, ksb, tw, tws, sc_sh);
}

// Forward levels [l0, R) / inverse levels R-1 .. l_stop: the compile-time
// schedules for the tile shapes of the large transforms' pass plans (strided
// passes of 7-9 levels, contiguous passes of 10-11), the runtime loop
// otherwise.  Only the per-call kernels take them (CT); the batch kernel
// keeps one code path per width.
template <int C, int PR, bool CT, int MAXK = 3, bool PAD = true>
__device__ __forceinline__ void tile_forward_any(u64* sm, int R, u64 ksb, const u64* tw, const u64* tws, int l0) {
  if constexpr (CT && C == 2) {
    if (R == 11 && l0 == 0) return tile_forward_ct<C, PR, 11, 0, MAXK, PAD>(sm, ksb, tw, tws);
    if (R == 10 && l0 == 0) return tile_forward_ct<C, PR, 10, 0, 3, PAD>(sm, ksb, tw, tws);
  } else if constexpr (CT && C == 16) {
    if (R == 8 && l0 == 0) return tile_forward_ct<C, PR, 8, 0, MAXK, PAD>(sm, ksb, tw, tws);
    if (R == 8 && l0 == 1) return tile_forward_ct<C, PR, 8, 1, 3, PAD>(sm, ksb, tw, tws);
    if (R == 9 && l0 == 0) return tile_forward_ct<C, PR, 9, 0, 3, PAD>(sm, ksb, tw, tws);
    if (R == 9 && l0 == 1) return tile_forward_ct<C, PR, 9, 1, 3, PAD>(sm, ksb, tw, tws);
    if (R == 7 && l0 == 0) return tile_forward_ct<C, PR, 7, 0, 3, PAD>(sm, ksb, tw, tws);
    if (R == 7 && l0 == 1) return tile_forward_ct<C, PR, 7, 1, 3, PAD>(sm, ksb, tw, tws);
  }
  tile_forward<C, PR, PAD>(sm, R, ksb, tw, tws, l0);
}
// SC: a compile-time schedule also applies the scale 2^-sc_sh in its last
// group; returns whether it did (the runtime loop leaves the scale to the
// caller).
template <int C, int PR, bool CT, int MAXK = 3, bool PAD = true, bool SC = false>
__device__ __forceinline__ bool tile_inverse_any(u64* sm, int R, u64 ksb, const u64* tw, const u64* tws, int l_stop,
                                                 u32 sc_sh = 0) {
  if constexpr (CT && C == 2) {
    if (R == 11 && l_stop == 0) return tile_inverse_ct<C, PR, 11, 0, MAXK, PAD, SC>(sm, ksb, tw, tws, sc_sh), SC;
    if (R == 10 && l_stop == 0) return tile_inverse_ct<C, PR, 10, 0, 3, PAD, SC>(sm, ksb, tw, tws, sc_sh), SC;
  } else if constexpr (CT && C == 16) {
    if (R == 8 && l_stop == 0) return tile_inverse_ct<C, PR, 8, 0, MAXK, PAD, SC>(sm, ksb, tw, tws, sc_sh), SC;
    if (R == 9 && l_stop == 0) return tile_inverse_ct<C, PR, 9, 0, 3, PAD, SC>(sm, ksb, tw, tws, sc_sh), SC;
    if (R == 7 && l_stop == 0) return tile_inverse_ct<C, PR, 7, 0, 3, PAD, SC>(sm, ksb, tw, tws, sc_sh), SC;
  }
  tile_inverse<C, PR, PAD>(sm, R, ksb, tw, tws, l_stop);
  return false;
}

// Pointwise product of one group of 4 residues (a0..a3)(b0..b3), lazy forward
// values as inputs, [0,p) outputs: degree-1 residues mod (x^2 - w) and (x^2 + w),
// w = root[2g] (ntt_info.h:224-231, asmLinux.asm:910-1057).
template <int PR>
__device__ __forceinline__ void pointwise4(u64 (&o)[4], const u64 (&A)[4], const u64 (&Bv)[4], ulonglong2 wv) {
  constexpr u64 p = PrimeC<PR>::p;
  const u64 a0 = canon_c<PR>(A[0]), a1 = canon_c<PR>(A[1]), a2 = canon_c<PR>(A[2]), a3 = canon_c<PR>(A[3]);
  const u64 b0 = canon_c<PR>(Bv[0]), b1 = canon_c<PR>(Bv[1]), b2 = canon_c<PR>(Bv[2]), b3 = canon_c<PR>(Bv[3]);
  const u64 wb1 = shoup_mul_c<PR>(b1, wv.x, wv.y);
  const u64 wb3 = shoup_mul_c<PR>(b3, wv.x, wv.y);
  const u64 nwb3 = wb3 ? p - wb3 : 0;
  o[0] = barrett_c<PR>(add128(mul_wide(a0, b0), mul_wide(a1, wb1)));
  o[1] = barrett_c<PR>(add128(mul_wide(a0, b1), mul_wide(a1, b0)));
  o[2] = barrett_c<PR>(add128(mul_wide(a2, b2), mul_wide(a3, nwb3)));
  o[3] = barrett_c<PR>(add128(mul_wide(a2, b3), mul_wide(a3, b2)));
}

// The first pass's tile from limbs: element idx < nload (row idx / C, column
// idx % C) is limb base + row * 2^lg_s + column reduced mod p (zero at and
// beyond n_in); with `half`, every limb lies in the lower half of the
// transform and level 0 pairs it with a zero, so its residue also goes to
// element idx + nload.  PAD: the padded shared layout (pad16), else dense.
// kLoadBatch pairs of limbs a thread are loaded before any is reduced, so
// their latencies overlap (the compiler keeps generic loads in order with the
// shared-memory stores between them).
template <int C, int PR, bool PAD>
__device__ __forceinline__ void load_limbs_tile(u64* sm, const u64* in, u64 n_in, u64 base, int lg_s, u32 nload,
                                                bool half) {
  constexpr u64 p = PrimeC<PR>::p;
  constexpr u32 ch = PrimeC<PR>::c_hi;
  constexpr int LGC = C == 2 ? 1 : C == 16 ? 4 : C == 32 ? 5 : C == 64 ? 6 : 7;
  constexpr int kLoadBatch = 4;
  auto at = [](u32 i) { return PAD ? pad16(i) : i; };
  const bool vec = ((reinterpret_cast<unsigned long long>(in) & 15) == 0);
  for (u32 idx0 = 2 * threadIdx.x; idx0 < nload; idx0 += 2 * kLoadBatch * blockDim.x) {
    u64 x0[kLoadBatch], x1[kLoadBatch];
#pragma unroll
    for (int b = 0; b < kLoadBatch; ++b) {
      const u32 idx = idx0 + 2 * b * blockDim.x;
      const u64 pos = base + ((u64)(idx >> LGC) << lg_s) + (idx & (C - 1));
      x0[b] = 0;
      x1[b] = 0;
      if (idx < nload) {
        if (vec && pos + 1 < n_in) {
          const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(in + pos);
          x0[b] = v.x;
          x1[b] = v.y;
        } else {
          if (pos < n_in) x0[b] = in[pos];
          if (pos + 1 < n_in) x1[b] = in[pos + 1];
        }
      }
    }
#pragma unroll
    for (int b = 0; b < kLoadBatch; ++b) {
      const u32 idx = idx0 + 2 * b * blockDim.x;
      if (idx < nload) {
        const u64 pos = base + ((u64)(idx >> LGC) << lg_s) + (idx & (C - 1));
        const u64 r0 = pos < n_in ? limb_mod(x0[b], PrimeC<PR>::m64, p, ch) : 0;
        const u64 r1 = pos + 1 < n_in ? limb_mod(x1[b], PrimeC<PR>::m64, p, ch) : 0;
        sm[at(idx)] = r0;
        sm[at(idx + 1)] = r1;
        if (half) {
          sm[at(idx + nload)] = r0;
          sm[at(idx + nload + 1)] = r1;
        }
      }
    }
  }
}

// One tile of a pass over levels [lambda0, lambda0+R): C columns x 2^R rows of
// prime PR.  FIRST: `in` is n_in limbs (zero beyond) reduced on the fly;
// otherwise residues [3][2^s].  SCALE: multiply by 2^-(s-1) on the way out.
// FUSED (contiguous passes only): after the forward levels, multiply
// pointwise by the other operand's residues `other` and run the inverse
// levels before writing back.
// skip: the first `skip` local levels are not run (already done by the pass
// before).  A contiguous tile of R levels with skip = w is 2^w consecutive
// tiles of R - w levels, so small tiles can be worked on together.
template <int C, bool FIRST, bool INV, bool SCALE, bool CG, bool FUSED, int PR, int MAXK = 3>
__device__ __forceinline__ void pass_tile_p(u64* sm, const u64* in, u64* out, u64 n_in, int s, int lambda0, int R,
                                            const u64* __restrict__ tab, const u64* __restrict__ itab, u64 tab_stride,
                                            u64 tile, const u64* other, int skip) {
  constexpr u64 p = PrimeC<PR>::p;
  const u64 L = 1ull << s;
  const u64* tw = tab + (u64)PR * tab_stride;
  const int lg_s = s - lambda0 - R;
  const u64 tiles_per_sb = (1ull << lg_s) / C;
  const u64 ksb = tile / tiles_per_sb;
  const u64 base = (ksb << (lg_s + R)) + (tile % tiles_per_sb) * C;
  const u32 nel = (u32)C << R;
  static_assert(C == 2 || C == 16 || C == 32 || C == 64 || C == 128, "tile widths");
  constexpr int LGC = C == 2 ? 1 : C == 16 ? 4 : C == 32 ? 5 : C == 64 ? 6 : 7;

  // With every limb in the lower half of the transform (n_in <= L/2), level 0
  // pairs each limb with a zero: both outputs are the limb's residue, written
  // at once, and the tile starts at level 1.
  const bool half = FIRST && lambda0 == 0 && n_in <= (L >> 1);
  if (FIRST) {
    load_limbs_tile<C, PR, true>(sm, in, n_in, base, lg_s, half ? nel / 2 : nel, half);
  } else {
    const u64* src = in + (u64)PR * L;
    for (u32 idx = 2 * threadIdx.x; idx < nel; idx += 2 * blockDim.x) {
      const u64 pos = base + ((u64)(idx >> LGC) << lg_s) + (idx & (C - 1));
      cp_async16(sm + pad16(idx), src + pos);
    }
  }
  u64* tws = sm + tile_words(nel);
  if (C == 2) stage_twiddles(tws, tw, ksb, R);
  cp_async_wait_all();
  __syncthreads();

  if (!INV) {
    tile_forward_any<C, PR, !CG, MAXK>(sm, R, ksb, tw, tws, half ? 1 : skip);
    if (FUSED) {  // contiguous tile: smem index == position - base; other == nullptr squares
      const u64* oth = other ? other + (u64)PR * L : nullptr;
      const ulonglong2* twsv = reinterpret_cast<const ulonglong2*>(tws);
      const u32 deep = (1u << (R - 1)) - 1;  // local level R-1: the blocks of 4 residues
      for (u32 g4 = 4 * threadIdx.x; g4 < nel; g4 += 4 * blockDim.x) {
        const u64 Bv[4] = {sm[pad16(g4)], sm[pad16(g4 + 1)], sm[pad16(g4 + 2)], sm[pad16(g4 + 3)]};
        u64 A[4] = {Bv[0], Bv[1], Bv[2], Bv[3]};
        if (oth) {
          const ulonglong2 A0 = ld2<CG>(oth + base + g4), A1 = ld2<CG>(oth + base + g4 + 2);
          A[0] = A0.x;
          A[1] = A0.y;
          A[2] = A1.x;
          A[3] = A1.y;
        }
        u64 o[4];
        pointwise4<PR>(o, A, Bv, twsv[deep + (g4 >> 2)]);
#pragma unroll
        for (int q = 0; q < 4; ++q) sm[pad16(g4 + q)] = o[q];
      }
      __syncthreads();
      const u64* itw = itab + (u64)PR * tab_stride;
      stage_twiddles(tws, itw, ksb, R);
      cp_async_wait_all();
      __syncthreads();
      tile_inverse_any<C, PR, !CG, MAXK>(sm, R, ksb, itw, tws, skip);
    }
  } else {
    tile_inverse_any<C, PR, !CG>(sm, R, ksb, tw, tws, skip);
  }

  u64* dst = out + (u64)PR * L;
  for (u32 idx = 2 * threadIdx.x; idx < nel; idx += 2 * blockDim.x) {
    const u64 pos = base + ((u64)(idx >> LGC) << lg_s) + (idx & (C - 1));
    ulonglong2 v = make_ulonglong2(sm[pad16(idx)], sm[pad16(idx + 1)]);
    if (SCALE) {
      v.x = div_pow2(canon_c<PR>(v.x), (u32)(s - 1), p);
      v.y = div_pow2(canon_c<PR>(v.y), (u32)(s - 1), p);
    }
    st2<CG>(dst + pos, v);
  }
}

// MAXK: the largest register group (levels) the compile-time schedules may
// use; 4 only where the kernel has the registers for 16 residues a thread.
template <int C, bool FIRST, bool INV, bool SCALE, bool CG, bool FUSED = false, int MAXK = 3>
__device__ __forceinline__ void pass_tile(u64* sm, const u64* in, u64* out, u64 n_in, int s, int lambda0, int R,
                                          const u64* __restrict__ tab, u64 tab_stride, int prime, u64 tile,
                                          const u64* __restrict__ itab = nullptr, const u64* other = nullptr,
                                          int skip = 0) {
  if (prime == 0)
    pass_tile_p<C, FIRST, INV, SCALE, CG, FUSED, 0, MAXK>(sm, in, out, n_in, s, lambda0, R, tab, itab, tab_stride,
                                                         tile, other, skip);
  else if (prime == 1)
    pass_tile_p<C, FIRST, INV, SCALE, CG, FUSED, 1, MAXK>(sm, in, out, n_in, s, lambda0, R, tab, itab, tab_stride,
                                                         tile, other, skip);
  else
    pass_tile_p<C, FIRST, INV, SCALE, CG, FUSED, 2, MAXK>(sm, in, out, n_in, s, lambda0, R, tab, itab, tab_stride,
                                                         tile, other, skip);
}

// Pointwise product of one group g (4 residues) of prime i.
template <bool CG>
__device__ __forceinline__ void pointwise_group(u64* dst, const u64* a, const u64* b, u64 L,
                                                const u64* __restrict__ tab, u64 tab_stride, int i, u64 g) {
  const ulonglong2 wv = __ldg(reinterpret_cast<const ulonglong2*>(tab + (u64)i * tab_stride) + g);
  const u64 off = (u64)i * L + 4 * g;
  const ulonglong2 A0 = ld2<CG>(a + off), A1 = ld2<CG>(a + off + 2);
  const ulonglong2 B0 = ld2<CG>(b + off), B1 = ld2<CG>(b + off + 2);
  const u64 A[4] = {A0.x, A0.y, A1.x, A1.y}, Bv[4] = {B0.x, B0.y, B1.x, B1.y};
  u64 o[4];
  if (i == 0)
    pointwise4<0>(o, A, Bv, wv);
  else if (i == 1)
    pointwise4<1>(o, A, Bv, wv);
  else
    pointwise4<2>(o, A, Bv, wv);
  st2<CG>(dst + off, make_ulonglong2(o[0], o[1]));
  st2<CG>(dst + off + 2, make_ulonglong2(o[2], o[3]));
}

}  // namespace nn

// ntt_tiles.cuh — tile-level device code of the NTT passes and the pointwise
// product, shared by the per-call kernels (ntt.cu) and the persistent batch
// kernel (batch.cu).  See ntt.cu for the level/pass decomposition.
#pragma once

#include "nn_device.cuh"

namespace nn {

// Residue loads/stores.  The persistent kernel reads data other CTAs wrote
// earlier in the same launch, so it bypasses L1 (.cg); per-call kernels use
// plain accesses.
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

template <int K, int C, bool INV>
__device__ __forceinline__ void level_group(u64* sm, int l, int R, u64 ksb, const u64* __restrict__ tw, u64 p,
                                            u32 ch) {
  const int nsub = R - l - K;
  const int units = C << (R - K);
  for (int u = threadIdx.x; u < units; u += blockDim.x) {
    const int i = u & (C - 1);
    const int v = u / C;
    const int t0 = v & ((1 << nsub) - 1);
    const int rb = v >> nsub;
    const int row0 = (rb << (R - l)) + t0;
    const int rstep = 1 << nsub;
    const u64 bidx = (ksb << l) + (u64)rb;
    u64 x[1 << K];
#pragma unroll
    for (int m = 0; m < (1 << K); ++m) x[m] = sm[(row0 + m * rstep) * C + i];
    if (!INV) {
#pragma unroll
      for (int lv = 0; lv < K; ++lv) {
        const int half = (1 << K) >> (lv + 1);
#pragma unroll
        for (int g = 0; g < (1 << lv); ++g) {
          const ulonglong2 wv = __ldg(reinterpret_cast<const ulonglong2*>(tw) + ((bidx << lv) + g));
#pragma unroll
          for (int m = 0; m < half; ++m) fwd_bfly(x[g * 2 * half + m], x[g * 2 * half + m + half], wv.x, wv.y, p, ch);
        }
      }
    } else {
#pragma unroll
      for (int lv = K - 1; lv >= 0; --lv) {
        const int half = (1 << K) >> (lv + 1);
#pragma unroll
        for (int g = 0; g < (1 << lv); ++g) {
          const ulonglong2 wv = __ldg(reinterpret_cast<const ulonglong2*>(tw) + ((bidx << lv) + g));
#pragma unroll
          for (int m = 0; m < half; ++m) inv_bfly(x[g * 2 * half + m], x[g * 2 * half + m + half], wv.x, wv.y, p, ch);
        }
      }
    }
#pragma unroll
    for (int m = 0; m < (1 << K); ++m) sm[(row0 + m * rstep) * C + i] = x[m];
  }
}

// One tile of a pass over levels [lambda0, lambda0+R): C columns x 2^R rows of
// one prime.  FIRST: `in` is n_in limbs (zero beyond) reduced on the fly;
// otherwise residues [3][2^s].  SCALE: multiply by 2^-(s-1) on the way out.
template <int C, bool FIRST, bool INV, bool SCALE, bool CG>
__device__ __forceinline__ void pass_tile(u64* sm, const u64* in, u64* out, u64 n_in, int s, int lambda0, int R,
                                          const u64* __restrict__ tab, u64 tab_stride, int prime, u64 tile) {
  const u64 p = g_primes.p[prime];
  const u32 ch = g_primes.c_hi[prime];
  const u64 L = 1ull << s;
  const u64* tw = tab + (u64)prime * tab_stride;
  const int lg_s = s - lambda0 - R;
  const u64 tiles_per_sb = (1ull << lg_s) / C;
  const u64 ksb = tile / tiles_per_sb;
  const u64 base = (ksb << (lg_s + R)) + (tile % tiles_per_sb) * C;
  const int nel = C << R;

  if (FIRST) {
    const u64 m64 = g_primes.m64[prime];
    for (int idx = threadIdx.x; idx < nel; idx += blockDim.x) {
      const u64 pos = base + ((u64)(idx / C) << lg_s) + (idx & (C - 1));
      sm[idx] = pos < n_in ? limb_mod(in[pos], m64, p, ch) : 0;
    }
  } else {
    const u64* src = in + (u64)prime * L;
    for (int idx = 2 * threadIdx.x; idx < nel; idx += 2 * blockDim.x) {
      const u64 pos = base + ((u64)(idx / C) << lg_s) + (idx & (C - 1));
      const ulonglong2 v = ld2<CG>(src + pos);
      sm[idx] = v.x;
      sm[idx + 1] = v.y;
    }
  }
  __syncthreads();

  if (!INV) {
    for (int l = 0; l < R;) {
      const int k = R - l >= 3 ? 3 : R - l;
      if (k == 3)
        level_group<3, C, false>(sm, l, R, ksb, tw, p, ch);
      else if (k == 2)
        level_group<2, C, false>(sm, l, R, ksb, tw, p, ch);
      else
        level_group<1, C, false>(sm, l, R, ksb, tw, p, ch);
      __syncthreads();
      l += k;
    }
  } else {
    for (int l = R; l > 0;) {
      const int k = l >= 3 ? 3 : l;
      l -= k;
      if (k == 3)
        level_group<3, C, true>(sm, l, R, ksb, tw, p, ch);
      else if (k == 2)
        level_group<2, C, true>(sm, l, R, ksb, tw, p, ch);
      else
        level_group<1, C, true>(sm, l, R, ksb, tw, p, ch);
      __syncthreads();
    }
  }

  u64* dst = out + (u64)prime * L;
  for (int idx = 2 * threadIdx.x; idx < nel; idx += 2 * blockDim.x) {
    const u64 pos = base + ((u64)(idx / C) << lg_s) + (idx & (C - 1));
    ulonglong2 v = make_ulonglong2(sm[idx], sm[idx + 1]);
    if (SCALE) {
      v.x = div_pow2(v.x, (u32)(s - 1), p);
      v.y = div_pow2(v.y, (u32)(s - 1), p);
    }
    st2<CG>(dst + pos, v);
  }
}

// Pointwise product of one group g (4 residues) of prime i: degree-1 residues
// mod (x^2 - w) and (x^2 + w), w = root[2g] (ntt_info.h:224-231,
// asmLinux.asm:910-1057).  Inputs in [0,2p), outputs in [0,p).
template <bool CG>
__device__ __forceinline__ void pointwise_group(u64* dst, const u64* a, const u64* b, u64 L,
                                                const u64* __restrict__ tab, u64 tab_stride, int i, u64 g) {
  const u64 p = g_primes.p[i];
  const u32 ch = g_primes.c_hi[i];
  const ulonglong2 wv = __ldg(reinterpret_cast<const ulonglong2*>(tab + (u64)i * tab_stride) + g);
  const u64 off = (u64)i * L + 4 * g;
  const ulonglong2 A0 = ld2<CG>(a + off), A1 = ld2<CG>(a + off + 2);
  const ulonglong2 B0 = ld2<CG>(b + off), B1 = ld2<CG>(b + off + 2);
  const u64 a0 = reduce2p(A0.x, p), a1 = reduce2p(A0.y, p), a2 = reduce2p(A1.x, p), a3 = reduce2p(A1.y, p);
  const u64 b0 = reduce2p(B0.x, p), b1 = reduce2p(B0.y, p), b2 = reduce2p(B1.x, p), b3 = reduce2p(B1.y, p);
  const u64 wb1 = shoup_mul(b1, wv.x, wv.y, p, ch);
  const u64 wb3 = shoup_mul(b3, wv.x, wv.y, p, ch);
  const u64 nwb3 = wb3 ? p - wb3 : 0;
  ulonglong2 R0, R1;
  R0.x = barrett(add128(mul_wide(a0, b0), mul_wide(a1, wb1)), i);
  R0.y = barrett(add128(mul_wide(a0, b1), mul_wide(a1, b0)), i);
  R1.x = barrett(add128(mul_wide(a2, b2), mul_wide(a3, nwb3)), i);
  R1.y = barrett(add128(mul_wide(a2, b3), mul_wide(a3, b2)), i);
  st2<CG>(dst + off, R0);
  st2<CG>(dst + off + 2, R1);
}

}  // namespace nn

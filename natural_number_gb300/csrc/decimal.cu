// decimal.cu — the decimal digits of many short naturals at once: the leaves
// of the split tree of _format_dec (natural.h:994-1011).
//
// The reference splits each value down to 10^18-sized leaves (_dec_split,
// natural.h:953-967; the last split is div_base by 10^18, natural.h:566-573)
// and prints each leaf as 18 zero-padded digits (the first one unpadded).
// The decimal digits of a value are unique, so a node of the tree at any
// level has exactly one digit string of its width; here one warp takes one
// node and peels off its 18-digit groups from the low end by repeated exact
// division by 10^18, which is div_base's step applied 2^(i+1) times.
//
// A division's remainder chain runs from the top limb down, one limb after
// the other.  The warp splits it: lane l takes a segment of the node's limbs
// and reduces it to the map r -> (r * 2^(64 len) + segment) mod 10^18 (the
// remainder its segment leaves for a remainder r coming in from above); a
// scan over the lanes composes these maps from the top, so every lane knows
// the remainder entering its segment, and the lanes then form their
// quotient limbs at once.  A division costs two passes over a segment plus
// five compositions instead of one pass over the whole node.
//
// Layout: node k's limbs at w[k * stride ...), copied into shared memory,
// divided there; its digits go to out[k * width, (k + 1) * width), width =
// 18 * groups, most significant group first.
#include <cuda_runtime.h>

#include "nn_device.cuh"
#include "nn_internal.h"

#include <algorithm>
#include <atomic>

namespace nn {

namespace {

constexpr u64 kGroup = 1000000000000000000ull;  // 10^18 (dec_base_0)
constexpr int kNorm = 4;                        // leading zero bits of 10^18
constexpr u64 kGroupNorm = kGroup << kNorm;     // top bit set

// Division of the two-word value (u1, u0), u1 < d, by a normalised divisor d
// with its precomputed reciprocal v = floor((2^128 - 1) / d) - 2^64: the
// two-by-one division of Moller and Granlund, "Improved division by
// invariant integers" (IEEE Trans. Computers 60(2), 2011), Algorithm 4.
__device__ __forceinline__ u64 div_2by1(u64 u1, u64 u0, u64 d, u64 v, u64& r) {
  const u64 p_lo = v * u1;
  const u64 p_hi = __umul64hi(v, u1);
  u64 q0 = p_lo + u0;
  u64 q1 = p_hi + u1 + (q0 < p_lo ? 1 : 0);
  q1 += 1;
  u64 rr = u0 - q1 * d;
  if (rr > q0) {
    q1 -= 1;
    rr += d;
  }
  if (rr >= d) {
    q1 += 1;
    rr -= d;
  }
  r = rr;
  return q1;
}

// The 18 digits of x < 10^18, zero-padded, as nine 2-byte stores (o even).
__device__ __forceinline__ void put18(char* o, u64 x) {
  u32 hi = (u32)(x / 1000000000ull);
  u32 lo = (u32)(x - (u64)hi * 1000000000ull);
  unsigned char d[18];
#pragma unroll
  for (int t = 8; t >= 0; --t) {
    d[9 + t] = (unsigned char)('0' + lo % 10);
    lo /= 10;
    d[t] = (unsigned char)('0' + hi % 10);
    hi /= 10;
  }
  unsigned short* o2 = reinterpret_cast<unsigned short*>(o);
#pragma unroll
  for (int t = 0; t < 9; ++t) o2[t] = (unsigned short)(d[2 * t] | (d[2 * t + 1] << 8));
}

// (a * b) mod 10^18 for a, b < 10^18: the product's high word is below the
// divisor, as the two-by-one division wants after the shift by kNorm.
__device__ __forceinline__ u64 mulmod_group(u64 a, u64 b, u64 v) {
  const u64 lo = a * b, hi = __umul64hi(a, b);
  u64 r;
  div_2by1((hi << kNorm) | (lo >> (64 - kNorm)), lo << kNorm, kGroupNorm, v, r);
  return r >> kNorm;
}

// 2^(64 j) mod 10^18 for the segment lengths j <= kMaxSegment.
constexpr int kMaxSegment = 256;
constexpr int kMaxDevices = 64;
__constant__ u64 c_limb_pow[kMaxSegment + 1];

// One warp a node; `per_cta` warps a CTA, each with `stride` limbs of shared
// memory.  A division pass over the current m limbs: segments of
// ceil(m / 32) limbs, lane l holding limbs [l * seg, (l + 1) * seg).
__global__ void __launch_bounds__(128) dec_groups_kernel(const u64* __restrict__ w, u64 stride,
                                                         const u32* __restrict__ len, u64 n, u32 groups, u64 v,
                                                         char* out) {
  extern __shared__ u64 node_sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u64 k = (u64)blockIdx.x * (blockDim.x >> 5) + warp;
  if (k >= n) return;  // a whole warp leaves together
  u64* a = node_sm + (u64)warp * stride;
  u32 m = len[k];
  for (u32 j = lane; j < m; j += 32) a[j] = w[k * stride + j];
  __syncwarp();
  char* o = out + k * (u64)groups * 18;
  for (u32 g = groups; g-- > 0;) {
    const u32 seg = (m + 31) / 32;  // at most kMaxSegment: m is below 32 * kMaxSegment
    const u32 lo = min(lane * seg, m), hi = min(lo + seg, m);
    // this lane's map r -> A r + B: B = its segment mod 10^18, A = 2^(64 len) mod 10^18
    u64 rn = 0;
    for (u32 j = hi; j-- > lo;) {
      const u64 x = a[j];
      div_2by1(rn | (x >> (64 - kNorm)), x << kNorm, kGroupNorm, v, rn);
    }
    u64 A = c_limb_pow[hi - lo], B = rn >> kNorm;
    // compose from the top: lane l ends with the map of segments l .. 31
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const u64 A2 = __shfl_down_sync(0xffffffffu, A, d), B2 = __shfl_down_sync(0xffffffffu, B, d);
      if (lane + d < 32) {
        B = mulmod_group(A, B2, v) + B;
        if (B >= kGroup) B -= kGroup;
        A = mulmod_group(A, A2, v);
      }
    }
    const u64 group = __shfl_sync(0xffffffffu, B, 0);  // the remainder of the whole node
    u64 rin = __shfl_down_sync(0xffffffffu, B, 1);
    if (lane == 31) rin = 0;
    // the quotient limbs, every segment at once
    rn = rin << kNorm;
    u64 top_q = 1;
    for (u32 j = hi; j-- > lo;) {
      const u64 x = a[j];
      const u64 q = div_2by1(rn | (x >> (64 - kNorm)), x << kNorm, kGroupNorm, v, rn);
      a[j] = q;
      if (j == m - 1) top_q = q;
    }
    // the value loses at most one limb a division (10^18 < 2^64)
    const bool lost = __any_sync(0xffffffffu, m > 0 && hi == m && hi > lo && top_q == 0);
    __syncwarp();
    if (lost) --m;
    if (lane == 0) put18(o + (u64)g * 18, group);
  }
}

}  // namespace

cudaError_t dec_groups(const u64* w, u64 stride, const u32* len, u64 n, u32 groups, char* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (stride > (u64)32 * kMaxSegment || stride % 2) return cudaErrorInvalidValue;
  // 2^(64 j) mod 10^18 into the constant bank, once per device (each device
  // has its own copy of c_limb_pow)
  static std::atomic<bool> powers[kMaxDevices];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (!powers[dev].load()) {
    u64 t[kMaxSegment + 1];
    unsigned __int128 x = 1;
    for (int j = 0; j <= kMaxSegment; ++j, x = (x << 64) % kGroup) t[j] = (u64)x;
    e = cudaMemcpyToSymbol(c_limb_pow, t, sizeof t);
    if (e != cudaSuccess) return e;
    powers[dev].store(true);
  }
  const unsigned __int128 all = ~(unsigned __int128)0;
  const u64 v = (u64)(all / kGroupNorm);  // floor((2^128-1)/d) - 2^64: the 2^64 bit drops in the cast
  // warps a CTA: as many nodes as 48 KiB of shared memory holds, at most four
  const unsigned per_cta = (unsigned)std::max<u64>(1, std::min<u64>(4, (48 * 1024) / (8 * stride)));
  const size_t smem = (size_t)per_cta * stride * 8;
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(dec_groups_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  launch_begin("dec_groups", st);
  dec_groups_kernel<<<(unsigned)((n + per_cta - 1) / per_cta), 32 * per_cta, smem, st>>>(w, stride, len, n, groups, v,
                                                                                          out);
  launch_end(st);
  return cudaGetLastError();
}

}  // namespace nn

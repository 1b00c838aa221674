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
// Layout: node k's len[k] limbs at nodes[k], copied into `stride` limbs of
// shared memory and divided there; its digits go to out[k * width, (k + 1) *
// width), width = 18 * groups, most significant group first.
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
__global__ void __launch_bounds__(128) dec_groups_kernel(const u64* const* __restrict__ nodes, u64 stride,
                                                         const u32* __restrict__ len, u64 n, u32 groups, u64 v,
                                                         char* out) {
  extern __shared__ u64 node_sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u64 k = (u64)blockIdx.x * (blockDim.x >> 5) + warp;
  if (k >= n) return;  // a whole warp leaves together
  u64* a = node_sm + (u64)warp * stride;
  u32 m = len[k];
  const u64* w = nodes[k];
  for (u32 j = lane; j < m; j += 32) a[j] = w[j];
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

// out = in >> shift bits (n_out limbs, in read as zero past n_in): block
// (x, y) covers limbs [x * 4096, x * 4096 + 4096) of job y.
__global__ void __launch_bounds__(256) shr_batch_kernel(const ShrJob* __restrict__ jobs) {
  const ShrJob J = jobs[blockIdx.y];
  const u64 ls = J.shift >> 6;
  const u32 bs = (u32)(J.shift & 63);
  for (u64 t = (u64)blockIdx.x * kShrChunk + threadIdx.x; t < J.n_out && t < (u64)(blockIdx.x + 1) * kShrChunk;
       t += blockDim.x) {
    const u64 i = t + ls;
    const u64 a = i < J.n_in ? J.in[i] : 0, b = i + 1 < J.n_in ? J.in[i + 1] : 0;
    J.out[t] = bs ? (a >> bs) | (b << (64 - bs)) : a;
  }
}

// One warp: x (nx limbs) against y (ny limbs): -1, 0 or 1.
__device__ int warp_cmp(const u64* x, u64 nx, const u64* y, u64 ny, u32 lane) {
  const u64 n = nx > ny ? nx : ny;
  for (u64 top = (n + 31) & ~31ull; top > 0; top -= 32) {
    const u64 k = top - 32 + lane;
    const u64 a = k < nx ? x[k] : 0, b = k < ny ? y[k] : 0;
    const u32 d = __ballot_sync(0xffffffffu, a != b);
    if (d) {
      const int hl = 31 - __clz(d);
      const int gt = __shfl_sync(0xffffffffu, a > b ? 1 : 0, hl);
      return gt ? 1 : -1;
    }
  }
  return 0;
}

// One warp: x (n limbs) += y (or -= y with `sub`), carries by ballots; past
// y's limbs the walk ends once no carry (borrow) is left.
__device__ void warp_addsub(u64* x, u64 n, const u64* y, u64 ny, bool sub, u32 lane) {
  const u64 flip = sub ? ~0ull : 0;
  const u32 idle = sub ? 1 : 0;  // the carry word when nothing is pending
  u32 carry = idle;
  for (u64 base = 0; base < n; base += 32) {
    if (base >= ny && carry == idle) break;
    const u64 k = base + lane;
    const u64 a = k < n ? x[k] : 0, b = (k < ny ? y[k] : 0) ^ flip;
    const u64 sum = a + b;
    const u32 G = __ballot_sync(0xffffffffu, sum < a), GP = __ballot_sync(0xffffffffu, sum < a || sum == ~0ull);
    const u64 t = (u64)G + GP + carry;
    if (k < n) x[k] = sum + ((((u32)t ^ G ^ GP) >> lane) & 1);
    carry = (u32)(t >> 32);
  }
}

// The split's correction (natural.h:962-965): while lo >= base, hi += 1 and
// lo -= base, at most kMaxFix times (an error otherwise); zero[k] = hi == 0.
constexpr int kMaxFix = 8;
__global__ void __launch_bounds__(256) dec_fix_kernel(const DecFixJob* __restrict__ jobs, u64 m, const u64* base,
                                                      u64 nb, u32* zero, u32* err) {
  const u64 k = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const u32 lane = threadIdx.x & 31;
  if (k >= m) return;  // whole warps leave together
  const DecFixJob J = jobs[k];
  const u64 one = 1;
  int it = 0;
  for (; it < kMaxFix && warp_cmp(J.lo, J.n_lo, base, nb, lane) >= 0; ++it) {
    warp_addsub(J.lo, J.n_lo, base, nb, true, lane);
    __syncwarp();
    warp_addsub(J.hi, J.n_hi, &one, 1, false, lane);
    __syncwarp();
  }
  if (it == kMaxFix && lane == 0) atomicExch(err, 1u);
  // hi == 0: the walk ends at the first nonzero limb (within the first 32
  // limbs but for a zero or nearly zero hi)
  u32 nz = 0;
  for (u64 i0 = 0; i0 < J.n_hi && !nz; i0 += 32) {
    const u64 i = i0 + lane;
    nz = __any_sync(0xffffffffu, i < J.n_hi && J.hi[i] != 0);
  }
  if (lane == 0) zero[k] = !nz;
}

__global__ void __launch_bounds__(256) dec_need_kernel(const DecFixJob* __restrict__ jobs, u64 m, const u64* base,
                                                       u64 nb, u32* need) {
  const u64 k = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const u32 lane = threadIdx.x & 31;
  if (k >= m) return;  // whole warps leave together
  const int c = warp_cmp(jobs[k].lo, jobs[k].n_lo, base, nb, lane);
  if (lane == 0) need[k] = c >= 0;
}

// hi += 1 for the jobs with need[k] set, one warp a job (the walk stops once
// no carry is left).
__global__ void __launch_bounds__(256) dec_inc_kernel(const DecFixJob* __restrict__ jobs, u64 m,
                                                      const u32* __restrict__ need) {
  const u64 k = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const u32 lane = threadIdx.x & 31;
  if (k >= m || !need[k]) return;  // whole warps leave together
  const u64 one = 1;
  warp_addsub(jobs[k].hi, jobs[k].n_hi, &one, 1, false, lane);
}

}  // namespace

cudaError_t dec_groups(const u64* const* nodes, u64 stride, const u32* len, u64 n, u32 groups, char* out,
                       cudaStream_t st) {
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
  dec_groups_kernel<<<(unsigned)((n + per_cta - 1) / per_cta), 32 * per_cta, smem, st>>>(nodes, stride, len, n, groups,
                                                                                          v, out);
  launch_end(st);
  return cudaGetLastError();
}

cudaError_t shr_batch(const ShrJob* d_jobs, const std::vector<ShrJob>& jobs, cudaStream_t st) {
  u64 chunks = 1;
  for (const ShrJob& j : jobs) chunks = std::max<u64>(chunks, (j.n_out + kShrChunk - 1) / kShrChunk);
  for (u64 j0 = 0; j0 < jobs.size(); j0 += 65535) {  // grid y holds at most 65535 jobs
    const unsigned ny = (unsigned)std::min<u64>(65535, jobs.size() - j0);
    launch_begin("dec_shift", st);
    shr_batch_kernel<<<dim3((unsigned)chunks, ny), 256, 0, st>>>(d_jobs + j0);
    launch_end(st);
  }
  return cudaGetLastError();
}

cudaError_t dec_need(const DecFixJob* d_jobs, u64 m, const u64* base, u64 nb, u32* need, cudaStream_t st) {
  if (m == 0) return cudaSuccess;
  launch_begin("dec_need", st);
  dec_need_kernel<<<(unsigned)((m * 32 + 255) / 256), 256, 0, st>>>(d_jobs, m, base, nb, need);
  launch_end(st);
  return cudaGetLastError();
}

cudaError_t dec_inc(const DecFixJob* d_jobs, u64 m, const u32* need, cudaStream_t st) {
  if (m == 0) return cudaSuccess;
  launch_begin("dec_inc", st);
  dec_inc_kernel<<<(unsigned)((m * 32 + 255) / 256), 256, 0, st>>>(d_jobs, m, need);
  launch_end(st);
  return cudaGetLastError();
}

cudaError_t dec_fix(const DecFixJob* d_jobs, u64 m, const u64* base, u64 nb, u32* zero, u32* err, cudaStream_t st) {
  if (m == 0) return cudaSuccess;
  launch_begin("dec_fix", st);
  dec_fix_kernel<<<(unsigned)((m * 32 + 255) / 256), 256, 0, st>>>(d_jobs, m, base, nb, zero, err);
  launch_end(st);
  return cudaGetLastError();
}

}  // namespace nn

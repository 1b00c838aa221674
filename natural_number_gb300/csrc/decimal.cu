// decimal.cu — the decimal digits of many short naturals at once: the leaves
// of the split tree of _format_dec (natural.h:994-1011).
//
// The reference splits each value down to 10^18-sized leaves (_dec_split,
// natural.h:953-967; the last split is div_base by 10^18, natural.h:566-573)
// and prints each leaf as 18 zero-padded digits (the first one unpadded).
// The decimal digits of a value are unique, so a node of the tree at any
// level has exactly one digit string of its width; here one thread takes one
// node and peels off its 18-digit groups from the low end by repeated exact
// division by 10^18, which is div_base's step applied 2^(i+1) times.
//
// Layout: the nodes' limbs are limb-major, w[j * n + k] = limb j of node k,
// so that the threads of a warp, each on its own node, touch consecutive
// words.  Node k's digits go to out[k * width, (k + 1) * width), width = 18 *
// groups, most significant group first.  Every division is done in place.
#include <cuda_runtime.h>

#include "nn_device.cuh"
#include "nn_internal.h"

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

// Limbs a thread loads at once while it divides the previous batch: the
// division chain runs from the top limb down, so the loads of the next
// kChunk limbs are independent of it and their latency overlaps the work.
constexpr int kChunk = 8;

__global__ void __launch_bounds__(128) dec_groups_kernel(u64* w, const u32* len, u64 n, u32 groups, u64 v, char* out) {
  const u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  u32 m = len[k];
  char* o = out + k * (u64)groups * 18;
  // limb j of this node, or 0 below limb 0
  auto load = [&](long long j) -> u64 { return j >= 0 ? w[(u64)j * n + k] : 0; };
  for (u32 g = groups; g-- > 0;) {
    // node := floor(node / 10^18), remainder r: the dividend is shifted left
    // by kNorm bits on the fly (u1 = 16 r + top bits of the limb, u1 < 16 * 10^18)
    u64 rn = 0;
    const u32 top = m;
    u64 cur[kChunk], nxt[kChunk];
#pragma unroll
    for (int t = 0; t < kChunk; ++t) cur[t] = load((long long)top - 1 - t);
    for (long long j0 = (long long)top - 1; j0 >= 0; j0 -= kChunk) {
#pragma unroll
      for (int t = 0; t < kChunk; ++t) nxt[t] = load(j0 - kChunk - t);
#pragma unroll
      for (int t = 0; t < kChunk; ++t) {
        const long long j = j0 - t;
        if (j >= 0) {
          const u64 a = cur[t];
          const u64 q = div_2by1(rn | (a >> (64 - kNorm)), a << kNorm, kGroupNorm, v, rn);
          w[(u64)j * n + k] = q;
          if (j == (long long)top - 1 && q == 0) --m;  // at most one limb lost a division (10^18 < 2^64)
        }
      }
#pragma unroll
      for (int t = 0; t < kChunk; ++t) cur[t] = nxt[t];
    }
    put18(o + (u64)g * 18, rn >> kNorm);
  }
}

}  // namespace

cudaError_t dec_groups(u64* w, const u32* len, u64 n, u32 groups, char* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const unsigned __int128 all = ~(unsigned __int128)0;
  const u64 v = (u64)(all / kGroupNorm);  // floor((2^128-1)/d) - 2^64: the 2^64 bit drops in the cast
  const unsigned threads = 128;
  launch_begin("dec_groups", st);
  dec_groups_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, st>>>(w, len, n, groups, v, out);
  launch_end(st);
  return cudaGetLastError();
}

}  // namespace nn

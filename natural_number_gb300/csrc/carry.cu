// carry.cu — multiword carry propagation on sm_103a: CRT recombination fused
// with a decoupled-lookback carry scan, plus the same scan driving the
// schoolbook base case and shifted multiword adds.
//
// Each position k contributes a three-word value x_k (< 2^186) at limb k; the
// output is sum_k x_k * B^k, B = 2^64 (asmCRT, asmLinux.asm:1369-1450, does
// this serially with a two-word running carry).  Thread t of a tile owns E
// consecutive positions and forms S_t = sum_e x_{k0+e} B^e = lo_t + H_t B^E
// with a zero carry-in (H_t: two words).  Adding the neighbour's H_{t-1} into
// lo_t leaves an E-limb value u_t plus a one-bit generate g_t; the remaining
// carries are one bit each (propagate p_t = u_t is all ones; g_t and p_t are
// exclusive), resolved by warp ballots inside a tile and by a decoupled
// lookback on one status word per tile across tiles.  Tile ids come from an
// atomic counter so every predecessor of a tile is already resident; each
// wait is bounded and records an error instead of hanging.
#include <cuda_runtime.h>

#include "nn_device.cuh"
#include "nn_internal.h"

namespace nn {

NN_DEFINE_PRIME_UPLOADER(upload_primes_carry)

namespace {

constexpr u32 kFlagAggregate = 1, kFlagInclusive = 2;
constexpr int kSpinLimit = 1 << 22;

struct W3 {
  u64 w0, w1, w2;
};

// Garner: x = r0 + p0*u + p0*p1*v with u = (r1-r0)/p0 mod p1 and
// v = ((r2-r0)/p0 - u)/p1 mod p2; residues in [0,p) after the inverse.
struct CrtProducer {
  const u64* res;
  u64 L;
  u64 count;
  __device__ __forceinline__ W3 operator()(u64 k) const {
    if (k >= count) return W3{0, 0, 0};
    const PrimeSet& P = g_primes;
    const u64 x0 = res[k], x1 = res[L + k], x2 = res[2 * L + k];
    const u64 p1 = P.p[1], p2 = P.p[2];
    const u64 d1 = x1 >= x0 ? x1 - x0 : x1 + p1 - x0;
    const u64 u = shoup_mul(d1, P.inv01, P.inv01s, p1, P.c_hi[1]);
    const u64 d2 = x2 >= x0 ? x2 - x0 : x2 + p2 - x0;
    const u64 t2 = shoup_mul(d2, P.inv02, P.inv02s, p2, P.c_hi[2]);
    const u64 e2 = t2 >= u ? t2 - u : t2 + p2 - u;
    const u64 v = shoup_mul(e2, P.inv12, P.inv12s, p2, P.c_hi[2]);
    // lo = p0*u + x0
    u64 l0 = P.p[0] * u, l1 = mulhi(P.p[0], u);
    l0 += x0;
    l1 += (l0 < x0);
    // m = p01_lo * v, h = p01_hi * v
    const u64 m0 = P.p01_lo * v, m1 = mulhi(P.p01_lo, v);
    const u64 h0 = P.p01_hi * v, h1 = mulhi(P.p01_hi, v);
    W3 r;
    r.w0 = l0 + m0;
    u64 c = r.w0 < l0;
    u64 s1 = l1 + m1;
    u64 c2 = s1 < l1;
    s1 += h0;
    c2 += s1 < h0;
    s1 += c;
    c2 += s1 < c;
    r.w1 = s1;
    r.w2 = h1 + c2;
    return r;
  }
};

// Column sums of a schoolbook product (asmMul1's column order, asmLinux.asm:188-278).
struct ColumnProducer {
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

// x[k] + y[k - shift] (two words).
struct AddProducer {
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

__device__ __forceinline__ u32 flag_load(const u32* f) {
  u32 v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
  return v;
}
__device__ __forceinline__ void flag_store(u32* f, u32 v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(f), "r"(v) : "memory");
}

// Scans positions [0, total): limbs below out_limit go to out, the rest to side.
template <class Prod>
__global__ void __launch_bounds__(kScanThreads) scan_kernel(Prod prod, u64 total, u64* out, u64 out_limit,
                                                            u64* side, u32* flags, u32* counter, u32* err) {
  constexpr int E = kScanE;
  __shared__ u64 s_h0[kScanThreads], s_h1[kScanThreads];
  __shared__ u32 s_wg[kScanThreads / 32], s_wp[kScanThreads / 32];
  __shared__ u32 s_tile, s_cin;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  const u64 tile = s_tile;
  const u64 k0 = tile * kScanTile + (u64)tid * E;

  u64 y[E];
  u64 c0 = 0, c1 = 0;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const u64 k = k0 + e;
    W3 x = k < total ? prod(k) : W3{0, 0, 0};
    const u64 s0 = x.w0 + c0;
    const u64 cy0 = s0 < c0;
    u64 s1 = x.w1 + c1;
    u64 cy1 = s1 < c1;
    s1 += cy0;
    cy1 += s1 < cy0;
    y[e] = s0;
    c0 = s1;
    c1 = x.w2 + cy1;
  }
  s_h0[tid] = c0;
  s_h1[tid] = c1;
  u64 hp0 = 0, hp1 = 0;
  if (tid == 0 && k0 != 0) {  // overflow of the E positions before this tile
    u64 d0 = 0, d1 = 0;
    for (int e = 0; e < E; ++e) {
      W3 x = prod(k0 - E + e);
      const u64 s0 = x.w0 + d0;
      const u64 cy0 = s0 < d0;
      u64 s1 = x.w1 + d1;
      u64 cy1 = s1 < d1;
      s1 += cy0;
      cy1 += s1 < cy0;
      d0 = s1;
      d1 = x.w2 + cy1;
    }
    hp0 = d0;
    hp1 = d1;
  }
  __syncthreads();
  if (tid > 0) {
    hp0 = s_h0[tid - 1];
    hp1 = s_h1[tid - 1];
  }
  // u_t = lo_t + H_{t-1}
  {
    u64 t = y[0] + hp0;
    u64 cy = t < hp0;
    y[0] = t;
    u64 t1 = y[1] + hp1;
    u64 cy1 = t1 < hp1;
    t1 += cy;
    cy1 += t1 < cy;
    y[1] = t1;
    u64 c = cy1;
#pragma unroll
    for (int e = 2; e < E; ++e) {
      y[e] += c;
      c = c && y[e] == 0;
    }
    hp0 = c;  // generate bit
  }
  const u32 g = (u32)hp0;
  u32 pr = 1;
#pragma unroll
  for (int e = 0; e < E; ++e) pr &= (y[e] == ~0ull);
  pr &= !g;

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
    if (tile > 0) {
      flag_store(&flags[tile], kFlagAggregate | (tg << 2) | (tp << 3));
      long long j = (long long)tile - 1;
      for (;;) {
        if (j < 0) {
          cin = 0;
          break;
        }
        u32 f;
        int spins = 0;
        while ((f = flag_load(&flags[j])) == 0) {
          if (++spins > kSpinLimit) break;
          __nanosleep(32);
        }
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
    flag_store(&flags[tile], kFlagInclusive | ((tg | (tp & cin)) << 2));
    s_cin = cin;
  }
  __syncthreads();
  u32 wc = s_cin;
  for (int w = 0; w < warp; ++w) wc = s_wg[w] | (s_wp[w] & wc);
  const u64 sum = (u64)G + GP + wc;
  const u32 cin_bits = (u32)sum ^ G ^ GP;
  u32 c = (cin_bits >> lane) & 1;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    y[e] += c;
    c = c && y[e] == 0;
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

// Adds side[0] + side[1]*B into out[0..L) and wraps the final carry around to
// limb 0 (ntt_info.h:238-242): the result is the product mod B^L - 1.
__global__ void __launch_bounds__(1024) wrap_fix_kernel(u64* out, u64 L, const u64* side) {
  __shared__ int s_carry;
  __shared__ unsigned long long s_first;
  const int tid = threadIdx.x;
  if (tid == 0) {
    const u64 c0 = side[0], c1 = side[1];
    const u64 v0 = out[0] + c0;
    const u64 cy = v0 < c0;
    u64 t = out[1] + c1;
    u64 cy2 = t < c1;
    const u64 v1 = t + cy;
    cy2 += v1 < cy;
    out[0] = v0;
    out[1] = v1;
    s_carry = (int)cy2;
    s_first = ~0ull;
  }
  __syncthreads();
  if (!s_carry) return;
  for (u64 base = 2; base < L; base += blockDim.x) {
    const u64 i = base + tid;
    const bool stop = i < L && out[i] != ~0ull;
    if (stop) atomicMin(&s_first, (unsigned long long)i);
    __syncthreads();
    const u64 first = s_first;
    if (first != ~0ull) {
      if (i < first && i < L) out[i] = 0;
      __syncthreads();
      if (tid == 0) out[first] += 1;
      return;
    }
    if (i < L) out[i] = 0;
    __syncthreads();
  }
  if (tid == 0) {  // carry left limb L-1: end-around into limb 0
    for (u64 i = 0; i < L; ++i)
      if (++out[i] != 0) break;
  }
}

template <class Prod>
cudaError_t run_scan(const Prod& prod, u64 total, u64* out, u64 out_limit, Scan& sc, cudaStream_t st,
                     const char* name) {
  const u64 tiles = scan_tiles(total);
  cudaError_t e = scan_reserve(sc, tiles);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(sc.flags, 0, (tiles + 1) * sizeof(u32), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(sc.counter, 0, sizeof(u32), st);
  if (e != cudaSuccess) return e;
  launch_begin(name, st);
  scan_kernel<Prod><<<(unsigned)tiles, kScanThreads, 0, st>>>(prod, total, out, out_limit, sc.side, sc.flags,
                                                              sc.counter, sc.err);
  launch_end(st);
  return cudaGetLastError();
}

}  // namespace

u64 scan_tiles(u64 positions) { return positions ? (positions + kScanTile - 1) / kScanTile : 1; }

cudaError_t scan_reserve(Scan& sc, u64 tiles) {
  if (sc.flags && sc.max_tiles >= tiles) return cudaSuccess;
  if (sc.flags) cudaFree(sc.flags);
  u64 cap = sc.max_tiles ? sc.max_tiles : 1024;
  while (cap < tiles) cap *= 2;
  cudaError_t e = cudaMalloc((void**)&sc.flags, (cap + 1) * sizeof(u32));
  if (e != cudaSuccess) {
    sc.flags = nullptr;
    sc.max_tiles = 0;
    return e;
  }
  sc.max_tiles = cap;
  if (!sc.counter) {
    e = cudaMalloc((void**)&sc.counter, 4 * sizeof(u32) + 4 * sizeof(u64));
    if (e != cudaSuccess) return e;
    sc.err = sc.counter + 1;
    sc.side = reinterpret_cast<u64*>(sc.counter + 4);
    e = cudaMemset(sc.counter, 0, 4 * sizeof(u32) + 4 * sizeof(u64));
  }
  return e;
}

void scan_free(Scan& sc) {
  if (sc.flags) cudaFree(sc.flags);
  if (sc.counter) cudaFree(sc.counter);
  sc = Scan{};
}

cudaError_t ntt_save(const u64* res, int s, u64* out, u64 size, Scan& sc, u64* written, cudaStream_t st) {
  const u64 L = 1ull << s;
  cudaError_t e = scan_reserve(sc, 1);
  if (e != cudaSuccess) return e;
  if (size - 1 > L) {  // wrap mode
    e = run_scan(CrtProducer{res, L, L}, L + 2, out, L, sc, st, "crt_carry_scan");
    if (e != cudaSuccess) return e;
    launch_begin("wrap_fix", st);
    wrap_fix_kernel<<<1, 1024, 0, st>>>(out, L, sc.side);
    launch_end(st);
    *written = L;
    return cudaGetLastError();
  }
  *written = size;
  return run_scan(CrtProducer{res, L, size - 1}, size, out, size, sc, st, "crt_carry_scan");
}

cudaError_t school_mul(const u64* a, u64 na, const u64* b, u64 nb, u64* out, Scan& sc, cudaStream_t st) {
  cudaError_t e = scan_reserve(sc, 1);
  if (e != cudaSuccess) return e;
  return run_scan(ColumnProducer{a, na, b, nb}, na + nb, out, na + nb, sc, st, "school_column_scan");
}

cudaError_t add_shifted(const u64* x, u64 nx, const u64* y, u64 ny, u64 shift, u64* out, u64 n, Scan& sc,
                        cudaStream_t st) {
  cudaError_t e = scan_reserve(sc, 1);
  if (e != cudaSuccess) return e;
  return run_scan(AddProducer{x, nx, y, ny, shift}, n, out, n, sc, st, "add_scan");
}

}  // namespace nn

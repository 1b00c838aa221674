// carry.cu — multiword carry propagation on sm_103a: CRT recombination fused
// with a carry scan, plus the same scan driving the schoolbook base case and
// shifted multiword adds.
//
// Each position k contributes a three-word value x_k (< 2^186) at limb k; the
// output is sum_k x_k * B^k, B = 2^64 (asmCRT, asmLinux.asm:1369-1450, does
// this serially with a two-word running carry).  Thread t of a tile owns E
// consecutive positions and forms S_t = sum_e x_{k0+e} B^e = lo_t + H_t B^E
// with a zero carry-in (H_t: two words).  Adding the neighbour's H_{t-1} into
// lo_t leaves an E-limb value u_t plus a one-bit generate g_t; the remaining
// carries are one bit each (propagate p_t = u_t is all ones; g_t and p_t are
// exclusive), resolved by warp ballots inside a tile.
//
// Between tiles the per-call scans of more than 1024 tiles take three
// launches and never wait:
//  1. every tile runs with carry-in 0, writes its limbs and records its
//     one-bit generate and propagate (no tile waits for another);
//  2. one CTA composes those bits over the tiles (a scan of the maps
//     carry-in -> carry-out) and records each tile's carry-in;
//  3. each tile whose carry-in is 1 adds it at its first limb, where it
//     ripples only while limbs wrap to zero.
// Smaller per-call scans, the persistent batch kernel and the
// allocation-free entry point take the decoupled lookback instead (scan_tile
// with LOOKBACK: one launch, each tile's carry-in from its predecessors'
// status words), whose waits are bounded and record an error instead of
// hanging.
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>

#include "nn_device.cuh"
#include "nn_internal.h"
#include "scan_tiles.cuh"

namespace nn {

NN_DEFINE_PRIME_UPLOADER(upload_primes_carry)

namespace {

// Scans of at most kLookbackTiles tiles take one launch: tile ids come from
// an atomic counter (from tile_base), so every predecessor of a tile has
// started before it, and each tile takes its carry-in by the decoupled
// lookback.  Their tiles fit in one or two waves, so a lookback waits about
// one tile's work; larger scans take the three steps below, which never wait.
constexpr u64 kLookbackTiles = 1024;
template <class Prod>
__global__ void __launch_bounds__(kScanThreads, 3) scan_lookback_kernel(Prod prod, u64 total, u64* out, u64 out_limit,
                                                                     u64* side, u32* flags, u32* counter, u32* err,
                                                                     u32 tile_base) {
  __shared__ u32 s_tile;
  if (threadIdx.x == 0) s_tile = tile_base + atomicAdd(counter, 1u);
  __syncthreads();
  scan_tile(prod, s_tile, total, out, out_limit, side, flags, err);
}

// Step 1: tile tile_base + blockIdx.x with carry-in 0; flags[tile] receives
// its generate (bit 0) and propagate (bit 1) bits.
template <class Prod>
__global__ void __launch_bounds__(kScanThreads, 3) scan_kernel(Prod prod, u64 total, u64* out, u64 out_limit,
                                                            u64* side, u32* flags, u64 tile_base) {
  scan_tile<Prod, false>(prod, tile_base + blockIdx.x, total, out, out_limit, side, flags, nullptr);
}

// Step 2: the carries between tiles [t0, t1), in chunks of kCarryChunk
// tiles.  The chunk's status words come into shared memory with coalesced
// loads; each thread folds kCarryPer consecutive tiles into the map carry-in
// -> carry-out (the pair of outputs for carry-in 0 and 1); a scan over the
// threads composes the maps; each thread walks its tiles again and sets bit 2
// to the tile's carry-in; the words go back with coalesced stores.  The
// carry into t0 is *chain (left there by the previous range of the same
// scan) or 0 when t0 = 0; the carry out of t1 - 1 is left in *chain.
constexpr int kCarryThreads = 1024, kCarryPer = 32, kCarryChunk = kCarryThreads * kCarryPer;
__global__ void __launch_bounds__(kCarryThreads) tile_carry_kernel(u32* flags, u64 t0, u64 t1, u32* chain) {
  __shared__ unsigned char sb[kCarryChunk];
  __shared__ unsigned char m0[kCarryThreads], m1[kCarryThreads];
  __shared__ u32 s_carry;
  const int j = threadIdx.x;
  if (j == 0) s_carry = t0 > 0 ? *chain : 0u;
  for (u64 c0 = t0; c0 < t1; c0 += kCarryChunk) {
    const u64 n = min((u64)kCarryChunk, t1 - c0);
#pragma unroll 8
    for (int i = 0; i < kCarryPer; ++i) {
      const u64 k = (u64)i * kCarryThreads + j;
      sb[k] = k < n ? (unsigned char)flags[c0 + k] : 2;  // past the range: propagates (the identity map)
    }
    __syncthreads();
    u32 f0 = 0, f1 = 1;
#pragma unroll 8
    for (int i = 0; i < kCarryPer; ++i) {
      const u32 v = sb[j * kCarryPer + i], g = v & 1, p = (v >> 1) & 1;
      f0 = g | (p & f0);
      f1 = g | (p & f1);
    }
    // inclusive scan: thread j ends with the map of the tiles of threads 0..j
    for (int d = 1; d < kCarryThreads; d <<= 1) {
      m0[j] = (unsigned char)f0;
      m1[j] = (unsigned char)f1;
      __syncthreads();
      if (j >= d) {  // the earlier threads' map first, then this one's
        const u32 e0 = m0[j - d], e1 = m1[j - d];
        const u32 h0 = e0 ? f1 : f0, h1 = e1 ? f1 : f0;
        f0 = h0;
        f1 = h1;
      }
      __syncthreads();
    }
    m0[j] = (unsigned char)f0;
    m1[j] = (unsigned char)f1;
    __syncthreads();
    const u32 cin = s_carry;
    u32 c = j == 0 ? cin : (cin ? m1[j - 1] : m0[j - 1]);
#pragma unroll 8
    for (int i = 0; i < kCarryPer; ++i) {
      const u32 v = sb[j * kCarryPer + i];
      sb[j * kCarryPer + i] = (unsigned char)((v & 3) | (c << 2));
      c = (v & 1) | ((v >> 1) & c);
    }
    __syncthreads();  // every thread has read s_carry and written its tiles
    if (j == kCarryThreads - 1) s_carry = c;  // tiles past the range propagate: c is the carry out of c0 + n - 1
#pragma unroll 8
    for (int i = 0; i < kCarryPer; ++i) {
      const u64 k = (u64)i * kCarryThreads + j;
      if (k < n) flags[c0 + k] = sb[k];
    }
    __syncthreads();
  }
  if (j == 0) *chain = s_carry;
}

// Step 3: a tile whose carry-in is 1 adds it at its first limb; it ripples
// while limbs wrap to zero, at most to the tile's end (a tile of all-ones
// limbs passes the carry on through its propagate bit instead).
__global__ void __launch_bounds__(256) carry_fix_kernel(const u32* flags, u64 t0, u64 t1, u64 total, u64* out,
                                                        u64 out_limit, u64* side) {
  const u64 t = t0 + (u64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= t1 || !((flags[t] >> 2) & 1)) return;
  const u64 end = min((t + 1) * kScanTile, total);
  for (u64 k = t * kScanTile; k < end; ++k) {
    u64* q = k < out_limit ? out + k : side + (k - out_limit);
    const u64 v = *q + 1;
    *q = v;
    if (v != 0) break;
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

// out[0..n] = in[0..n) << cl and out[0..n) = in[0..n) >> cl, 1 <= cl <= 63
// (asmShl / asmShr, asm.h:31-33); out does not overlap in.
__global__ void shl_bits_kernel(u64* out, const u64* in, u64 n, unsigned cl) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (u64)gridDim.x * blockDim.x)
    out[i] = (i < n ? in[i] << cl : 0) | (i > 0 ? in[i - 1] >> (64 - cl) : 0);
}
__global__ void shr_bits_kernel(u64* out, const u64* in, u64 n, unsigned cl) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)
    out[i] = (in[i] >> cl) | (i + 1 < n ? in[i + 1] << (64 - cl) : 0);
}

// The lookback's bounded wait on a status word that nothing sets: after
// `limit` polls it gives up and records the error, as a scan tile does.
__global__ void wait_probe_kernel(const u32* flag, u32* err, int limit) {
  if (threadIdx.x == 0 && wait_flag(flag, limit) == 0) atomicExch(err, 1u);
}

// Base-case products of at most kColumnSumPositions positions go in two
// launches: their column sums into the scan's sums, then the carry scan over
// them.  A column sum is split over kSumLanes threads (thread j of a column
// takes every kSumLanes-th term from its own start, so the threads of a
// column read consecutive limbs of a and of b) and the partial three-word
// sums meet in three shuffle steps.  The one-launch scan gives each thread
// eight whole columns, so a product of a few hundred limbs had one CTA of
// threads that each add eight columns in turn (measured: 383 x 383 limbs,
// 137 us); one thread a column took 27 us.
constexpr u64 kColumnSumPositions = 1 << 20;  // at most 24 MiB of sums
constexpr int kSumLanes = 8;
__global__ void __launch_bounds__(256) column_sums_kernel(ColumnProducer prod, u64 total, u64* sums) {
  const u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x;
  const u64 k = t / kSumLanes;
  const u32 j = (u32)(t % kSumLanes);
  W3 r{0, 0, 0};
  if (k < total && k + 1 < prod.na + prod.nb) {
    const u64 lo = k >= prod.nb ? k - prod.nb + 1 : 0;
    const u64 hi = k < prod.na - 1 ? k : prod.na - 1;
    for (u64 i = lo + j; i <= hi; i += kSumLanes) {
      const u64 x = prod.a[i], y = prod.b[k - i];
      r = add_w3(r, W3{x * y, mulhi(x, y), 0});
    }
  }
#pragma unroll
  for (int d = kSumLanes / 2; d >= 1; d >>= 1) {  // every lane of the warp takes part
    const W3 o{__shfl_down_sync(0xffffffffu, r.w0, d, kSumLanes), __shfl_down_sync(0xffffffffu, r.w1, d, kSumLanes),
               __shfl_down_sync(0xffffffffu, r.w2, d, kSumLanes)};
    r = add_w3(r, o);
  }
  if (j == 0 && k < total) {
    sums[k] = r.w0;
    sums[total + k] = r.w1;
    sums[2 * total + k] = r.w2;
  }
}

// One warp a job: lane i adds limb base + i of x and y; the block's carries
// are those of the integer sum G + (G | P) + carry-in over the lanes' generate
// and propagate bits (the same identity as the scan's warp step).  A
// difference adds the complement of y with a carry-in of 1.
__global__ void __launch_bounds__(256) add_batch_kernel(const AddJob* __restrict__ jobs, u64 m) {
  const u64 j = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const u32 lane = threadIdx.x & 31;
  if (j >= m) return;  // whole warps leave together
  const AddJob J = jobs[j];
  const u64 flip = J.sub ? ~0ull : 0;
  u32 carry = J.sub ? 1 : 0;
  // four 32-limb steps' loads issued together, then their carries in order
  constexpr int kSteps = 4;
  for (u64 base = 0; base < J.nout; base += 32 * kSteps) {
    u64 a[kSteps], b[kSteps];
#pragma unroll
    for (int q = 0; q < kSteps; ++q) {
      const u64 k = base + 32 * q + lane;
      a[q] = k < J.nx ? J.x[k] : 0;
      b[q] = (k < J.ny ? J.y[k] : 0) ^ flip;
    }
#pragma unroll
    for (int q = 0; q < kSteps; ++q) {
      if (base + 32 * q >= J.nout) break;  // the same for every lane
      const u64 k = base + 32 * q + lane;
      const u64 sum = a[q] + b[q];
      const u32 G = __ballot_sync(0xffffffffu, sum < a[q]),
                GP = __ballot_sync(0xffffffffu, sum < a[q] || sum == ~0ull);
      const u64 t = (u64)G + GP + carry;
      const u32 cin = (((u32)t ^ G ^ GP) >> lane) & 1;
      if (k < J.nout) J.out[k] = sum + cin;
      carry = (u32)(t >> 32);
    }
  }
}

// Tiles [tile_begin, tile_end) of the scan (all of them by default).  The
// ranges of one scan go in order on one stream (each range's carry-in comes
// from the range before: through the status words of the lookback, or the
// chain word of the three steps).
template <class Prod>
cudaError_t run_scan(const Prod& prod, u64 total, u64* out, u64 out_limit, Scan& sc, cudaStream_t st,
                     const char* name, u64 tile_begin = 0, u64 tile_end = ~0ull) {
  const u64 tiles = scan_tiles(total);
  tile_end = std::min(tile_end, tiles);
  cudaError_t e = scan_reserve(sc, tiles);
  if (e != cudaSuccess || tile_end <= tile_begin) return e;
  const u64 n = tile_end - tile_begin;
  if (tiles <= kLookbackTiles) {
    if (tile_begin == 0) {
      e = cudaMemsetAsync(sc.flags, 0, (tiles + 1) * sizeof(u32), st);
      if (e != cudaSuccess) return e;
    }
    e = cudaMemsetAsync(sc.counter, 0, sizeof(u32), st);
    if (e != cudaSuccess) return e;
    launch_begin(name, st);
    scan_lookback_kernel<Prod><<<(unsigned)n, kScanThreads, 0, st>>>(prod, total, out, out_limit, sc.side, sc.flags,
                                                                      sc.counter, sc.err, (u32)tile_begin);
    launch_end(st);
    return cudaGetLastError();
  }
  launch_begin(name, st);
  scan_kernel<Prod><<<(unsigned)n, kScanThreads, 0, st>>>(prod, total, out, out_limit, sc.side, sc.flags, tile_begin);
  launch_end(st);
  launch_begin("scan_tile_carries", st);
  tile_carry_kernel<<<1, kCarryThreads, 0, st>>>(sc.flags, tile_begin, tile_end, sc.chain);
  launch_end(st);
  launch_begin("scan_carry_fix", st);
  carry_fix_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(sc.flags, tile_begin, tile_end, total, out, out_limit,
                                                                 sc.side);
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
    sc.chain = sc.counter + 2;
    sc.side = reinterpret_cast<u64*>(sc.counter + 4);
    e = cudaMemset(sc.counter, 0, 4 * sizeof(u32) + 4 * sizeof(u64));
  }
  return e;
}

void scan_free(Scan& sc) {
  if (sc.flags) cudaFree(sc.flags);
  if (sc.counter) cudaFree(sc.counter);
  if (sc.sums) cudaFree(sc.sums);
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

cudaError_t ntt_save_chunks(const u64* res, int s, u64* out, u64 size, Scan& sc, cudaStream_t st, int chunks,
                            const std::function<cudaError_t(u64, u64)>& done) {
  const u64 L = 1ull << s;
  if (size - 1 > L || chunks < 1) return cudaErrorInvalidValue;  // normal mode only
  const u64 tiles = scan_tiles(size);
  cudaError_t e = scan_reserve(sc, tiles);
  for (int k = 0; k < chunks && e == cudaSuccess; ++k) {
    const u64 t0 = tiles * k / chunks, t1 = tiles * (k + 1) / chunks;
    if (t1 == t0) continue;
    e = run_scan(CrtProducer{res, L, size - 1}, size, out, size, sc, st, "crt_carry_scan", t0, t1);
    if (e == cudaSuccess) e = done(t0 * kScanTile, std::min(size, t1 * kScanTile));
  }
  return e;
}

cudaError_t add_batch(const AddJob* d_jobs, u64 m, cudaStream_t st) {
  if (m == 0) return cudaSuccess;
  launch_begin("add_batch", st);
  add_batch_kernel<<<(unsigned)((m * 32 + 255) / 256), 256, 0, st>>>(d_jobs, m);
  launch_end(st);
  return cudaGetLastError();
}

cudaError_t school_mul(const u64* a, u64 na, const u64* b, u64 nb, u64* out, Scan& sc, cudaStream_t st) {
  cudaError_t e = scan_reserve(sc, 1);
  if (e != cudaSuccess) return e;
  const u64 total = na + nb;
  if (total > kColumnSumPositions)
    return run_scan(ColumnProducer{a, na, b, nb}, total, out, total, sc, st, "school_column_scan");
  if (sc.sums_cap < total) {  // grow-only, by doubling from 4096 positions (96 KiB)
    u64 cap = std::max<u64>(sc.sums_cap, 4096);
    while (cap < total) cap *= 2;
    if (sc.sums) cudaFree(sc.sums);
    sc.sums = nullptr;
    sc.sums_cap = 0;
    e = cudaMalloc((void**)&sc.sums, 3 * cap * sizeof(u64));
    if (e != cudaSuccess) return e;
    sc.sums_cap = cap;
  }
  launch_begin("school_column_sums", st);
  column_sums_kernel<<<(unsigned)((total * kSumLanes + 255) / 256), 256, 0, st>>>(ColumnProducer{a, na, b, nb}, total,
                                                                                 sc.sums);
  launch_end(st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return run_scan(SumsProducer{sc.sums, total}, total, out, total, sc, st, "school_column_scan");
}

cudaError_t add_shifted(const u64* x, u64 nx, const u64* y, u64 ny, u64 shift, u64* out, u64 n, Scan& sc,
                        cudaStream_t st) {
  cudaError_t e = scan_reserve(sc, 1);
  if (e != cudaSuccess) return e;
  return run_scan(AddProducer{x, nx, y, ny, shift}, n, out, n, sc, st, "add_scan");
}

cudaError_t lin_combine(u64* out, u64 n_out, const u64* x, u64 nx, u64 xs, const u64* y, u64 ny, u64 ys, bool sub,
                        int cin, Scan& sc, cudaStream_t st, const u64* flip) {
  cudaError_t e = scan_reserve(sc, 1);
  if (e != cudaSuccess) return e;
  return run_scan(LinProducer{x, nx, xs, y, ny, ys, n_out, sub ? 1 : 0, cin, flip}, n_out + 1, out, n_out + 1, sc,
                  st, sub ? "sub_scan" : "add_scan");
}

cudaError_t shl_bits(u64* out, const u64* in, u64 n, unsigned cl, cudaStream_t st) {
  if (cl == 0) {
    cudaError_t e = cudaMemcpyAsync(out, in, n * 8, cudaMemcpyDeviceToDevice, st);
    return e == cudaSuccess ? cudaMemsetAsync(out + n, 0, 8, st) : e;
  }
  const unsigned blocks = (unsigned)std::min<u64>((n + 1 + 255) / 256, 152 * 16);
  launch_begin("shift_bits", st);
  shl_bits_kernel<<<blocks, 256, 0, st>>>(out, in, n, cl);
  launch_end(st);
  return cudaGetLastError();
}

cudaError_t shr_bits(u64* out, const u64* in, u64 n, unsigned cl, cudaStream_t st) {
  if (cl == 0) return cudaMemcpyAsync(out, in, n * 8, cudaMemcpyDeviceToDevice, st);
  const unsigned blocks = (unsigned)std::min<u64>((n + 255) / 256, 152 * 16);
  launch_begin("shift_bits", st);
  shr_bits_kernel<<<blocks, 256, 0, st>>>(out, in, n, cl);
  launch_end(st);
  return cudaGetLastError();
}

cudaError_t wait_probe(Scan& sc, int limit, cudaStream_t st) {
  cudaError_t e = scan_reserve(sc, 1);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(sc.flags, 0, sizeof(u32), st);
  if (e != cudaSuccess) return e;
  launch_begin("wait_probe", st);
  wait_probe_kernel<<<1, 32, 0, st>>>(sc.flags, sc.err, limit);
  launch_end(st);
  return cudaGetLastError();
}

}  // namespace nn

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

#include <algorithm>
#include <functional>

#include "nn_device.cuh"
#include "nn_internal.h"
#include "scan_tiles.cuh"

namespace nn {

NN_DEFINE_PRIME_UPLOADER(upload_primes_carry)

namespace {

// Per-call scan: tile ids come from an atomic counter (from tile_base), so
// every predecessor of a tile has started before it, in this launch or in an
// earlier one on the stream.
template <class Prod>
__global__ void __launch_bounds__(kScanThreads, 3) scan_kernel(Prod prod, u64 total, u64* out, u64 out_limit,
                                                            u64* side, u32* flags, u32* counter, u32* err,
                                                            u32 tile_base) {
  __shared__ u32 s_tile;
  if (threadIdx.x == 0) s_tile = tile_base + atomicAdd(counter, 1u);
  __syncthreads();
  scan_tile(prod, s_tile, total, out, out_limit, side, flags, err);
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

// Tiles [tile_begin, tile_end) of the scan (all of them by default); the
// status words are cleared with the first range, so the ranges of one scan
// go in order on one stream.
template <class Prod>
cudaError_t run_scan(const Prod& prod, u64 total, u64* out, u64 out_limit, Scan& sc, cudaStream_t st,
                     const char* name, u64 tile_begin = 0, u64 tile_end = ~0ull) {
  const u64 tiles = scan_tiles(total);
  tile_end = std::min(tile_end, tiles);
  cudaError_t e = scan_reserve(sc, tiles);
  if (e != cudaSuccess) return e;
  if (tile_begin == 0) {
    e = cudaMemsetAsync(sc.flags, 0, (tiles + 1) * sizeof(u32), st);
    if (e != cudaSuccess) return e;
  }
  e = cudaMemsetAsync(sc.counter, 0, sizeof(u32), st);
  if (e != cudaSuccess) return e;
  launch_begin(name, st);
  scan_kernel<Prod><<<(unsigned)(tile_end - tile_begin), kScanThreads, 0, st>>>(
      prod, total, out, out_limit, sc.side, sc.flags, sc.counter, sc.err, (u32)tile_begin);
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

// batch.cu — thousands of products of uneven lengths in one persistent launch.
//
// The host (engine.cpp) turns a batch into a work queue: every product is a
// job with a short pipeline of steps — for an NTT job at scale s: the forward
// passes of both operands (step k = pass k), the pointwise product, the
// inverse passes, the CRT + carry scan; for a short operand (schoolbook job):
// one column-sum scan — and every step is cut into tiles (items).  When the
// transform has two passes or more, the first operand's last forward pass,
// the pointwise product and the first inverse pass are one step (fused
// items), after the second operand's last pass.  An unbalanced product may
// be split: the longer operand (operand 0) in pieces, each with its own
// transform, sharing the shorter operand's; the CRT + carry scan sums the
// pieces' overlapping coefficients.  Items are
// sorted by step, then job, then tile.  A fixed grid of CTAs (all resident)
// pulls items from an atomic head; an item of step k of job j waits until all
// items of step k-1 of job j have completed (a per-(job, step) counter).
// Because every item of step k-1 was dequeued before any item of step k,
// the wait always ends; it is bounded anyway and records an error.  Data that
// other CTAs wrote in the same launch is read around L1 (.cg).
#include <cuda_runtime.h>

#include "nn_device.cuh"
#include "nn_internal.h"
#include "ntt_tiles.cuh"
#include "scan_tiles.cuh"

namespace nn {

NN_DEFINE_PRIME_UPLOADER(upload_primes_batch)

namespace {

constexpr int kWaitLimit = 1 << 24;

__device__ __forceinline__ u32 ld_acquire(const u32* p) {
  u32 v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Wide strided tiles (32, 64 or 128 columns) of a transform's first pass:
// the forward pass that loads limbs, or the last inverse pass, which scales.
template <bool INV>
__device__ __forceinline__ void wide_tile(int C, u64* sm, const u64* in, u64* out, u64 n_in, int s, int l0, int R,
                                          const u64* tab, const Tables& t, int prime, u64 tile) {
  if (C == 32)
    pass_tile<32, !INV, INV, INV, true>(sm, in, out, n_in, s, l0, R, tab, t.cap, prime, tile);
  else if (C == 64)
    pass_tile<64, !INV, INV, INV, true>(sm, in, out, n_in, s, l0, R, tab, t.cap, prime, tile);
  else
    pass_tile<128, !INV, INV, INV, true>(sm, in, out, n_in, s, l0, R, tab, t.cap, prime, tile);
}

// A base-case item: the column sums of one scan tile's positions and of the
// kScanE positions before them (the scan reads those too), all 256 threads
// at once, eight lanes a position, into shared memory as three word arrays
// of kColumnTileWords; the scan then reads them from there.  (With one
// thread computing its scan positions' sums in turn, a product of a few
// hundred limbs kept a few dozen threads of the CTA busy.)
struct SmemSumsProducer {
  static constexpr bool kBulk = true;
  const u64* s;
  u64 first;  // the position at s[0] (mod 2^64: tile 0's is -kScanE)
  u64 total;
  __device__ __forceinline__ W3 operator()(u64 k) const {
    if (k >= total) return W3{0, 0, 0};
    const u64 i = k - first;
    return W3{s[i], s[kColumnTileWords + i], s[2 * kColumnTileWords + i]};
  }
  __device__ __forceinline__ void bulk(u64 k0, W3 (&x)[kScanE]) const {
#pragma unroll
    for (int e = 0; e < kScanE; ++e) x[e] = (*this)(k0 + e);
  }
};

__device__ __forceinline__ void column_tile_sums(u64* sm, const BatchJob& J, u64 tile) {
  constexpr u32 kLanes = 8, kGroups = 256 / kLanes;
  const u64 size = J.na + J.nb;
  const long long first = (long long)(tile * kScanTile) - kScanE;
  const u64 end = min(size, (tile + 1) * kScanTile);
  const u32 npos = (u32)((long long)end - first);  // at most kColumnTileWords
  const u32 g = threadIdx.x / kLanes, j = threadIdx.x % kLanes;
  const u32 rounds = (npos + kGroups - 1) / kGroups;  // the same for every thread
  for (u32 r = 0; r < rounds; ++r) {
    const u32 q = r * kGroups + g;
    const long long p = first + q;
    W3 acc{0, 0, 0};
    if (q < npos && p >= 0 && (u64)p + 1 < size) {
      const u64 k = (u64)p;
      const u64 lo = k >= J.nb ? k - J.nb + 1 : 0;
      const u64 hi = k < J.na - 1 ? k : J.na - 1;
      for (u64 i = lo + j; i <= hi; i += kLanes) {
        const u64 x = J.a[i], y = J.b[k - i];
        acc = add_w3(acc, W3{x * y, mulhi(x, y), 0});
      }
    }
#pragma unroll
    for (u32 d = kLanes / 2; d >= 1; d >>= 1) {  // every lane of the warp takes part
      const W3 o{__shfl_down_sync(0xffffffffu, acc.w0, d, kLanes), __shfl_down_sync(0xffffffffu, acc.w1, d, kLanes),
                 __shfl_down_sync(0xffffffffu, acc.w2, d, kLanes)};
      acc = add_w3(acc, o);
    }
    if (j == 0 && q < npos) {
      sm[q] = acc.w0;
      sm[kColumnTileWords + q] = acc.w1;
      sm[2 * kColumnTileWords + q] = acc.w2;
    }
  }
}

// The transform that tile g of a pass over the first operand's pieces
// belongs to, and the tile's index within it.
struct PieceTile {
  u64 piece, tile;
};
__device__ __forceinline__ PieceTile piece_tile(const BatchJob& J, u64 g, u64 tiles_per_transform) {
  if (J.pieces == 1) return {0, g};
  const u64 i = g / tiles_per_transform;
  return {i, g - i * tiles_per_transform};
}

// One pass item: forward passes of operand 0 (the pieces of the longer
// operand) or 1 (the shorter), inverse passes of operand 0.
template <bool INV, bool SCALE>
__device__ __forceinline__ void run_pass(u64* sm, const BatchJob& J, const BatchItem& it, int operand,
                                         const Tables& t, bool first) {
  const int pk = it.pass;
  const int s = J.s, l0 = J.lambda0[pk], R = J.R[pk], C = J.C[pk], skip = J.skip[pk];
  const u64 L = 1ull << s;
  const u64* tab = INV ? t.iroot : t.root;
  for (u32 k = 0; k < it.ntile; ++k) {
    if (k) __syncthreads();  // the previous tile's write-back has read shared memory
    const u64* in;
    u64* out;
    u64 n_in = 0, tile = (u64)it.tile + k;
    if (operand == 0) {
      const PieceTile pt = piece_tile(J, tile, L / ((u64)C << R));
      tile = pt.tile;
      out = J.res_a + pt.piece * 3 * L;
      in = out;
      if (first) {
        in = J.a + pt.piece * J.piece;
        n_in = min(J.piece, J.na - pt.piece * J.piece);
      }
    } else {
      out = J.res_b;
      in = first ? J.b : out;
      n_in = J.nb;
    }
    if (C == 16) {
      if (first)
        pass_tile<16, true, INV, SCALE, true>(sm, in, out, n_in, s, l0, R, tab, t.cap, it.prime, tile);
      else
        pass_tile<16, false, INV, SCALE, true>(sm, in, out, n_in, s, l0, R, tab, t.cap, it.prime, tile);
    } else if (C == 2) {
      if (first)
        pass_tile<2, true, INV, SCALE, true>(sm, in, out, n_in, s, l0, R, tab, t.cap, it.prime, tile);
      else
        pass_tile<2, false, INV, SCALE, true>(sm, in, out, n_in, s, l0, R, tab, t.cap, it.prime, tile, nullptr,
                                              nullptr, skip);
    } else if constexpr (INV == SCALE) {  // the planner widens pass 0 only
      wide_tile<INV>(C, sm, in, out, n_in, s, l0, R, tab, t, it.prime, tile);
    }
  }
}

// The last forward pass of the first operand's pieces (or of the only
// operand, for a square), the pointwise product with the second operand's
// finished residues and the first inverse pass, tile by tile (the contiguous
// pass only).
__device__ __forceinline__ void run_fused(u64* sm, const BatchJob& J, const BatchItem& it, const Tables& t) {
  const int pk = it.pass;
  const u64 L = 1ull << J.s;
  const u64* other = J.square ? nullptr : J.res_b;
  for (u32 k = 0; k < it.ntile; ++k) {
    if (k) __syncthreads();
    const PieceTile pt = piece_tile(J, (u64)it.tile + k, L / (2ull << J.R[pk]));
    u64* r = J.res_a + pt.piece * 3 * L;
    pass_tile<2, false, false, false, true, true>(sm, r, r, 0, J.s, J.lambda0[pk], J.R[pk], t.root, t.cap, it.prime,
                                                  pt.tile, t.iroot, other, J.skip[pk]);
  }
}

__global__ void __launch_bounds__(256, 3) batch_kernel(const BatchJob* __restrict__ jobs,
                                                    const BatchItem* __restrict__ items, u32 n_items,
                                                    const u32* __restrict__ need, u32* done, u32* head, u32* flags,
                                                    u32* err, Tables t) {
  extern __shared__ u64 sm[];
  __shared__ u32 s_item;
  // Thread 0 claims the next item while the current one runs, so the queue
  // atomic's latency is hidden.  Items are claimed in queue order and depend
  // only on earlier ones, so the earliest unfinished item is always being
  // worked on: a claimed-but-waiting item never blocks its own dependencies.
  u32 next = 0;
  if (threadIdx.x == 0) next = atomicAdd(head, 1u);
  for (;;) {
    if (threadIdx.x == 0) s_item = next;
    __syncthreads();
    const u32 idx = s_item;
    if (idx >= n_items) break;
    if (threadIdx.x == 0) next = atomicAdd(head, 1u);
    const BatchItem it = items[idx];
    const BatchJob& J = jobs[it.job];
    if (threadIdx.x == 0 && it.step > 0) {
      const u32 c = J.ctr_base + it.step - 1;
      const u32 want = need[c];
      int spins = 0;
      while (ld_acquire(&done[c]) < want) {
        if (++spins > kWaitLimit) {
          atomicExch(err, 2u);
          break;
        }
        __nanosleep(64);
      }
      __threadfence();
    }
    __syncthreads();
    const u64 L = 1ull << J.s;
    switch (it.kind) {
      case kItemFwd:
        run_pass<false, false>(sm, J, it, it.operand, t, it.pass == 0);
        break;
      case kItemPointwise: {  // piece i's residues times the other operand's, in place
        const u64 groups = L / 4;
        const u64 chunks = (groups + kBatchPointwiseChunk - 1) / kBatchPointwiseChunk;
        const PieceTile pt = piece_tile(J, it.tile, chunks);
        const u64 g0 = pt.tile * kBatchPointwiseChunk;
        u64* d = J.res_a + pt.piece * 3 * L;
        const u64* b = J.square ? d : J.res_b;
        for (u64 g = g0 + threadIdx.x; g < g0 + kBatchPointwiseChunk && g < groups; g += blockDim.x)
          pointwise_group<true>(d, d, b, L, t.root, t.cap, it.prime, g);
        break;
      }
      case kItemInv:
        if (it.pass == 0)
          run_pass<true, true>(sm, J, it, 0, t, false);
        else
          run_pass<true, false>(sm, J, it, 0, t, false);
        break;
      case kItemFused:
        run_fused(sm, J, it, t);
        break;
      case kItemCrt: {
        const u64 size = J.na + J.nb;
        if (J.pieces == 1) {
          CrtProducerT<true> prod{J.res_a, L, size - 1};
          scan_tile(prod, it.tile, size, J.out, size, nullptr, flags + J.flag_base, err);
        } else {
          PieceCrtProducer prod{J.res_a, L, J.piece, J.pieces, J.nb, size - 1};
          scan_tile(prod, it.tile, size, J.out, size, nullptr, flags + J.flag_base, err);
        }
        break;
      }
      case kItemColumn: {
        const u64 size = J.na + J.nb;
        column_tile_sums(sm, J, it.tile);
        __syncthreads();
        const SmemSumsProducer prod{sm, (u64)it.tile * kScanTile - kScanE, size};
        scan_tile(prod, it.tile, size, J.out, size, nullptr, flags + J.flag_base, err);
        break;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(&done[J.ctr_base + it.step], 1u);
    }
  }
}

}  // namespace

cudaError_t batch_configure(int* blocks_per_sm, size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, batch_kernel, 256, smem);
}

cudaError_t batch_launch(const BatchJob* jobs, const BatchItem* items, u32 n_items, const u32* need, u32* done,
                         u32* head, u32* flags, u32* err, const Tables& t, int grid, size_t smem, cudaStream_t st) {
  // Recorded into a CUDA graph by the caller, which accounts for the launch
  // at each replay.
  batch_kernel<<<grid, 256, smem, st>>>(jobs, items, n_items, need, done, head, flags, err, t);
  return cudaGetLastError();
}

}  // namespace nn

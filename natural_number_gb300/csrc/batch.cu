// batch.cu — thousands of products of uneven lengths in one persistent launch.
//
// The host (engine.cpp) turns a batch into a work queue: every product is a
// job with a short pipeline of steps — for an NTT job at scale s: the forward
// passes of both operands (step k = pass k), the pointwise product, the
// inverse passes, the CRT + carry scan; for a short operand (schoolbook job):
// one column-sum scan — and every step is cut into tiles (items).  When the
// transform has two passes or more, the second operand's last forward pass,
// the pointwise product and the first inverse pass are one step (fused
// items), after the first operand's last pass.  Items are
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

template <bool INV, bool SCALE>
__device__ __forceinline__ void run_pass(u64* sm, const BatchJob& J, const BatchItem& it, const u64* in, u64* out,
                                         u64 n_in, const Tables& t, bool first) {
  const int pk = it.pass;
  const int s = J.s, l0 = J.lambda0[pk], R = J.R[pk], C = J.C[pk], skip = J.skip[pk];
  const u64* tab = INV ? t.iroot : t.root;
  for (u32 k = 0; k < it.ntile; ++k) {
    if (k) __syncthreads();  // the previous tile's write-back has read shared memory
    const u64 tile = (u64)it.tile + k;
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

// The last forward pass of the second operand (or of the only one, for a
// square), the pointwise product with the first operand's finished residues
// and the first inverse pass, tile by tile (the contiguous pass only).
__device__ __forceinline__ void run_fused(u64* sm, const BatchJob& J, const BatchItem& it, u64* r, const u64* other,
                                          const Tables& t) {
  const int pk = it.pass;
  for (u32 k = 0; k < it.ntile; ++k) {
    if (k) __syncthreads();
    pass_tile<2, false, false, false, true, true>(sm, r, r, 0, J.s, J.lambda0[pk], J.R[pk], t.root, t.cap, it.prime,
                                                  (u64)it.tile + k, t.iroot, other, J.skip[pk]);
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
      case kItemFwd: {
        const bool first = it.pass == 0;
        const u64* src = first ? (it.operand ? J.b : J.a) : (it.operand ? J.res_b : J.res_a);
        u64* dst = it.operand ? J.res_b : J.res_a;
        run_pass<false, false>(sm, J, it, src, dst, it.operand ? J.nb : J.na, t, first);
        break;
      }
      case kItemPointwise: {
        const u64 groups = L / 4;
        const u64 g0 = (u64)it.tile * kBatchPointwiseChunk;
        const u64* a = J.res_a;
        const u64* b = J.square ? J.res_a : J.res_b;
        u64* d = J.square ? J.res_a : J.res_b;
        for (u64 g = g0 + threadIdx.x; g < g0 + kBatchPointwiseChunk && g < groups; g += blockDim.x)
          pointwise_group<true>(d, a, b, L, t.root, t.cap, it.prime, g);
        break;
      }
      case kItemInv: {
        u64* r = J.square ? J.res_a : J.res_b;
        if (it.pass == 0)
          run_pass<true, true>(sm, J, it, r, r, 0, t, false);
        else
          run_pass<true, false>(sm, J, it, r, r, 0, t, false);
        break;
      }
      case kItemFused:
        run_fused(sm, J, it, J.square ? J.res_a : J.res_b, J.square ? nullptr : J.res_a, t);
        break;
      case kItemCrt: {
        const u64 size = J.na + J.nb;
        CrtProducerT<true> prod{J.square ? J.res_a : J.res_b, L, size - 1};
        scan_tile(prod, it.tile, size, J.out, size, nullptr, flags + J.flag_base, err);
        break;
      }
      case kItemColumn: {
        const u64 size = J.na + J.nb;
        ColumnProducer prod{J.a, J.na, J.b, J.nb};
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

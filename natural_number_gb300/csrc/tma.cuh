// tma.cuh — the Tensor Memory Accelerator on sm_103a: tile copies between
// global and shared memory issued by one thread and completed on an
// mbarrier, so the rest of the CTA spends no instructions on addresses and
// loads.  Inline PTX: mbarrier.*, cp.async.bulk.tensor.* (tensor boxes,
// described by a CUtensorMap) and cp.async.bulk.* (contiguous runs).
//
// Rules kept by every caller: shared destinations and sources 128-byte
// aligned for tensor boxes and 16-byte aligned for contiguous runs; global
// addresses and sizes of contiguous runs multiples of 16 bytes; the
// innermost box coordinate times the element size a multiple of 16 bytes;
// tensor maps cover this GPU's own memory only (no multicast).  Every wait
// is bounded: a wait that runs out returns false, and the caller records an
// error instead of hanging.
#pragma once

#include <cuda.h>

#include "nn_device.cuh"

namespace nn {

// Polls of an mbarrier phase before a wait gives up; each poll suspends the
// thread for at most kMbarSuspendNs.
constexpr int kMbarWaitLimit = 1 << 20;
constexpr u32 kMbarSuspendNs = 1000;

__device__ __forceinline__ u32 smem_u32(const void* p) { return (u32)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(u64* bar, u32 arrivals) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(arrivals) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// The calling thread arrives and the phase also waits for `bytes` of copies.
__device__ __forceinline__ void mbar_arrive_expect(u64* bar, u32 bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Waits for the phase of parity `parity` to complete, at most `limit` polls.
__device__ __forceinline__ bool mbar_wait(u64* bar, u32 parity, int limit = kMbarWaitLimit) {
  const u32 a = smem_u32(bar);
  for (int i = 0; i < limit; ++i) {
    u32 done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(kMbarSuspendNs)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Generic-proxy writes of this thread to shared memory become visible to the
// copy engine (before a bulk store reads them, or a bulk load overwrites
// what was read).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Box of a 3-D tensor map at element coordinates (x, y, z) -> shared memory.
__device__ __forceinline__ void tma_load_3d(u64* dst, const CUtensorMap* tm, int x, int y, int z, u64* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(tm), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
// Shared memory -> box of a 3-D tensor map at (x, y, z).
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* tm, int x, int y, int z, const u64* src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(tm),
               "r"(x), "r"(y), "r"(z), "r"(smem_u32(src))
               : "memory");
}
// Contiguous run of `bytes` (a multiple of 16) global -> shared.
__device__ __forceinline__ void bulk_load(u64* dst, const u64* src, u32 bytes, u64* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// Contiguous run of `bytes` shared -> global.
__device__ __forceinline__ void bulk_store(u64* dst, const u64* src, u32 bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)), "r"(bytes)
               : "memory");
}
// Closes this thread's bulk stores into a group and waits until their
// shared-memory sources have been read (the CTA may then exit or reuse them).
__device__ __forceinline__ void bulk_store_drain() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

}  // namespace nn

// host_pool.cpp — nn_host_alloc, nn_host_free, nn_host_pool_reserved.
#include <cuda_runtime.h>

#include <algorithm>
#include <bit>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/natural_gb300.h"

namespace {

using u64 = uint64_t;

// Page-locked host memory for limb buffers and transfer staging.
// cudaMallocHost pins pages at about 14 GB/s, far too slow to call per
// buffer, and a pool that only recycles blocks of one size pins afresh for
// every new size: a computation whose buffers double level by level (a
// binary-splitting tree) would pin its whole history.  So blocks come from a
// buddy allocator over page-locked slabs: a request takes a power-of-two
// block (at least 64 KiB) split from a free larger one, and a freed block
// merges with its free buddy, so fresh pinning stays near the peak of live
// bytes.  Slabs hold 64 MiB to 1 GiB; a request above 1 GiB gets its own
// block, recycled by size class.  Without page-locked memory (no device) the
// slabs are ordinary memory.  Intentionally never destroyed: blocks may be
// freed during static destruction.
struct HostPool {
  static constexpr int kMinOrder = 16, kMinSlab = 26, kMaxSlab = 30;
  std::mutex mu;
  std::map<uintptr_t, int> slabs;                           // base -> order
  std::unordered_set<uintptr_t> free_at[kMaxSlab + 1];      // free blocks by order
  std::unordered_map<u64, std::vector<void*>> big_free;     // class bytes -> blocks
  std::unordered_set<void*> big_pinned;
};
HostPool& host_pool() {
  static HostPool* p = new HostPool;
  return *p;
}
u64 host_class(u64 bytes) {
  if (bytes <= 4096) return 4096;
  const u64 half = std::bit_floor(bytes - 1), step = half / 4;  // classes half * {1.25, 1.5, 1.75, 2}
  return half + (bytes - half + step - 1) / step * step;
}
int host_order(u64 bytes) { return std::max<int>(HostPool::kMinOrder, (int)std::bit_width(std::max<u64>(bytes, 2) - 1)); }
void* host_pages(u64 bytes, bool* pinned) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) == cudaSuccess && p) {
    *pinned = true;
    return p;
  }
  cudaGetLastError();
  *pinned = false;
  return std::aligned_alloc(4096, bytes);
}

}  // namespace

extern "C" {


void* nn_host_alloc(uint64_t bytes) {
  HostPool& P = host_pool();
  const int o = host_order(bytes);
  if (o > HostPool::kMaxSlab) {
    bytes = host_class(bytes);
    {
      std::lock_guard<std::mutex> g(P.mu);
      auto it = P.big_free.find(bytes);
      if (it != P.big_free.end() && !it->second.empty()) {
        void* p = it->second.back();
        it->second.pop_back();
        return p;
      }
    }
    bool pinned = false;
    void* p = host_pages(bytes, &pinned);
    if (p && pinned) {
      std::lock_guard<std::mutex> g(P.mu);
      P.big_pinned.insert(p);
    }
    return p;
  }
  std::lock_guard<std::mutex> g(P.mu);
  int k = o;
  while (k <= HostPool::kMaxSlab && P.free_at[k].empty()) ++k;
  if (k > HostPool::kMaxSlab) {  // a new slab, twice the last one (64 MiB .. 1 GiB)
    int so = std::max(o, HostPool::kMinSlab);
    for (const auto& [base, order] : P.slabs) so = std::max(so, std::min(HostPool::kMaxSlab, order + 1));
    bool pinned = false;
    void* base = host_pages(1ull << so, &pinned);
    if (!base) return nullptr;
    P.slabs[(uintptr_t)base] = so;
    P.free_at[so].insert((uintptr_t)base);
    k = so;
  }
  const uintptr_t b = *P.free_at[k].begin();
  P.free_at[k].erase(b);
  while (k > o) {  // split: keep the lower half, free the upper
    --k;
    P.free_at[k].insert(b + (1ull << k));
  }
  return reinterpret_cast<void*>(b);
}

void nn_host_free(void* p, uint64_t bytes) {
  if (!p) return;
  HostPool& P = host_pool();
  int o = host_order(bytes);
  std::lock_guard<std::mutex> g(P.mu);
  if (o > HostPool::kMaxSlab) {
    if (P.big_pinned.count(p))
      P.big_free[host_class(bytes)].push_back(p);
    else
      std::free(p);
    return;
  }
  uintptr_t b = reinterpret_cast<uintptr_t>(p);
  auto slab = P.slabs.upper_bound(b);
  if (slab == P.slabs.begin()) return;  // not from this pool
  --slab;
  const uintptr_t base = slab->first;
  const int top = slab->second;
  if (b >= base + (1ull << top) || o > top) return;  // not from this pool
  while (o < top) {  // merge with the free buddy, order by order
    const uintptr_t buddy = base + ((b - base) ^ (1ull << o));
    auto it = P.free_at[o].find(buddy);
    if (it == P.free_at[o].end()) break;
    P.free_at[o].erase(it);
    b = std::min(b, buddy);
    ++o;
  }
  P.free_at[o].insert(b);
}

uint64_t nn_host_pool_reserved(void) {
  HostPool& P = host_pool();
  std::lock_guard<std::mutex> g(P.mu);
  uint64_t n = 0;
  for (const auto& [base, order] : P.slabs) n += 1ull << order;
  for (const auto& [bytes, blocks] : P.big_free) n += bytes * blocks.size();
  return n;
}

}  // extern "C"

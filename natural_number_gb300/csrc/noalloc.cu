// noalloc.cu — the schoolbook product without any allocation.
//
// Some callers cannot allocate device memory at the point where they need a
// product: code that runs inside another framework whose memory pool owns the
// device memory, or latency-sensitive loops where cudaMalloc/cudaFree would
// synchronise the device and stall every other stream.  nn_mul_base_noalloc
// serves them: it needs no context and allocates nothing.  The only scratch
// it uses — the per-tile status words of the carry scan, a tile counter and an
// error word — lives in the fixed array below, which every GPU that loads the
// library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/natural_gb300.h"
#include "nn_device.cuh"
#include "nn_internal.h"
#include "scan_tiles.cuh"

namespace nn {
namespace {

// Products up to 2^22 limbs (n_a + n_b): 2048 scan tiles.
constexpr u64 kNoAllocMaxLimbs = 1ull << 22;
constexpr u64 kNoAllocTiles = kNoAllocMaxLimbs / kScanTile;
// [0, tiles]: tile status words, [kNoAllocTiles + 1]: tile counter,
// [kNoAllocTiles + 2]: error word (set when a carry wait gives up).
static __device__ __align__(256) u32 g_noalloc_scratch[kNoAllocTiles + 8];

__global__ void __launch_bounds__(kScanThreads) noalloc_school_kernel(ColumnProducer prod, u64 total, u64* out,
                                                                      u32* scratch) {
  __shared__ u32 s_tile;
  u32* counter = scratch + kNoAllocTiles + 1;
  if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  scan_tile(prod, s_tile, total, out, total, nullptr, scratch, scratch + kNoAllocTiles + 2);
}

// Device address of the scratch array, looked up once per device with that
// device current (the symbol's host-side name is not a device address).
u32* scratch_address(int device, cudaError_t* err) {
  static std::mutex mu;
  static u32* addr[64] = {};
  *err = cudaSuccess;
  if (device < 0 || device >= 64) {
    *err = cudaErrorInvalidDevice;
    return nullptr;
  }
  std::lock_guard<std::mutex> g(mu);
  if (!addr[device]) {
    void* p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (*err != cudaSuccess) return nullptr;
    addr[device] = static_cast<u32*>(p);
  }
  return addr[device];
}

}  // namespace
}  // namespace nn

extern "C" nn_status nn_mul_base_noalloc(const uint64_t* d_a, uint64_t n_a, const uint64_t* d_b, uint64_t n_b,
                                         uint64_t* d_out, void* stream) {
  using namespace nn;
  if (!d_a || !d_b || !d_out || n_a == 0 || n_b == 0) return NN_ERR_INVALID;
  if (n_a + n_b > kNoAllocMaxLimbs) return NN_ERR_INVALID;  // beyond the fixed scratch
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) {
    cudaGetLastError();
    return NN_ERR_NO_DEVICE;
  }
  cudaError_t e;
  u32* scratch = scratch_address(device, &e);
  if (!scratch) {
    cudaGetLastError();
    return NN_ERR_CUDA;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const u64 total = n_a + n_b;
  const u64 tiles = scan_tiles(total);
  // The previous call's status words and counter must start from zero.
  e = cudaMemsetAsync(scratch, 0, (tiles + 1) * sizeof(u32), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch + kNoAllocTiles + 1, 0, sizeof(u32), st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return NN_ERR_CUDA;
  }
  noalloc_school_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(ColumnProducer{d_a, n_a, d_b, n_b}, total, d_out,
                                                                  scratch);
  e = cudaGetLastError();
  return e == cudaSuccess ? NN_OK : NN_ERR_CUDA;
}

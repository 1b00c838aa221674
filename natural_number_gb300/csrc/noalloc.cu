// noalloc.cu — the schoolbook product without any allocation.
//
// Some callers cannot allocate device memory at the point where they need a
// product: code that runs inside another framework whose memory pool owns the
// device memory, or latency-sensitive loops where cudaMalloc/cudaFree would
// synchronise the device and stall every other stream.  nn_mul_base_noalloc
// serves them: it needs no context and allocates nothing.  The only scratch
// it uses — the per-tile status words of the carry scan, a tile counter and an
// error word — lives in the fixed array below, which every GPU that loads the
// library holds until the process exits (each device has its own copy).
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
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

// Failure-path test hook: with NN_NOALLOC_SKIP_FIRST_TILE=1 in the
// environment a call starts its tile counter at 1, so no CTA runs tile 0 and
// tile 1's carry wait polls a status word that nothing sets until it gives
// up.  The call then reports NN_ERR_TIMEOUT, as it would for a wait that ran
// out for any other reason.  The last CTA then claims tile `tiles`, one past
// the product: it writes no limb and only its own status word, which lies
// inside the cleared range [0, tiles].
bool skip_first_tile() {
  const char* v = std::getenv("NN_NOALLOC_SKIP_FIRST_TILE");
  return v && std::strcmp(v, "1") == 0;
}

}  // namespace
}  // namespace nn

extern "C" nn_status nn_mul_base_noalloc(const uint64_t* d_a, uint64_t n_a, const uint64_t* d_b, uint64_t n_b,
                                         uint64_t* d_out, void* stream) {
  using namespace nn;
  if (!d_a || !d_b || !d_out || n_a == 0 || n_b == 0) return NN_ERR_INVALID;
  // beyond the fixed scratch (written so that n_a + n_b cannot wrap around)
  if (n_a > kNoAllocMaxLimbs || n_b > kNoAllocMaxLimbs - n_a) return NN_ERR_INVALID;
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
  // The previous call's status words, counter and error word must start from
  // zero (the counter from one under the test hook above).
  const u32 start[2] = {skip_first_tile() ? 1u : 0u, 0u};
  e = cudaMemsetAsync(scratch, 0, (tiles + 1) * sizeof(u32), st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + kNoAllocTiles + 1, start, sizeof start, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return NN_ERR_CUDA;
  }
  noalloc_school_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(ColumnProducer{d_a, n_a, d_b, n_b}, total, d_out,
                                                                  scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return NN_ERR_CUDA;
  // A carry wait that gave up leaves a wrong product behind: read the error
  // word back (into host memory of this frame; nothing is allocated) and
  // wait for the stream, so the status returned covers the product.
  u32 err = 0;
  e = cudaMemcpyAsync(&err, scratch + kNoAllocTiles + 2, sizeof err, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return NN_ERR_CUDA;
  }
  return err ? NN_ERR_TIMEOUT : NN_OK;
}

// ntt.cu — three-prime NTT on sm_103a: twiddle tables, tiled forward/inverse
// passes and the pointwise product.
//
// The transform is the reference's CRT-tree decomposition (ntt_info.h:180-221):
// level lambda (0 <= lambda <= s-2) splits each block of 2^(s-lambda) words into
// halves x, y and applies (x, y) -> (x + w y, x - w y) with w = root[2b] for
// block b.  Level 0 is the load's radix-2 stage (ntt_info.h:153-171, twiddle
// 1); the last level (pairs) is folded into the pointwise product.  The
// residues after each level equal the reference's modulo each prime, whatever
// the grouping of levels; only their lazy representatives differ for p0 and
// p1 (values kept in [0, 4p), see ntt_tiles.cuh).
//
// GPU mapping: levels are grouped into passes.  A pass over levels
// [lambda0, lambda0+R) sees, inside each block of 2^(s-lambda0) words, S = 2^(s-
// lambda0-R) interleaved columns of 2^R rows (row stride S).  A CTA stages
// C columns x 2^R rows of one prime in shared memory with coalesced row
// segments, runs the R levels as radix-8/4/2 register units (twiddles read
// as 16-byte (w, w') pairs: through the read-only cache in the strided
// passes, staged in shared memory with the tile in the contiguous ones), and
// writes the tile back.  The first forward pass reads limbs and reduces them on the fly; the
// last inverse pass applies the 2^-(s-1) scale on the way out.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "nn_device.cuh"
#include "nn_internal.h"
#include "ntt_tiles.cuh"
#include "tma.cuh"

namespace nn {

NN_DEFINE_PRIME_UPLOADER(upload_primes_ntt)

namespace {

typedef unsigned __int128 h128;

const u64 kCoef[3] = {27, 58, 87};
const u64 kGen[3] = {11, 2, 310};  // primitive 2^56-th roots; root_base[i][j] = g^(2^(55-j))

u64 h_mulmod(u64 a, u64 b, u64 p) { return (u64)((h128)a * b % p); }
u64 h_pow(u64 b, u64 e, u64 p) {
  u64 r = 1;
  for (; e; e >>= 1, b = h_mulmod(b, b, p))
    if (e & 1) r = h_mulmod(r, b, p);
  return r;
}
u64 h_comp(u64 w, u64 p) { return (u64)(((h128)w << 64) / p) + 1; }

PrimeSet make_primes() {
  PrimeSet ps{};
  for (int i = 0; i < 3; ++i) {
    u64 p = kCoef[i] << 56 | 1;
    ps.p[i] = p;
    ps.m64[i] = (u64)(~(u64)0 / p) + 1;
    ps.mu[i] = (u64)(((h128)1 << (124 + i)) / p);
    ps.c_hi[i] = (u32)(kCoef[i] << 24);
  }
  const u64 p0 = ps.p[0], p1 = ps.p[1], p2 = ps.p[2];
  ps.inv01 = h_pow(p0 % p1, p1 - 2, p1);
  ps.inv01s = h_comp(ps.inv01, p1);
  ps.inv02 = h_pow(p0 % p2, p2 - 2, p2);
  ps.inv02s = h_comp(ps.inv02, p2);
  ps.inv12 = h_pow(p1 % p2, p2 - 2, p2);
  ps.inv12s = h_comp(ps.inv12, p2);
  h128 p01 = (h128)p0 * p1;
  ps.p01_lo = (u64)p01;
  ps.p01_hi = (u64)(p01 >> 64);
  return ps;
}

// ---------------------------------------------------------------------------
// Twiddle tables
// ---------------------------------------------------------------------------

// Extends one prime's table from n to 2n words: entry n+2k is entry 2k times
// root_base[j] (ntt_info.h:29-31), followed by its Shoup companion.  The
// companion floor(w*2^64/p)+1 uses V = floor((2^128-1)/p): q0 = floor(w*V/2^64)
// is floor(w*2^64/p) or one less, decided by the remainder w*2^64 - q0*p < 2p.
__global__ void twiddle_extend_kernel(u64* tab, u64 n, u64 bw, u64 bwp, int prime, u64 v_hi, u64 v_lo) {
  u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x;
  if (2 * k >= n) return;
  const u64 p = g_primes.p[prime];
  const u32 ch = g_primes.c_hi[prime];
  u64 w = shoup_mul(tab[2 * k], bw, bwp, p, ch);
  u64 q0 = mulhi(w, v_lo) + w * v_hi;
  u64 r = (u64)0 - mul_p(q0, ch);
  if (r >= p) ++q0;
  tab[n + 2 * k] = w;
  tab[n + 2 * k + 1] = q0 + 1;
}

// ---------------------------------------------------------------------------
// Tiled passes
// ---------------------------------------------------------------------------

// FIRST: input is limbs (n_in of them, zero beyond); otherwise residues [3][L].
// SCALE: multiply by 2^-(s-1) on the way out (last inverse pass).
// The first pass numbers its CTAs prime-fastest (x = 3 * tile + prime): the
// three CTAs that reduce the same limbs run together, so the limbs cross HBM
// about once and reach the other two through L2.
template <int C, bool FIRST, bool INV, bool SCALE>
__global__ void __launch_bounds__(256, 4) ntt_pass_kernel(const u64* in, u64* out, u64 n_in, int s, int lambda0, int R,
                                                       const u64* __restrict__ tab, u64 tab_stride) {
  extern __shared__ u64 sm[];
  const int prime = FIRST ? (int)(blockIdx.x % 3) : (int)blockIdx.y;
  const u64 tile = FIRST ? blockIdx.x / 3 : blockIdx.x;
  pass_tile<C, FIRST, INV, SCALE, false>(sm, in, out, n_in, s, lambda0, R, tab, tab_stride, prime, tile);
}

// Contiguous last pass: forward levels, pointwise by `other` (nullptr
// squares), inverse levels, in one visit of each tile.
// Two register budgets: with tiles of up to 2^10 rows (33 KiB of shared
// memory with their twiddles) four CTAs fit an SM if each stays within 64
// registers; larger tiles fit three, which may use 80.
template <int BLOCKS>
__global__ void __launch_bounds__(256, BLOCKS) ntt_fused_kernel(u64* res, const u64* other, int s, int lambda0, int R,
                                                             const u64* __restrict__ tab,
                                                             const u64* __restrict__ itab, u64 tab_stride) {
  extern __shared__ u64 sm[];
  // three CTAs an SM leave 80 registers a thread: room for radix-16 groups
  pass_tile<2, false, false, false, false, true, BLOCKS == 3 ? 4 : 3>(sm, res, res, 0, s, lambda0, R, tab, tab_stride,
                                                                     blockIdx.y, blockIdx.x, itab, other);
}

__global__ void __launch_bounds__(256) pointwise_kernel(u64* dst, const u64* a, const u64* b, u64 L,
                                                        const u64* __restrict__ tab, u64 tab_stride) {
  const u64 g = (u64)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= L / 4) return;
  pointwise_group<false>(dst, a, b, L, tab, tab_stride, blockIdx.y, g);
}

// Strided pass over residues with TMA: one CTA's tile (16 columns x 2^R
// rows of one prime, R <= 9) is one or two boxes of the 3-D view
// [3 * 2^lambda0 super-blocks][2^R rows][2^lg_s columns] of the residues,
// loaded by one thread onto an mbarrier and stored back from shared memory
// by the same engine.  The 16-column rows are 128 bytes, so the unpadded
// tile has no bank conflicts (a warp reads two full rows).  SCALE applies
// the 2^-(s-1) scale: in the last register group where the tile shape has a
// compile-time schedule, else in shared memory before the store.
template <bool INV, bool SCALE, int PR, int MAXK>
__device__ __forceinline__ void col_tile_tma(u64* sm, u64* bar, const CUtensorMap* tm, int s, int lambda0, int R,
                                             const u64* __restrict__ tw, u64 tile, u32* err) {
  constexpr int C = 16;
  constexpr u64 p = PrimeC<PR>::p;
  const int lg_s = s - lambda0 - R;
  const u64 tiles_per_sb = (1ull << lg_s) / C;
  const u64 ksb = tile / tiles_per_sb;
  const int x = (int)((tile % tiles_per_sb) * C);  // a multiple of 16 columns: 128-byte aligned
  const int z = (int)(((u64)PR << lambda0) + ksb);
  const u32 rows = 1u << R, nel = (u32)C << R, box_rows = rows < 256 ? rows : 256;
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_arrive_expect(bar, nel * 8);
    for (u32 y = 0; y < rows; y += box_rows) tma_load_3d(sm + (u64)y * C, tm, x, (int)y, z, bar);
    s_ok = mbar_wait(bar, 0);
  }
  __syncthreads();
  if (!s_ok) {  // the copy never completed: record it, give the copy one more bounded wait, leave the tile
    if (threadIdx.x == 0) {
      if (err) atomicExch(err, 1u);
      mbar_wait(bar, 0);
    }
    return;
  }
  mbar_wait(bar, 0);  // completed phase: this thread sees the copied tile
  bool scaled = false;  // the compile-time schedules scale in their last register group
  if (!INV)
    tile_forward_any<C, PR, true, MAXK, false>(sm, R, ksb, tw, nullptr, 0);
  else
    scaled = tile_inverse_any<C, PR, true, MAXK, false, SCALE>(sm, R, ksb, tw, nullptr, 0, (u32)(s - 1));
  if (SCALE && !scaled) {
    for (u32 idx = 2 * threadIdx.x; idx < nel; idx += 2 * blockDim.x) {
      ulonglong2 v = ld2<false>(sm + idx);
      v.x = div_pow2(canon_c<PR>(v.x), (u32)(s - 1), p);
      v.y = div_pow2(canon_c<PR>(v.y), (u32)(s - 1), p);
      st2<false>(sm + idx, v);
    }
  }
  fence_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    for (u32 y = 0; y < rows; y += box_rows) tma_store_3d(tm, x, (int)y, z, sm + (u64)y * C);
    bulk_store_drain();
  }
}

template <bool INV, bool SCALE, int BLOCKS, int THREADS = 256>
__global__ void __launch_bounds__(THREADS, BLOCKS) ntt_col_tma_kernel(const __grid_constant__ CUtensorMap tm, int s, int lambda0,
                                                          int R, const u64* __restrict__ tab, u64 tab_stride,
                                                          u32* err) {
  extern __shared__ __align__(128) u64 sm[];
  __shared__ __align__(8) u64 bar;
  constexpr int K = BLOCKS == 3 ? 4 : 3;  // three CTAs an SM leave 80 registers: radix-16 groups
  const u64* tw = tab + blockIdx.y * tab_stride;
  if (blockIdx.y == 0)
    col_tile_tma<INV, SCALE, 0, K>(sm, &bar, &tm, s, lambda0, R, tw, blockIdx.x, err);
  else if (blockIdx.y == 1)
    col_tile_tma<INV, SCALE, 1, K>(sm, &bar, &tm, s, lambda0, R, tw, blockIdx.x, err);
  else
    col_tile_tma<INV, SCALE, 2, K>(sm, &bar, &tm, s, lambda0, R, tw, blockIdx.x, err);
}

// The first pass (levels [0, R) from limbs) with a bulk store: the tile (16
// columns x 2^R rows of one prime, dense 128-byte rows) is filled from the
// limbs by the threads, reduced mod p on the way, and goes back to the
// residues as the same tensor-map boxes as a strided pass's tile.  CTAs are
// numbered prime-fastest (x = 3 * tile + prime): the three CTAs that read the
// same limbs run together, so the limbs cross HBM about once.
template <int PR>
__device__ __forceinline__ void load_tile_tma(u64* sm, const CUtensorMap* tm, const u64* in, u64 n_in, int s, int R,
                                              const u64* __restrict__ tw, u64 tile) {
  constexpr int C = 16;
  const int lg_s = s - R;
  const u64 base = tile * C;  // one super-block at level 0: the tile's first column
  const u32 rows = 1u << R, nel = (u32)C << R, box_rows = rows < 256 ? rows : 256;
  const bool half = n_in <= (1ull << (s - 1));
  load_limbs_tile<C, PR, false>(sm, in, n_in, base, lg_s, half ? nel / 2 : nel, half);
  __syncthreads();
  tile_forward_any<C, PR, true, 3, false>(sm, R, 0, tw, nullptr, half ? 1 : 0);
  fence_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    for (u32 y = 0; y < rows; y += box_rows) tma_store_3d(tm, (int)base, (int)y, PR, sm + (u64)y * C);
    bulk_store_drain();
  }
}

template <int BLOCKS, int THREADS>
__global__ void __launch_bounds__(THREADS, BLOCKS) ntt_load_tma_kernel(const __grid_constant__ CUtensorMap tm, const u64* in,
                                                           u64 n_in, int s, int R, const u64* __restrict__ tab,
                                                           u64 tab_stride, u64 tile0) {
  extern __shared__ __align__(128) u64 sm[];
  const int prime = (int)(blockIdx.x % 3);
  const u64 tile = tile0 + blockIdx.x / 3;
  const u64* tw = tab + prime * tab_stride;
  if (prime == 0)
    load_tile_tma<0>(sm, &tm, in, n_in, s, R, tw, tile);
  else if (prime == 1)
    load_tile_tma<1>(sm, &tm, in, n_in, s, R, tw, tile);
  else
    load_tile_tma<2>(sm, &tm, in, n_in, s, R, tw, tile);
}

// All threads learn whether the copies of phase `parity` completed: thread 0
// waits (bounded), the others then observe the completed phase, which makes
// the copied bytes visible to them.  A wait that ran out is recorded in *err;
// thread 0 gives the copies one more bounded wait before the tile is left.
__device__ __forceinline__ bool tile_arrived(u64* bar, u32 parity, u32* err, int* s_ok) {
  if (threadIdx.x == 0) *s_ok = mbar_wait(bar, parity);
  __syncthreads();
  if (!*s_ok) {
    if (threadIdx.x == 0) {
      if (err) atomicExch(err, 1u);
      mbar_wait(bar, parity);
    }
    return false;
  }
  mbar_wait(bar, parity);
  return true;
}

// Groups of 4 residues a thread takes in the fused bulk pass's pointwise
// product (256 threads): 4 for tiles of 2^11 rows (4096 residues, three CTAs
// an SM), 2 for tiles of up to 2^10 rows (four CTAs an SM, 64 registers).
constexpr int kPointwiseGroups = 4;

// Contiguous pass with bulk copies: a tile is 2 columns x 2^R rows of one
// prime, 2^(R+1) consecutive residues, which arrive as 256-byte runs placed
// at the padded layout's 34-word stride (pad16 of word 32c is 34c), while
// the tile's 2^R - 1 twiddle pairs arrive as one run per level (level j:
// 2^j pairs from ksb * 2^j); all complete on one mbarrier.  FUSED (256
// threads, at most 4 * PG * 256 residues): after the forward levels each
// thread keeps the twiddle pairs and the other operand's residues of its PG
// pointwise groups in registers, so the inverse twiddle pairs (the barrier's
// second phase) are copied into the same shared words while the pointwise
// product (by `other`; nullptr squares) runs; then the inverse levels.  The
// tile goes back as 256-byte runs.
template <bool INV, bool FUSED, int PR, int MAXK, int PG = kPointwiseGroups>
__device__ __forceinline__ void row_tile_bulk(u64* sm, u64* bar, u64* res, const u64* other, int s, int R,
                                              const u64* __restrict__ tab, const u64* __restrict__ itab,
                                              u64 tab_stride, u64 tile, u32* err) {
  constexpr int C = 2;
  const u32 nel = (u32)C << R;
  const u64 ksb = tile;  // a contiguous pass has one tile per block of 2^(R+1) words
  u64* g = res + ((u64)PR << s) + (ksb << (R + 1));
  const u32 run = nel < 32 ? nel : 32;
  const u32 nruns = nel / run;
  const u64* tw = tab + (u64)PR * tab_stride;
  u64* tws = sm + tile_words(nel);
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_arrive_expect(bar, nel * 8 + 16u * ((1u << R) - 1));
  }
  __syncthreads();
  for (u32 c = threadIdx.x; c < nruns; c += blockDim.x) bulk_load(sm + 34 * c, g + (u64)run * c, run * 8, bar);
  for (int j = threadIdx.x; j < R; j += blockDim.x)
    bulk_load(tws + 2 * ((1u << j) - 1), tw + 2 * (ksb << j), 16u << j, bar);
  if (!tile_arrived(bar, 0, err, &s_ok)) return;
  if (!INV) {
    tile_forward_any<C, PR, true, MAXK>(sm, R, ksb, tw, tws, 0);
    if (FUSED) {
      const ulonglong2* twsv = reinterpret_cast<const ulonglong2*>(tws);
      const u64* oth = other ? other + ((u64)PR << s) + (ksb << (R + 1)) : nullptr;
      const u32 deep = (1u << (R - 1)) - 1;  // local level R-1: the blocks of 4 residues
      ulonglong2 pw[PG], A01[PG], A23[PG];
#pragma unroll
      for (int k = 0; k < PG; ++k) {
        const u32 g4 = 4 * (threadIdx.x + k * blockDim.x);
        if (g4 < nel) {
          pw[k] = twsv[deep + (g4 >> 2)];
          if (oth) {
            A01[k] = ld2<false>(oth + g4);
            A23[k] = ld2<false>(oth + g4 + 2);
          }
        }
      }
      fence_async_smem();  // the forward pairs have been read before the inverse ones overwrite them
      __syncthreads();
      if (threadIdx.x == 0) mbar_arrive_expect(bar, 16u * ((1u << R) - 1));
      const u64* itw = itab + (u64)PR * tab_stride;
      for (int j = threadIdx.x; j < R; j += blockDim.x)
        bulk_load(tws + 2 * ((1u << j) - 1), itw + 2 * (ksb << j), 16u << j, bar);
#pragma unroll
      for (int k = 0; k < PG; ++k) {
        const u32 g4 = 4 * (threadIdx.x + k * blockDim.x);
        if (g4 < nel) {
          const u64 Bv[4] = {sm[pad16(g4)], sm[pad16(g4 + 1)], sm[pad16(g4 + 2)], sm[pad16(g4 + 3)]};
          const u64 A[4] = {oth ? A01[k].x : Bv[0], oth ? A01[k].y : Bv[1], oth ? A23[k].x : Bv[2],
                            oth ? A23[k].y : Bv[3]};
          u64 o[4];
          pointwise4<PR>(o, A, Bv, pw[k]);
#pragma unroll
          for (int q = 0; q < 4; ++q) sm[pad16(g4 + q)] = o[q];
        }
      }
      if (!tile_arrived(bar, 1, err, &s_ok)) return;  // its barrier also orders the products before the levels
      tile_inverse_any<C, PR, true, MAXK>(sm, R, ksb, itw, tws, 0);
    }
  } else {
    tile_inverse_any<C, PR, true, MAXK>(sm, R, ksb, tw, tws, 0);
  }
  fence_async_smem();
  __syncthreads();
  for (u32 c = threadIdx.x; c < nruns; c += blockDim.x) bulk_store(g + (u64)run * c, sm + 34 * c, run * 8);
  if (threadIdx.x < nruns) bulk_store_drain();
}

template <bool INV, int BLOCKS>
__global__ void __launch_bounds__(256, BLOCKS) ntt_row_bulk_kernel(u64* res, int s, int R, const u64* __restrict__ tab,
                                                                u64 tab_stride, u32* err) {
  extern __shared__ __align__(128) u64 sm[];
  __shared__ __align__(8) u64 bar;
  constexpr int K = BLOCKS == 3 ? 4 : 3;  // three CTAs an SM leave 80 registers: radix-16 groups
  if (blockIdx.y == 0)
    row_tile_bulk<INV, false, 0, K>(sm, &bar, res, nullptr, s, R, tab, nullptr, tab_stride, blockIdx.x, err);
  else if (blockIdx.y == 1)
    row_tile_bulk<INV, false, 1, K>(sm, &bar, res, nullptr, s, R, tab, nullptr, tab_stride, blockIdx.x, err);
  else
    row_tile_bulk<INV, false, 2, K>(sm, &bar, res, nullptr, s, R, tab, nullptr, tab_stride, blockIdx.x, err);
}

// The fused last pass with bulk copies; register budgets as ntt_fused_kernel.
template <int BLOCKS>
__global__ void __launch_bounds__(256, BLOCKS) ntt_fused_bulk_kernel(u64* res, const u64* other, int s, int R,
                                                                  const u64* __restrict__ tab,
                                                                  const u64* __restrict__ itab, u64 tab_stride,
                                                                  u32* err) {
  extern __shared__ __align__(128) u64 sm[];
  __shared__ __align__(8) u64 bar;
  constexpr int K = BLOCKS == 3 ? 4 : 3;
  constexpr int PG = BLOCKS == 3 ? kPointwiseGroups : kPointwiseGroups / 2;
  if (blockIdx.y == 0)
    row_tile_bulk<false, true, 0, K, PG>(sm, &bar, res, other, s, R, tab, itab, tab_stride, blockIdx.x, err);
  else if (blockIdx.y == 1)
    row_tile_bulk<false, true, 1, K, PG>(sm, &bar, res, other, s, R, tab, itab, tab_stride, blockIdx.x, err);
  else
    row_tile_bulk<false, true, 2, K, PG>(sm, &bar, res, other, s, R, tab, itab, tab_stride, blockIdx.x, err);
}

// Bulk copies want 16-byte aligned global runs: the residue arrays of the
// context's buffers always are; an unaligned caller buffer keeps the
// per-thread copies.
inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// cuTensorMapEncodeTiled from the driver, looked up once (nullptr where the
// driver has none: the passes then keep their per-thread copies).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (EncodeTiledFn) nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(f);
  }();
  return fn;
}

// The 3-D view of residues [3][2^s] for a strided pass over levels
// [lambda0, lambda0 + R): 2^lg_s columns (contiguous), 2^R rows 2^lg_s words
// apart, 3 * 2^lambda0 super-blocks of 2^(s - lambda0) words; boxes of 16
// columns x min(2^R, 256) rows.
bool col_tensor_map(CUtensorMap* m, const u64* res, int s, int lambda0, int R) {
  const EncodeTiledFn enc = encode_tiled();
  const int lg_s = s - lambda0 - R;
  if (!enc || lg_s < 4 || R > 9 || (reinterpret_cast<uintptr_t>(res) & 15)) return false;
  const cuuint64_t dims[3] = {1ull << lg_s, 1ull << R, 3ull << lambda0};
  const cuuint64_t strides[2] = {8ull << lg_s, 8ull << (s - lambda0)};
  const cuuint32_t box[3] = {16, (cuuint32_t)std::min(1 << R, 256), 1};
  const cuuint32_t elem[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<u64*>(res), dims, strides, box, elem,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <bool INV, bool SCALE, int BLOCKS, int THREADS = 256>
cudaError_t launch_col_tma_b(const CUtensorMap& tm, int s, const Pass& ps, const Tables& t, cudaStream_t st) {
  const size_t smem = ((size_t)16 << ps.R) * 8;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(ntt_col_tma_kernel<INV, SCALE, BLOCKS, THREADS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const u64 tiles = (1ull << s) / ((u64)16 << ps.R);
  launch_begin(INV ? (SCALE ? "ntt_inv_last_col_pass" : "ntt_inv_col_pass") : "ntt_fwd_col_pass", st);
  ntt_col_tma_kernel<INV, SCALE, BLOCKS, THREADS><<<dim3((unsigned)tiles, 3), THREADS, smem, st>>>(
      tm, s, ps.lambda0, ps.R, INV ? t.iroot : t.root, t.cap, t.err);
  launch_end(st);
  return cudaGetLastError();
}

// Radix-8 groups at 64 registers: radix-16 groups (three CTAs, 80 registers)
// spill in the column passes, whose twiddle pairs stay in registers, and
// measured slower (2^27 multiply 50.4 -> 52.4 ms).  Tiles of up to 2^8 rows
// (32 KiB) run as CTAs of 128 threads, six an SM: a barrier between register
// groups then waits for four warps instead of eight (2^27 column passes 3-4 %
// faster than 256-thread CTAs, four an SM).
template <bool INV, bool SCALE>
cudaError_t launch_col_tma(const CUtensorMap& tm, int s, const Pass& ps, const Tables& t, cudaStream_t st) {
  if (ps.R <= 8) return launch_col_tma_b<INV, SCALE, 8, 128>(tm, s, ps, t, st);
  return launch_col_tma_b<INV, SCALE, 4>(tm, s, ps, t, st);
}

template <bool INV, int BLOCKS>
cudaError_t launch_row_bulk(u64* out, int s, const Pass& ps, const Tables& t, cudaStream_t st) {
  const size_t smem = tile_smem_bytes(2, ps.R);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(ntt_row_bulk_kernel<INV, BLOCKS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const u64 tiles = (1ull << s) / ((u64)2 << ps.R);
  launch_begin(INV ? "ntt_inv_row_pass" : "ntt_fwd_row_pass", st);
  ntt_row_bulk_kernel<INV, BLOCKS><<<dim3((unsigned)tiles, 3), 256, smem, st>>>(out, s, ps.R, INV ? t.iroot : t.root,
                                                                                 t.cap, t.err);
  launch_end(st);
  return cudaGetLastError();
}

// Tiles [tile0, tile1) of the first pass (all of them by default).
template <int BLOCKS, int THREADS>
cudaError_t launch_load_tma(const CUtensorMap& tm, const u64* in, u64 n_in, int s, const Pass& ps, const Tables& t,
                            cudaStream_t st, u64 tile0 = 0, u64 tile1 = ~0ull) {
  const size_t smem = ((size_t)16 << ps.R) * 8;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(ntt_load_tma_kernel<BLOCKS, THREADS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const u64 tiles = std::min<u64>((1ull << s) / ((u64)16 << ps.R), tile1) - tile0;
  launch_begin("ntt_fwd_load_col_pass", st);
  ntt_load_tma_kernel<BLOCKS, THREADS><<<(unsigned)(3 * tiles), THREADS, smem, st>>>(tm, in, n_in, s, ps.R, t.root,
                                                                                     t.cap, tile0);
  launch_end(st);
  return cudaGetLastError();
}

template <int C, bool FIRST, bool INV, bool SCALE>
cudaError_t launch_pass(const u64* in, u64* out, u64 n_in, int s, const Pass& ps, const Tables& t, cudaStream_t st) {
  if constexpr (C == 16 && !FIRST) {
    CUtensorMap tm;
    if (in == out && col_tensor_map(&tm, out, s, ps.lambda0, ps.R)) return launch_col_tma<INV, SCALE>(tm, s, ps, t, st);
  }
  if constexpr (C == 16 && FIRST && !INV) {
    CUtensorMap tm;
    if (ps.lambda0 == 0 && col_tensor_map(&tm, out, s, 0, ps.R)) {
      // 256 threads, four CTAs an SM: as 128-thread CTAs the pass measured
      // slower (2^27 load passes 8.52 -> 9.03 ms), unlike the strided passes
      return launch_load_tma<4, 256>(tm, in, n_in, s, ps, t, st);
    }
  }
  if constexpr (C == 2 && !FIRST && !SCALE) {
    if (in == out && aligned16(out) && ps.lambda0 + ps.R == s - 1) {
      // tiles that leave room for three CTAs an SM only get 80 registers and radix-16 groups
      if (4 * tile_smem_bytes(2, ps.R) > 227 * 1024) return launch_row_bulk<INV, 3>(out, s, ps, t, st);
      return launch_row_bulk<INV, 4>(out, s, ps, t, st);
    }
  }
  const size_t smem = tile_smem_bytes(ps.C, ps.R);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(ntt_pass_kernel<C, FIRST, INV, SCALE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const u64 tiles = (1ull << s) / ((u64)ps.C << ps.R);
  const dim3 grid = FIRST ? dim3((unsigned)(3 * tiles), 1) : dim3((unsigned)tiles, 3);
  const char* name = C == 2 ? (INV ? "ntt_inv_row_pass" : "ntt_fwd_row_pass")
                            : FIRST ? "ntt_fwd_load_col_pass"
                                    : INV ? (SCALE ? "ntt_inv_last_col_pass" : "ntt_inv_col_pass") : "ntt_fwd_col_pass";
  if (C == 2 && FIRST) name = "ntt_fwd_load_row_pass";
  if (C == 2 && SCALE) name = "ntt_inv_last_row_pass";
  launch_begin(name, st);
  ntt_pass_kernel<C, FIRST, INV, SCALE><<<grid, 256, smem, st>>>(in, out, n_in, s, ps.lambda0, ps.R,
                                                                  INV ? t.iroot : t.root, t.cap);
  launch_end(st);
  return cudaGetLastError();
}

template <bool FIRST, bool INV, bool SCALE>
cudaError_t dispatch_pass(const u64* in, u64* out, u64 n_in, int s, const Pass& ps, const Tables& t, cudaStream_t st) {
  if (ps.C == 16) return launch_pass<16, FIRST, INV, SCALE>(in, out, n_in, s, ps, t, st);
  return launch_pass<2, FIRST, INV, SCALE>(in, out, n_in, s, ps, t, st);
}

}  // namespace

void primes_host(u64 p[3]) {
  for (int i = 0; i < 3; ++i) p[i] = kCoef[i] << 56 | 1;
}

cudaError_t upload_primes() {
  PrimeSet ps = make_primes();
  cudaError_t e = upload_primes_ntt(ps);
  if (e == cudaSuccess) e = upload_primes_carry(ps);
  return e == cudaSuccess ? upload_primes_batch(ps) : e;
}

cudaError_t tables_ensure(Tables& t, int s, cudaStream_t st, std::vector<u64*>* retired) {
  if (s < 2) s = 2;
  const u64 need = 1ull << (s - 1);
  if (t.cap >= need) return cudaSuccess;
  u64 *root = nullptr, *iroot = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&root, 3 * need * sizeof(u64), st);
  if (e != cudaSuccess) return e;
  e = cudaMallocAsync((void**)&iroot, 3 * need * sizeof(u64), st);
  if (e != cudaSuccess) {
    cudaFreeAsync(root, st);
    return e;
  }
  u64 have = t.cap;
  for (int i = 0; i < 3; ++i) {
    const u64 p = kCoef[i] << 56 | 1;
    if (have) {
      cudaMemcpyAsync(root + i * need, t.root + i * have, have * sizeof(u64), cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(iroot + i * need, t.iroot + i * have, have * sizeof(u64), cudaMemcpyDeviceToDevice, st);
    } else {
      const u64 init[2] = {1, h_comp(1, p)};  // ntt_info.h:141-143
      cudaMemcpyAsync(root + i * need, init, sizeof init, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(iroot + i * need, init, sizeof init, cudaMemcpyHostToDevice, st);
    }
  }
  const u64 start = have ? have : 2;
  for (int i = 0; i < 3; ++i) {
    const u64 p = kCoef[i] << 56 | 1;
    const h128 V = (~(h128)0) / p;
    const u64 v_hi = (u64)(V >> 64), v_lo = (u64)V;
    const u64 g = kGen[i], gi = h_pow(g, p - 2, p);
    for (u64 n = start; n < need; n <<= 1) {
      int j = 63 - __builtin_clzll(n);  // root_base index for this level
      u64 bw = h_pow(g, 1ull << (55 - j), p), bwi = h_pow(gi, 1ull << (55 - j), p);
      unsigned blocks = (unsigned)((n / 2 + 255) / 256);
      launch_begin("twiddle_extend", st);
      twiddle_extend_kernel<<<blocks, 256, 0, st>>>(root + i * need, n, bw, h_comp(bw, p), i, v_hi, v_lo);
      launch_end(st);
      launch_begin("twiddle_extend", st);
      twiddle_extend_kernel<<<blocks, 256, 0, st>>>(iroot + i * need, n, bwi, h_comp(bwi, p), i, v_hi, v_lo);
      launch_end(st);
    }
  }
  e = cudaGetLastError();
  // The new tables are built on `st`, but kernels on other streams of the
  // same context (a server's concurrent batches, a caller's set_stream) read
  // them from the next launch on: finish building before they are handed out.
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  for (u64* old : {t.root, t.iroot}) {
    if (!old) continue;
    if (retired)
      retired->push_back(old);
    else
      cudaFreeAsync(old, st);
  }
  t.root = root;
  t.iroot = iroot;
  t.cap = need;
  t.scale = s;
  return e;
}

void tables_free(Tables& t) {
  if (t.root) cudaFree(t.root);
  if (t.iroot) cudaFree(t.iroot);
  t = Tables{};
}

std::vector<Pass> plan_passes(int s, int r_last_max, int r_col) {
  // Levels 0..s-2.  The deepest pass works on contiguous blocks (C = 2 columns
  // of stride 2) of up to 2^(r_last_max+1) words; the levels above it go in
  // strided passes of at most r_col levels with 16-column (128-byte) rows.
  std::vector<Pass> out;
  const int total = s - 1;
  r_last_max = std::max(3, std::min(r_last_max, 12));
  r_col = std::max(1, std::min(r_col, 9));
  const int r_last = std::min(total, r_last_max);
  int rest = total - r_last;
  const int n_mid = (rest + r_col - 1) / r_col;
  int l = 0;
  for (int k = 0; k < n_mid; ++k) {
    int r = rest / (n_mid - k);
    out.push_back(Pass{l, r, 16});
    l += r;
    rest -= r;
  }
  out.push_back(Pass{l, r_last, 2});
  return out;
}

cudaError_t ntt_forward(const u64* limbs, u64 n, u64* res, int s, const Tables& t, cudaStream_t st,
                        const std::vector<Pass>* given) {
  std::vector<Pass> plan = given ? *given : plan_passes(s);
  for (size_t k = 0; k < plan.size(); ++k) {
    cudaError_t e = k == 0 ? dispatch_pass<true, false, false>(limbs, res, n, s, plan[k], t, st)
                           : dispatch_pass<false, false, false>(res, res, 0, s, plan[k], t, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t ntt_forward_head(const u64* limbs, u64 n, u64* res, int s, const Tables& t, cudaStream_t st,
                             const std::vector<Pass>& plan) {
  if (plan.size() < 2) return cudaErrorInvalidValue;  // the fused pass would have to load limbs
  for (size_t k = 0; k + 1 < plan.size(); ++k) {
    cudaError_t e = k == 0 ? dispatch_pass<true, false, false>(limbs, res, n, s, plan[k], t, st)
                           : dispatch_pass<false, false, false>(res, res, 0, s, plan[k], t, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

bool ntt_first_pass_tiles(int s, const Pass& ps, u64* tiles) {
  if (ps.C != 16 || ps.lambda0 != 0 || s - ps.R < 4 || ps.R > 9 || !encode_tiled()) return false;
  *tiles = (1ull << s) / ((u64)16 << ps.R);
  return true;
}

cudaError_t ntt_first_pass_range(const u64* limbs, u64 n, u64* res, int s, const Tables& t, const Pass& ps, u64 tile0,
                                 u64 tile1, cudaStream_t st) {
  CUtensorMap tm;
  if (!col_tensor_map(&tm, res, s, 0, ps.R)) return cudaErrorNotSupported;
  return launch_load_tma<4, 256>(tm, limbs, n, s, ps, t, st, tile0, tile1);
}

cudaError_t ntt_forward_tail(u64* res, int s, const Tables& t, cudaStream_t st, const std::vector<Pass>& plan) {
  for (size_t k = 1; k < plan.size(); ++k) {
    cudaError_t e = dispatch_pass<false, false, false>(res, res, 0, s, plan[k], t, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t ntt_fused_last(u64* res, const u64* other, int s, const Tables& t, cudaStream_t st,
                           const std::vector<Pass>& plan) {
  const Pass& ps = plan.back();
  if (ps.C != 2) return cudaErrorInvalidValue;
  const size_t smem = tile_smem_bytes(ps.C, ps.R);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(ntt_fused_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(ntt_fused_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const u64 tiles = (1ull << s) / ((u64)ps.C << ps.R);
  dim3 grid((unsigned)tiles, 3);
  const u64 nel = (u64)2 << ps.R;
  if (aligned16(res) && (!other || aligned16(other)) && ps.lambda0 + ps.R == s - 1 &&
      nel <= (u64)4 * kPointwiseGroups * 256) {
    static bool bulk_configured = false;
    if (!bulk_configured) {
      cudaError_t e = cudaFuncSetAttribute(ntt_fused_bulk_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           200 * 1024);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(ntt_fused_bulk_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      if (e != cudaSuccess) return e;
      bulk_configured = true;
    }
    launch_begin("ntt_fused_row_pass", st);
    if (4 * smem <= 227 * 1024 && nel <= (u64)2 * kPointwiseGroups * 256)
      ntt_fused_bulk_kernel<4><<<grid, 256, smem, st>>>(res, other, s, ps.R, t.root, t.iroot, t.cap, t.err);
    else
      ntt_fused_bulk_kernel<3><<<grid, 256, smem, st>>>(res, other, s, ps.R, t.root, t.iroot, t.cap, t.err);
    launch_end(st);
    return cudaGetLastError();
  }
  launch_begin("ntt_fused_row_pass", st);
  if (4 * smem <= 227 * 1024)
    ntt_fused_kernel<4><<<grid, 256, smem, st>>>(res, other, s, ps.lambda0, ps.R, t.root, t.iroot, t.cap);
  else
    ntt_fused_kernel<3><<<grid, 256, smem, st>>>(res, other, s, ps.lambda0, ps.R, t.root, t.iroot, t.cap);
  launch_end(st);
  return cudaGetLastError();
}

cudaError_t ntt_inverse(u64* res, int s, const Tables& t, cudaStream_t st, const std::vector<Pass>* given,
                        bool skip_last_pass) {
  std::vector<Pass> plan = given ? *given : plan_passes(s);
  for (size_t k = plan.size() - (skip_last_pass ? 1 : 0); k-- > 0;) {
    cudaError_t e = k == 0 ? dispatch_pass<false, true, true>(res, res, 0, s, plan[k], t, st)
                           : dispatch_pass<false, true, false>(res, res, 0, s, plan[k], t, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t ntt_pointwise(u64* dst, const u64* a, const u64* b, int s, const Tables& t, cudaStream_t st) {
  const u64 groups = (1ull << s) / 4;
  dim3 grid((unsigned)((groups + 255) / 256), 3);
  launch_begin("ntt_pointwise", st);
  pointwise_kernel<<<grid, 256, 0, st>>>(dst, a, b, 1ull << s, t.root, t.cap);
  launch_end(st);
  return cudaGetLastError();
}

}  // namespace nn

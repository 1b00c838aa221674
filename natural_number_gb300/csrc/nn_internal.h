// nn_internal.h — device-side building blocks shared by the engine.
// Host C++; no CUDA types leak past this header except cudaStream_t/cudaError_t.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace nn {

typedef std::uint64_t u64;
typedef unsigned int u32;

// Host copy of the prime constants; uploaded to __constant__ memory once per device.
void primes_host(u64 p[3]);
cudaError_t upload_primes();

// Twiddle tables in the reference's layout (ntt_info.h:22-41): per prime,
// words 2k and 2k+1 hold w_k = prod_{bit t of k} root_base[t+1] and its Shoup
// companion floor(w_k * 2^64 / p) + 1.  Grow-only; a table built for scale s
// serves every smaller scale.
struct Tables {
  u64* root = nullptr;   // [3][cap] forward
  u64* iroot = nullptr;  // [3][cap] inverse
  u64 cap = 0;           // words per prime (= 2^(scale-1))
  int scale = 0;
  u32* err = nullptr;    // device error word for kernels whose bounded waits run out (the context's)
};
// Grows the tables to scale s on stream st.  The tables they replace are
// handed to `retired` when given (freed by the caller once no stream can
// still read them: kernels on other streams may hold their pointers), else
// freed in stream order on st.
cudaError_t tables_ensure(Tables& t, int s, cudaStream_t st, std::vector<u64*>* retired = nullptr);
void tables_free(Tables& t);

// One tiled pass over transform levels [lambda0, lambda0 + R) with C columns per tile.
struct Pass {
  int lambda0, R, C;
};
// r_last: levels of the contiguous (deepest) pass; r_col: most levels of a
// strided column pass.
std::vector<Pass> plan_passes(int s, int r_last = 11, int r_col = 9);
// Shared memory of a pass tile (C << R words, padded two words per 32); a
// row pass (C = 2) also stages its 2^R - 1 twiddle pairs.
inline size_t tile_smem_bytes(int C, int R) {
  const size_t n = (size_t)C << R;
  const size_t tile = ((n + n / 16 + 3) & ~(size_t)1) * 8;  // even words: the twiddles start 16-byte aligned
  return C == 2 ? tile + (((size_t)1 << R) - 1) * 16 : tile;
}

// Scratch for the carry scan.
struct Scan {
  u32* flags = nullptr;  // per-tile status words
  u32* counter = nullptr;
  u32* err = nullptr;    // nonzero after a lookback wait gave up
  u32* chain = nullptr;  // carry between consecutive tile ranges of one scan
  u64* side = nullptr;   // limbs of the scan beyond the output (the carry words)
  u64 max_tiles = 0;
  u64* sums = nullptr;   // column sums of base-case products, three words a position
  u64 sums_cap = 0;      // positions they have room for
};
constexpr int kScanThreads = 256;
constexpr int kScanE = 8;  // limbs per thread
constexpr u64 kScanTile = (u64)kScanThreads * kScanE;
// A batched base-case item's column sums in shared memory: a scan tile's
// positions and the kScanE before them, three words each.
constexpr u64 kColumnTileWords = kScanTile + kScanE;
constexpr size_t kColumnTileSmem = 3 * kColumnTileWords * 8;

// Batched products (batch.cu): jobs, their work items, and the launch.  A
// pass item covers consecutive tiles worth at least kBatchItemWords residues
// and a pointwise item kBatchPointwiseChunk groups of 4, so an item's fixed
// cost (queue, dependency check, barriers) stays small beside its work.
constexpr u64 kBatchItemWords = 8192;
constexpr u64 kBatchPointwiseChunk = 4096;
enum : unsigned char { kItemFwd = 0, kItemPointwise = 1, kItemInv = 2, kItemCrt = 3, kItemColumn = 4, kItemFused = 5 };
struct BatchJob {
  const u64* a;  // NTT jobs: the longer operand (split into pieces)
  const u64* b;
  u64* out;      // na + nb limbs
  u64 na, nb;
  u64* res_a;    // [pieces][3][2^s] residues (NTT jobs)
  u64* res_b;    // [3][2^s]
  u64 piece;     // limbs of a per piece (na when not split)
  u64 pieces;
  u32 ctr_base;  // first (job, step) completion counter
  u32 flag_base; // first carry-scan status word
  int s;         // transform scale; 0 for a schoolbook job
  int square;    // a == b: one transform
  int n_pass;
  // Pass k covers levels [lambda0 + skip, lambda0 + R) in tiles of C columns x
  // 2^R rows: the batch widens pass 0's strided tiles (C up to 128) and runs
  // later contiguous passes in tiles of 2^skip consecutive tiles.
  int lambda0[4], R[4], C[4], skip[4];
};
struct BatchItem {
  u32 job;
  unsigned short step;
  unsigned char kind, pass, prime, operand;
  unsigned short ntile;  // consecutive tiles (pass items) handled by this item
  u32 tile;
};
cudaError_t batch_configure(int* blocks_per_sm, size_t smem);
cudaError_t batch_launch(const BatchJob* jobs, const BatchItem* items, u32 n_items, const u32* need, u32* done,
                         u32* head, u32* flags, u32* err, const Tables& t, int grid, size_t smem, cudaStream_t st);

// Many sums at once (carry.cu): job j writes out = x + y in nout >=
// max(nx, ny) + 1 limbs, or with `sub` out = x - y mod B^nout (x >= y: the
// difference), one warp a job walking 32 limbs a step with the carries of a
// step resolved by ballots.  For jobs of up to a few 10^4 limbs; longer sums
// take lin_combine.
struct AddJob {
  const u64* x;
  u64 nx;
  const u64* y;
  u64 ny;
  u64* out;
  u64 nout;
  u64 sub = 0;
};
cudaError_t add_batch(const AddJob* d_jobs, u64 m, cudaStream_t st);

// The first forward pass a range of tiles at a time, so that it can start
// on the columns of an operand already copied: *tiles receives the pass's
// tile count, tile j covering columns [16 j, 16 j + 16) of every row of
// 2^(s - R) limbs (false when the pass does not take this form).  Then
// ntt_forward_tail runs the plan's other passes.
bool ntt_first_pass_tiles(int s, const Pass& ps, u64* tiles);
cudaError_t ntt_first_pass_range(const u64* limbs, u64 n, u64* res, int s, const Tables& t, const Pass& ps, u64 tile0,
                                 u64 tile1, cudaStream_t st);
cudaError_t ntt_forward_tail(u64* res, int s, const Tables& t, cudaStream_t st, const std::vector<Pass>& plan);

// Forward transform: limbs (n <= 2^s) -> residues [3][2^s] equal to
// NTT_info::load + NTT (ntt_info.h:147-198) modulo each prime; lazy values in
// [0, 4p) for p0 and p1, [0, 2p) for p2.
cudaError_t ntt_forward(const u64* limbs, u64 n, u64* res, int s, const Tables& t, cudaStream_t st,
                        const std::vector<Pass>* plan = nullptr);
// Pointwise product of degree-1 residues (ntt_info.h:224-231); dst may alias a or b.
cudaError_t ntt_pointwise(u64* dst, const u64* a, const u64* b, int s, const Tables& t, cudaStream_t st);
// Inverse transform with the final 2^-(s-1) scale (ntt_info.h:200-221); values in [0,p).
cudaError_t ntt_inverse(u64* res, int s, const Tables& t, cudaStream_t st, const std::vector<Pass>* plan = nullptr,
                        bool skip_last_pass = false);
// The forward transform of limbs without its last (contiguous) pass.
cudaError_t ntt_forward_head(const u64* limbs, u64 n, u64* res, int s, const Tables& t, cudaStream_t st,
                             const std::vector<Pass>& plan);
// The last forward pass of `res` fused with the pointwise product by `other`
// (a complete forward transform; nullptr squares) and the first inverse pass.
cudaError_t ntt_fused_last(u64* res, const u64* other, int s, const Tables& t, cudaStream_t st,
                           const std::vector<Pass>& plan);
// CRT + carry into `size` limbs (normal mode) or the wrapped product mod
// B^L - 1 in L limbs when size-1 > L (ntt_info.h:237-248).  Returns the
// number of limbs written through *written (host value).
cudaError_t ntt_save(const u64* res, int s, u64* out, u64 size, Scan& sc, u64* written, cudaStream_t st);
// ntt_save in normal mode, run as `chunks` consecutive ranges of scan tiles;
// after each range is launched, done(limb_begin, limb_end) is called with the
// limbs that range writes (for instance to queue their copy to the host).
cudaError_t ntt_save_chunks(const u64* res, int s, u64* out, u64 size, Scan& sc, cudaStream_t st, int chunks,
                            const std::function<cudaError_t(u64, u64)>& done);
// Schoolbook product by column sums + carry scan: out[0..na+nb).
cudaError_t school_mul(const u64* a, u64 na, const u64* b, u64 nb, u64* out, Scan& sc, cudaStream_t st);
// out[0..n) = x (nx limbs) + y (ny limbs) shifted up by `shift` limbs; the
// carry out of limb n-1 is dropped.  out must not alias x or y (a tile
// re-reads the inputs just below it while its predecessor may be writing).
cudaError_t add_shifted(const u64* x, u64 nx, const u64* y, u64 ny, u64 shift, u64* out, u64 n, Scan& sc,
                        cudaStream_t st);

// out[0..n_out) = x*B^xs + y*B^ys (sub = false) or x*B^xs - y*B^ys - (1 - cin)
// modulo B^n_out (sub = true), and out[n_out] = the carry out of the top limb
// (for a subtraction with cin = 1: 1 exactly when x*B^xs >= y*B^ys).  out
// holds n_out + 1 limbs and does not alias x or y.  A nonzero *flip (device
// memory, when flip is given) swaps add and subtract.
cudaError_t lin_combine(u64* out, u64 n_out, const u64* x, u64 nx, u64 xs, const u64* y, u64 ny, u64 ys, bool sub,
                        int cin, Scan& sc, cudaStream_t st, const u64* flip = nullptr);
// out[0..n] = in << cl (n + 1 limbs) and out[0..n) = in >> cl, 0 <= cl <= 63;
// out does not overlap in.
cudaError_t shl_bits(u64* out, const u64* in, u64 n, unsigned cl, cudaStream_t st);
cudaError_t shr_bits(u64* out, const u64* in, u64 n, unsigned cl, cudaStream_t st);

// Runs the carry lookback's bounded wait on a status word nothing sets (at
// most `limit` polls); it gives up and sets sc.err, which the host reads.
cudaError_t wait_probe(Scan& sc, int limit, cudaStream_t st);

// The decimal split on the device (decimal.cu): out = in >> shift bits for
// many jobs (n_out limbs each, in read as zero past n_in); and the split's
// correction (natural.h:962-965): while lo >= base, hi += 1 and lo -= base,
// one warp a node, with zero[k] = (hi == 0) after it and *err set when a node
// needed more than 8 steps.
constexpr u64 kShrChunk = 4096;
struct ShrJob {
  const u64* in;
  u64 n_in;
  u64* out;
  u64 n_out;
  u64 shift;
};
cudaError_t shr_batch(const ShrJob* d_jobs, const std::vector<ShrJob>& jobs, cudaStream_t st);
struct DecFixJob {
  u64* lo;
  u64 n_lo;
  u64* hi;
  u64 n_hi;
};
cudaError_t dec_fix(const DecFixJob* d_jobs, u64 m, const u64* base, u64 nb, u32* zero, u32* err, cudaStream_t st);
// need[k] = (lo of job k >= base), one warp a job: the test of dec_fix's loop
// alone, for callers that correct long nodes with multiword scans.
cudaError_t dec_need(const DecFixJob* d_jobs, u64 m, const u64* base, u64 nb, u32* need, cudaStream_t st);
// hi += 1 for the jobs with need[k] set, one warp a job.
cudaError_t dec_inc(const DecFixJob* d_jobs, u64 m, const u32* need, cudaStream_t st);

// Decimal digits of n short naturals at once (decimal.cu): node k's len[k]
// limbs at nodes[k] (device pointers; len[k] <= stride, stride even and at
// most 8192); node k < 10^(18 * groups) goes to out[k * 18 * groups ...) as
// 18 * groups zero-padded digits, most significant first.
cudaError_t dec_groups(const u64* const* nodes, u64 stride, const u32* len, u64 n, u32 groups, char* out,
                       cudaStream_t st);

// Launch accounting (profile.cpp): every launch site brackets its kernel.
void launch_begin(const char* name, cudaStream_t st);
void launch_end(cudaStream_t st);
unsigned long long launch_count();
void profile_enable(bool on);
std::string profile_report();

u64 scan_tiles(u64 positions);
cudaError_t scan_reserve(Scan& sc, u64 tiles);
void scan_free(Scan& sc);

}  // namespace nn

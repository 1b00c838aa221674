/* natural_gb300.h — C ABI of the GB300 big-number multiply path.
 *
 * Drop-in boundary for Natural_Number's multiply hot path: the three-prime
 * NTT engine (struct NTT_info, ntt_info.h:10-67), the cached-transform helpers
 * (natural.h:452-527) and the natural-level products, squares and quotients
 * (natural.h:384-793).  Plain pointers and sizes only; limbs are little-endian
 * uint64_t words as in basic_natural (basic_natural.h:9-13).
 *
 * Conventions
 *  - Every call returns nn_status (the reference has no error returns and
 *    exits on allocation failure, basic_natural.h:17-18).
 *  - "d_" pointers are device pointers; device calls are ordered on the
 *    context's stream and return before the GPU finishes.  "_host" calls take
 *    host pointers, copy in, compute and copy out, and return when done.
 *  - Sizes are limb counts.  Products of n_a and n_b limbs occupy n_a + n_b
 *    limbs before normalisation (natural::std, natural.h:82-93).
 *  - A context is used by one host thread at a time.
 */
#ifndef NATURAL_GB300_H
#define NATURAL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  NN_OK = 0,
  NN_ERR_INVALID = 1,   /* argument outside the documented preconditions */
  NN_ERR_OOM = 2,       /* device allocation failed */
  NN_ERR_CUDA = 3,      /* CUDA runtime error; see nn_last_error */
  NN_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up (carry lookback) */
  NN_ERR_BUDGET = 5,    /* request exceeds the context's HBM budget */
  NN_ERR_NO_DEVICE = 6  /* no CUDA device / kernels not loadable */
} nn_status;

typedef struct nn_context nn_context;
typedef struct nn_transform nn_transform;

/* ---- context ------------------------------------------------------------ */
/* Creates a context on `device`.  hbm_budget_bytes = 0 means no budget.
 * The tunables of the tuning file are applied to it (see
 * nn_context_set_tunable): $NN_TUNING if set ("off": none), else the
 * tuning.json the autotuner wrote beside the package. */
nn_status nn_context_create(int device, uint64_t hbm_budget_bytes, nn_context** out);
nn_status nn_context_destroy(nn_context* ctx);
/* Order all work on a caller-owned cudaStream_t (NULL = the legacy default stream). */
nn_status nn_context_set_stream(nn_context* ctx, void* cuda_stream);
/* Go back to the context's own non-blocking stream (the initial state). */
nn_status nn_context_use_own_stream(nn_context* ctx);
void* nn_context_stream(nn_context* ctx);
/* Waits for the stream and reports any deferred device-side error. */
nn_status nn_context_synchronize(nn_context* ctx);
/* Runs the carry lookback's bounded device wait on a status word that nothing
 * sets, giving up after spin_limit polls: returns NN_ERR_TIMEOUT, and the
 * context stays usable.  Checks the timeout path without a fault or a hang
 * (the reference has no device waits). */
nn_status nn_context_probe_wait(nn_context* ctx, int spin_limit);
const char* nn_status_string(nn_status s);
const char* nn_last_error(const nn_context* ctx);
/* Bytes of device memory the context holds (tables, transforms, scratch). */
uint64_t nn_context_device_bytes(const nn_context* ctx);

/* ---- NTT_info: device-resident transforms (ntt_info.h:10-67) ------------- */
nn_status nn_transform_create(nn_context* ctx, nn_transform** out);
nn_status nn_transform_destroy(nn_context* ctx, nn_transform* t);
/* NTT_info::NTT_scale; 0 after a base-case "save" (natural.h:453-456). */
int nn_transform_scale(const nn_transform* t);
void nn_transform_set_scale(nn_transform* t, int scale);
/* NTT_info::load (ntt_info.h:147-173) fused with NTT_info::NTT
 * (ntt_info.h:180-198): residues of n <= 2^scale limbs under the three primes,
 * transformed.  Grows the twiddle tables as NTT_info::init does (ntt_info.h:22-41). */
nn_status nn_transform_forward(nn_context* ctx, nn_transform* t, const uint64_t* d_limbs, uint64_t n, int scale);
/* NTT_info::mul (ntt_info.h:224-231): dst = a (.) b; dst may be a or b. */
nn_status nn_transform_pointwise(nn_context* ctx, nn_transform* dst, const nn_transform* a, const nn_transform* b);
/* NTT_info::INTT (ntt_info.h:200-221) followed by NTT_info::save
 * (ntt_info.h:237-248): writes `size` limbs, or, when size-1 > 2^scale (wrap
 * mode), the product mod B^(2^scale) - 1 in 2^scale limbs.  The transform's
 * residues are consumed.  *written (host) receives the limb count written. */
nn_status nn_transform_inverse_save(nn_context* ctx, nn_transform* t, uint64_t* d_out, uint64_t size,
                                    uint64_t* written);
/* Copies the 3 x 2^scale residues (prime-major) to d_out (inspection/testing):
 * the reference's transform modulo each prime, as lazy representatives in
 * [0, 4p) for p0 and p1 and [0, 2p) for p2. */
nn_status nn_transform_residues(nn_context* ctx, const nn_transform* t, uint64_t* d_out);

/* ---- products on device pointers ---------------------------------------- */
/* natural::_mul (natural.h:444-450): base case below 384 limbs, NTT above,
 * with the unbalanced split of natural.h:391-419.  d_out: n_a + n_b limbs. */
nn_status nn_mul(nn_context* ctx, uint64_t* d_out, const uint64_t* d_a, uint64_t n_a, const uint64_t* d_b,
                 uint64_t n_b);
/* natural::_sqr (natural.h:529-535).  d_out: 2 n limbs. */
nn_status nn_sqr(nn_context* ctx, uint64_t* d_out, const uint64_t* d_a, uint64_t n);
/* The load/NTT/mul/INTT/save pipeline at a caller-chosen scale, as
 * _mul_NTT runs it (natural.h:399-405); size-1 > 2^scale selects wrap mode.
 * n_a, n_b <= 2^scale.  d_out: max(size, 2^scale) limbs; *written as above. */
nn_status nn_ntt_mul(nn_context* ctx, uint64_t* d_out, const uint64_t* d_a, uint64_t n_a, const uint64_t* d_b,
                     uint64_t n_b, int scale, uint64_t size, uint64_t* written);
/* Quotient and remainder with every step on the GPU: an exact Newton division
 * (normalisation, a Newton reciprocal with precision doubling, one quotient
 * estimate and at most a few corrections), not the reference's algorithm.  Quotient
 * and remainder are unique, so they equal natural::_div's (natural.h:749-769).
 * q gets n_a - n_b + 1 limbs and r n_b limbs, not normalised; n_a >= n_b >= 1
 * and the divisor's top limb is nonzero.  nn_div takes device pointers and
 * returns when done; nn_divmod_host takes host pointers. */
nn_status nn_div(nn_context* ctx, uint64_t* d_q, uint64_t* d_r, const uint64_t* d_a, uint64_t n_a,
                 const uint64_t* d_b, uint64_t n_b);
nn_status nn_divmod_host(nn_context* ctx, uint64_t* q, uint64_t* r, const uint64_t* a, uint64_t n_a,
                         const uint64_t* b, uint64_t n_b);
/* Schoolbook product (asmMul1 / mul_base, base.h:56-81) on the GPU: n_a+n_b limbs. */
nn_status nn_mul_base(nn_context* ctx, uint64_t* d_out, const uint64_t* d_a, uint64_t n_a, const uint64_t* d_b,
                      uint64_t n_b);

/* ---- batches: many products in one persistent launch -------------------- */
/* One product of a batch (device pointers; d_out holds n_a + n_b limbs, not
 * normalised).  d_a == d_b with n_a == n_b is a square (one transform). */
typedef struct {
  const uint64_t* d_a;
  uint64_t n_a;
  const uint64_t* d_b;
  uint64_t n_b;
  uint64_t* d_out;
} nn_mul_job;
typedef struct nn_batch nn_batch;
/* Plans a batch for these operand sizes (the reference has no batch API;
 * each job is natural::_mul, natural.h:444-450): jobs whose shorter operand
 * is below the "batch_ntt_min" tunable run as schoolbook column scans, the
 * others (but balanced ones below "batch_school_balanced") as three-prime
 * NTT products at scale ceil(log2(n_a+n_b-1)).  All
 * pipelines go into one work queue drained by one persistent launch; the
 * launch sequence is captured in a CUDA graph on first run and replayed.
 * Products at the "batch_solo_scale" tunable's scale and up run one at a
 * time after that launch, as nn_mul (nn_sqr for squares) would.
 * square[j] (optional) marks squares. */
nn_status nn_batch_create(nn_context* ctx, const uint64_t* n_a, const uint64_t* n_b, const int* square,
                          uint64_t count, nn_batch** out);
/* Runs the planned batch on these operands (sizes must match the plan). */
nn_status nn_batch_run(nn_context* ctx, nn_batch* batch, const nn_mul_job* jobs);
/* As nn_batch_run, but launched directly rather than from the CUDA graph
 * (for plans that run once). */
nn_status nn_batch_launch(nn_context* ctx, nn_batch* batch, const nn_mul_job* jobs);
/* Releases a plan; waits for its last run to finish first. */
nn_status nn_batch_destroy(nn_context* ctx, nn_batch* batch);
uint64_t nn_batch_items(const nn_batch* batch);
/* The same products one nn_mul at a time (one launch sequence per product):
 * the unbatched path, for comparison. */
nn_status nn_mul_each(nn_context* ctx, const nn_mul_job* jobs, uint64_t count);
/* Plan + run + release in one call. */
nn_status nn_batch_mul(nn_context* ctx, const nn_mul_job* jobs, uint64_t count);
/* Tunables: "r_last" (levels of the contiguous NTT pass, 3..12, default 11),
 * "r_col" (most levels of a strided pass, 1..9, default 9), "r_last@<s>" and
 * "r_col@<s>" (the same for transforms of scale s only; 0 = default),
 * "batch_r_last@<s>" (r_last for batched transforms of scale s; 0 = as for
 * one product),
 * "batch_ntt_min" (default 384), "batch_school_balanced" (default 256: a
 * product whose longer operand is at most twice its shorter also takes the
 * schoolbook route while the shorter is below this; 0 = off),
 * "batch_blocks_per_sm" (0 = occupancy limit),
 * "batch_item_words" (residues per prime a batch pass item covers at least,
 * in consecutive tiles; default 8192), "batch_fused" (1, the default: a
 * batched transform of two passes or more runs the second operand's last
 * forward pass, the pointwise product and the first inverse pass as one
 * step; 0: as separate steps), "batch_merge" (1, the default: a batched
 * pass whose tiles hold fewer than 2048 words works on several of them as one
 * tile; 0: tile by tile), "batch_split" (1, the default: an unbalanced
 * product may run as pieces of its longer operand, each through a smaller
 * transform sharing the shorter operand's, when that is estimated faster;
 * 0: one transform per product), "batch_solo_scale" (default 22: a batched
 * product whose transform has this scale or more runs on its own through the
 * one-product passes, after the batch kernel and before the run's completion;
 * 0: every product in the batch kernel; runs that overlap on different
 * streams of one context need 0, since those passes share the context's
 * carry-scan scratch, as nn_mul calls on two streams do). */
nn_status nn_context_set_tunable(nn_context* ctx, const char* name, int64_t value);
int64_t nn_context_get_tunable(const nn_context* ctx, const char* name);

/* ---- allocation-free schoolbook product ---------------------------------- */
/* No counterpart in the reference.  For callers that must not allocate device
 * memory where they multiply: code running under another framework's memory
 * pool, or latency-sensitive loops where cudaMalloc/cudaFree would stall the
 * device.  Same product as nn_mul_base (d_out: n_a + n_b limbs, not
 * normalised), ordered on `stream` (a cudaStream_t; NULL = default stream),
 * without a context and without any allocation: the carry scan's status words
 * live in a fixed device array of the library (2^11 + 8 32-bit words per
 * device), sized for n_a + n_b <= 2^22 limbs (larger products return
 * NN_ERR_INVALID).  The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress) with the device current and keeps it; make
 * that first call before any stream capture, and do not use the entry point
 * after cudaDeviceReset on that device.  The call returns once the product is
 * complete (it reads the scan's error word back and waits for `stream`):
 * NN_ERR_TIMEOUT means a carry wait gave up and d_out is not the product.
 * Every call on a device shares that device's array and clears what it needs,
 * so calls that overlap on the GPU of one device race: order them (each
 * device has its own array).  Test hook: NN_NOALLOC_SKIP_FIRST_TILE=1 in the
 * environment leaves one status word unset, so a carry wait runs out and the
 * call returns NN_ERR_TIMEOUT. */
nn_status nn_mul_base_noalloc(const uint64_t* d_a, uint64_t n_a, const uint64_t* d_b, uint64_t n_b,
                              uint64_t* d_out, void* stream);

/* ---- serving: continuous batching of multiply/divide requests ------------ */
/* No counterpart in the reference (which has no server).  Requests on host
 * memory are admitted in arrival order while their estimated device footprint
 * fits hbm_budget (0: no budget); each scheduler pass launches the newly
 * admitted products as one batch on the next of `streams` streams, so batches
 * of later arrivals overlap earlier ones on the device; divisions
 * (natural::_div, natural.h:749-769) run on `div_workers` threads with their
 * own contexts.  Operands stay on the device from admission to completion.
 * Host buffers must stay valid until the request is waited for. */
typedef struct nn_server nn_server;
typedef struct {
  nn_status status;
  uint64_t out_n;     /* product limbs (normalised) or quotient limbs */
  uint64_t r_n;       /* remainder limbs (division) */
  double t_submit, t_admit, t_done;  /* seconds on the server's clock */
} nn_request_info;
typedef struct {
  uint64_t in_flight_bytes, peak_bytes, waiting, batches, max_concurrent_batches, max_batch_jobs;
} nn_server_stats;
nn_status nn_server_create(int device, uint64_t hbm_budget, int streams, int div_workers, nn_server** out);
/* out: n_a + n_b limbs.  A request larger than the whole budget returns NN_ERR_BUDGET. */
nn_status nn_server_submit_mul(nn_server* s, const uint64_t* a, uint64_t n_a, const uint64_t* b, uint64_t n_b,
                               uint64_t* out, uint64_t* ticket);
/* q: n_a + 1 limbs, r: max(n_a, n_b) + 1 limbs (the reference's result sizes fit). */
nn_status nn_server_submit_div(nn_server* s, const uint64_t* a, uint64_t n_a, const uint64_t* b, uint64_t n_b,
                               uint64_t* q, uint64_t* r, uint64_t* ticket);
/* Waits for a request, fills info and forgets the ticket.  After timeout_s
 * it returns NN_ERR_TIMEOUT instead: the request is still queued or in
 * flight, its host buffers are still in use, and the ticket stays valid. */
nn_status nn_server_wait(nn_server* s, uint64_t ticket, double timeout_s, nn_request_info* info);
nn_status nn_server_get_stats(nn_server* s, nn_server_stats* out);
double nn_server_clock(nn_server* s);
/* Finishes every submitted request, then stops. */
nn_status nn_server_destroy(nn_server* s);

/* ---- launch accounting (process-wide) ------------------------------------ */
/* Number of kernels this library has launched since load. */
uint64_t nn_launch_count(void);
/* Bracket every launch with CUDA events (off by default). */
void nn_profile_enable(int on);
/* Writes "kernel count total_ms" lines for the launches recorded since the
 * last report (synchronises on their events) into buf; returns the length. */
uint64_t nn_profile_report(char* buf, uint64_t cap);

/* ---- host-pointer entry points (copy in, compute, copy out) ------------- */
/* Process-wide context on the current device, created on first use. */
nn_context* nn_default_context(void);
/* nn_transform_forward from host limbs (staged through device scratch). */
nn_status nn_transform_forward_host(nn_context* ctx, nn_transform* t, const uint64_t* limbs, uint64_t n, int scale);
/* nn_transform_inverse_save into host memory (out: max(size, 2^scale) limbs). */
nn_status nn_transform_inverse_save_host(nn_context* ctx, nn_transform* t, uint64_t* out, uint64_t size,
                                         uint64_t* written);
/* Schoolbook product on the GPU from host limbs: out holds n_a + n_b limbs (not normalised). */
nn_status nn_mul_base_host(nn_context* ctx, uint64_t* out, const uint64_t* a, uint64_t n_a, const uint64_t* b,
                           uint64_t n_b);
/* *out_n receives the normalised limb count; out holds n_a + n_b limbs. */
nn_status nn_mul_host(nn_context* ctx, uint64_t* out, uint64_t* out_n, const uint64_t* a, uint64_t n_a,
                      const uint64_t* b, uint64_t n_b);
nn_status nn_sqr_host(nn_context* ctx, uint64_t* out, uint64_t* out_n, const uint64_t* a, uint64_t n);

/* ---- natural-level algorithms on host limbs (products on the GPU) -------- */
/* Results are malloc'd little-endian limbs (release with nn_free); sizes are
 * as the reference's natural holds them (natural::std normalisation where it
 * applies). */
void nn_free(void* p);
/* Page-locked host memory for limb buffers (the drop-in natural's buffers of
 * 64 KiB and more): copies between such buffers and the GPU run at the host
 * link's speed.  Blocks are powers of two (at least 64 KiB) from a buddy
 * allocator over page-locked slabs of 64 MiB to 1 GiB, so freed blocks merge
 * and serve later requests of any size; larger requests get their own block.
 * Without page-locked memory the slabs are ordinary memory.  nn_host_free
 * takes bytes = the size passed to nn_host_alloc.  Thread-safe. */
void* nn_host_alloc(uint64_t bytes);
void nn_host_free(void* p, uint64_t bytes);
/* Host bytes the pool holds (its slabs, and free blocks above 1 GiB). */
uint64_t nn_host_pool_reserved(void);
/* Host limb arithmetic for long operands, run on all host cores with the
 * results of the sequential loops (asmAdd0/asmSub0/asmShl/asmShr, asm.h:7-33):
 * the drop-in natural's O(n) steps between GPU products.  add/sub return the
 * carry/borrow out, and d may be a or b.  shl writes n + 1 limbs and shr n,
 * 1 <= cl <= 63; d may be s, or overlap it the way an in-place shift by whole
 * limbs does (d above s for shl, below for shr), which then runs in sequence.
 * copy is memmove. */
int nn_host_add_n(uint64_t n, uint64_t* d, const uint64_t* a, const uint64_t* b);
int nn_host_sub_n(uint64_t n, uint64_t* d, const uint64_t* a, const uint64_t* b);
void nn_host_shl_n(unsigned cl, uint64_t n, const uint64_t* s, uint64_t* d);
void nn_host_shr_n(unsigned cl, uint64_t n, const uint64_t* s, uint64_t* d);
void nn_host_copy(uint64_t* d, const uint64_t* s, uint64_t n);
/* natural::_div (natural.h:749-769): quotient and remainder. */
nn_status nn_div_host(nn_context* ctx, const uint64_t* a, uint64_t n_a, const uint64_t* b, uint64_t n_b,
                      uint64_t** q, uint64_t* q_n, uint64_t** r, uint64_t* r_n);
/* pow (natural.h:554-564). */
nn_status nn_pow_host(nn_context* ctx, const uint64_t* b, uint64_t n_b, uint64_t e, uint64_t** out, uint64_t* out_n);
/* reciprocal(divs, divd_size) (natural.h:575-617) and the division variant
 * reciprocal(divisor, dividend_size, NTT_info&) (natural.h:619-687); the
 * divisor's top limb must be 1. */
nn_status nn_reciprocal_host(nn_context* ctx, const uint64_t* d, uint64_t n_d, uint64_t divd_size, int variant,
                             uint64_t** out, uint64_t* out_n);
/* Decimal digits of a natural (std::formatter<natural>, natural.h:1089-1091). */
nn_status nn_to_dec_host(nn_context* ctx, const uint64_t* a, uint64_t n_a, char** out, uint64_t* len);
/* The reference's pi and e recipes (calc_pi + sqrt_10005, calc_e; natural.h:841-902,
 * test.cpp:12-32): decimal digit strings. */
nn_status nn_pi_dec_host(nn_context* ctx, uint64_t terms, uint64_t acc, uint64_t digits, char** out, uint64_t* len);
nn_status nn_e_dec_host(nn_context* ctx, uint64_t terms, uint64_t digits, char** out, uint64_t* len);

/* The same recipes with the binary-splitting trees and the decimal split tree
 * evaluated level by level, each level's products as one GPU batch; the
 * series trees' bottom subtrees, whose values stay below about host_below
 * limbs (on a GB300 with 16 host cores: 128 for pi, 256 for e), run whole on
 * host threads.  The decimal split
 * runs its levels while the split powers have at least host_below limbs;
 * the nodes left become digits on the device (one thread a node peels off
 * 18-digit groups, natural.h:566-573 and 994-1011) and come back in one copy.
 * terms must be a power of two (the trees are then perfect).  timing (8
 * doubles, may be NULL): total s, tree s, division s, decimal s, GPU-batch s,
 * host-product s, GPU products, host products. */
nn_status nn_pi_dec_levels(nn_context* ctx, uint64_t terms, uint64_t acc, uint64_t digits, uint64_t host_below,
                           char** out, uint64_t* len, double* timing);
nn_status nn_e_dec_levels(nn_context* ctx, uint64_t terms, uint64_t digits, uint64_t host_below, char** out,
                          uint64_t* len, double* timing);
nn_status nn_to_dec_levels(nn_context* ctx, const uint64_t* a, uint64_t n_a, uint64_t host_below, char** out,
                           uint64_t* len);

#ifdef __cplusplus
}
#endif

#endif /* NATURAL_GB300_H */

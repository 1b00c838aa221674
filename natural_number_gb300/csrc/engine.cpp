// engine.cpp — context, device-resident transforms and the C ABI of
// include/natural_gb300.h.  Host C++ that orders the sm_103a kernels of
// ntt.cu / carry.cu on one CUDA stream; no computation happens on the host
// besides size bookkeeping and the final normalisation of host results.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <bit>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/natural_gb300.h"
#include "nn_internal.h"
#include "stage_ring.h"

using nn::u64;

namespace {
constexpr u64 kNttMulThreshold = 384;  // ntt_info.h:6
constexpr int kMergedTileWords = 2048;  // batch tiles: 256 threads x radix-8 units

int ntt_scale(u64 n1, u64 n2) {  // get_NTT_scale (natural.h:384-386)
  u64 v = n1 + n2 - 2;
  return 64 - std::countl_zero(v);
}

// Page-locked staging ring for the small host tables a call uploads (batch
// plans, job tables, sum tables).  A copy from pageable memory may wait for
// the stream's earlier work before it returns, which would stop the host
// from planning the next batch while the GPU runs this one; from this ring
// the copy is queued and the call returns at once.  Regions are handed out
// in order; one is reused after the event recorded behind its copy (the
// bookkeeping: RegionRing, stage_ring.h).
struct CudaEvents {
  using event = cudaEvent_t;
  std::vector<cudaEvent_t> spare;
  bool done(cudaEvent_t e) { return cudaEventQuery(e) == cudaSuccess; }
  void wait(cudaEvent_t e) { cudaEventSynchronize(e); }
  void recycle(cudaEvent_t e) { spare.push_back(e); }
};

struct Stager {
  char* base = nullptr;
  CudaEvents ev;
  nn::RegionRing<CudaEvents> ring;

  // bytes from host memory at src to device memory at dst, queued on st.
  cudaError_t upload(void* dst, const void* src, u64 bytes, cudaStream_t st) {
    if (!bytes) return cudaSuccess;
    const u64 n = ring.granule(bytes);
    if (n > ring.cap) {  // a larger ring, once every copy from this one is done
      ring.drain(ev);
      if (base) nn_host_free(base, ring.cap);
      ring.cap = std::max<u64>(std::bit_ceil(2 * n), 16ull << 20);
      ring.head = 0;
      base = static_cast<char*>(nn_host_alloc(ring.cap));
      if (!base) {  // no page-locked memory to be had
        ring.cap = 0;
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
      }
    }
    char* h = base + ring.place(n, ev);
    std::memcpy(h, src, bytes);
    cudaError_t e = cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
      ring.drop();
      return e;
    }
    cudaEvent_t done = nullptr;
    if (!ev.spare.empty()) {
      done = ev.spare.back();
      ev.spare.pop_back();
    } else {
      e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventRecord(done, st);
    if (e != cudaSuccess) {  // the copy is queued but no event marks its end: wait for it here
      if (done) ev.spare.push_back(done);
      cudaStreamSynchronize(st);
      ring.drop();
      return e;
    }
    ring.seal(done);
    return cudaSuccess;
  }
  void release() {
    ring.drain(ev);
    for (cudaEvent_t e : ev.spare) cudaEventDestroy(e);
    ev.spare.clear();
    if (base) nn_host_free(base, ring.cap);
    base = nullptr;
    ring.cap = ring.head = 0;
  }
};
}  // namespace

struct nn_context {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  // host-pointer calls: the second operand's copy runs on `copy` while the
  // first operand is transformed
  cudaStream_t copy = nullptr;
  cudaEvent_t ev_first = nullptr, ev_second = nullptr, ev_chunk = nullptr, ev_in = nullptr;
  u64 budget = 0;
  u64 held = 0;  // bytes of live allocations made through the context
  nn::Tables tables;
  nn::Scan scan;
  std::string err;
  u64* scratch[3] = {nullptr, nullptr, nullptr};  // grow-only device staging for host calls
  u64 scratch_words[3] = {0, 0, 0};
  Stager stage;  // page-locked ring for uploaded tables
  // Twiddle tables replaced by larger ones: kept until the context goes, as
  // work on another stream (set_stream, or a server's concurrent batches)
  // may still read them; together at most the size of the live tables.
  std::vector<u64*> retired_tables;
  // tunables (nn_context_set_tunable)
  int r_last = 11;            // levels of the contiguous NTT pass
  int r_col = 9;              // most levels of a strided column pass
  int r_last_at[64] = {};     // per-scale overrides (0: use r_last / r_col)
  int r_col_at[64] = {};
  int batch_r_last_at[64] = {};  // per-scale overrides for batched transforms (0: as above)
  std::vector<nn::Pass> passes(int s) const {
    const int rl = (s >= 0 && s < 64 && r_last_at[s]) ? r_last_at[s] : r_last;
    const int rc = (s >= 0 && s < 64 && r_col_at[s]) ? r_col_at[s] : r_col;
    return nn::plan_passes(s, rl, rc);
  }
  // Batched transforms merge small tiles, which favours other splits at the
  // scales where products are usually batched.
  std::vector<nn::Pass> batch_passes(int s) const {
    if (s < 0 || s >= 64 || !batch_r_last_at[s]) return passes(s);
    return nn::plan_passes(s, batch_r_last_at[s], r_col_at[s] ? r_col_at[s] : r_col);
  }
  u64 batch_ntt_min = 384;    // batches: schoolbook when min(n_a, n_b) is below this
  u64 batch_school_balanced = 256;  // ... or below this when max(n_a, n_b) <= 2 min(n_a, n_b) (0: off)
  u64 batch_item_words = nn::kBatchItemWords;  // residues a pass item covers at least
  int batch_fused = 1;        // batches: fused last pass (forward + pointwise + inverse)
  int batch_merge = 1;        // batches: small tiles worked on 2048 words at a time
  int batch_split = 1;        // batches: unbalanced products in pieces sharing one transform
  int batch_blocks_per_sm = 0;  // persistent CTAs per SM (0: occupancy limit)
  int batch_solo_scale = 22;    // batches: products of this scale and up run one at a time (0: never)
};

struct nn_batch {
  u64 count = 0;
  std::vector<u64> na, nb;
  std::vector<nn::BatchJob> jobs;
  std::vector<nn::BatchItem> items;
  std::vector<nn::u32> need;
  std::vector<u64> off_a, off_b;
  std::vector<char> swap;  // NTT job whose second operand is the longer one
  std::vector<u64> solo;   // jobs run one at a time after the batch kernel
  u64 arena_words = 0;
  nn::u32 n_ctrs = 0, n_flags = 0;
  size_t smem = 0;
  int grid = 0;
  nn::BatchJob* d_jobs = nullptr;
  nn::BatchItem* d_items = nullptr;
  nn::u32* d_need = nullptr;
  nn::u32* d_state = nullptr;  // done[n_ctrs], head, pad
  nn::u32* d_flags = nullptr;
  u64* d_arena = nullptr;
  u64 dev_words = 0;           // budget accounting of the above
  nn::BatchJob* h_jobs = nullptr;  // pinned staging of the job table
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ran = nullptr;
  bool pending = false;
};

struct nn_transform {
  u64* res = nullptr;  // [3][2^scale]
  u64 words = 0;       // allocated words (3 * 2^scale at most)
  int scale = 0;
};

namespace {

nn_status fail(nn_context* c, cudaError_t e, const char* what) {
  c->err = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();  // clear sticky-free errors
  return e == cudaErrorMemoryAllocation ? NN_ERR_OOM : NN_ERR_CUDA;
}

#define NN_CK(ctx, expr, what)                           \
  do {                                                   \
    cudaError_t _e = (expr);                             \
    if (_e != cudaSuccess) return fail((ctx), _e, what); \
  } while (0)

nn_status dev_alloc(nn_context* c, u64** p, u64 words) {
  const u64 bytes = std::max<u64>(words, 1) * sizeof(u64);
  if (c->budget && c->held + bytes > c->budget) {
    c->err = "HBM budget exceeded";
    return NN_ERR_BUDGET;
  }
  cudaError_t e = cudaMallocAsync((void**)p, bytes, c->stream);
  if (e != cudaSuccess) return fail(c, e, "cudaMallocAsync");
  c->held += bytes;
  return NN_OK;
}

void dev_free(nn_context* c, u64* p, u64 words) {
  if (!p) return;
  cudaFreeAsync(p, c->stream);
  c->held -= std::max<u64>(words, 1) * sizeof(u64);
}

// RAII device buffer tied to the context's stream.
struct DBuf {
  nn_context* c;
  u64* p = nullptr;
  u64 words = 0;
  explicit DBuf(nn_context* ctx) : c(ctx) {}
  nn_status alloc(u64 w) {
    words = w;
    return dev_alloc(c, &p, w);
  }
  ~DBuf() { dev_free(c, p, words); }
};

nn_status xform_reserve(nn_context* c, nn_transform* t, int s) {
  const u64 need = 3ull << s;
  if (t->words < need) {
    dev_free(c, t->res, t->words);
    t->res = nullptr;
    t->words = 0;
    nn_status st = dev_alloc(c, &t->res, need);
    if (st != NN_OK) return st;
    t->words = need;
  }
  t->scale = s;
  return NN_OK;
}

nn_status forward(nn_context* c, nn_transform* t, const u64* d_limbs, u64 n, int s) {
  if (s < 2 || s > 40 || n == 0 || n > (1ull << s)) {
    c->err = "forward: need 2 <= scale <= 40 and 1 <= n <= 2^scale";
    return NN_ERR_INVALID;
  }
  NN_CK(c, nn::tables_ensure(c->tables, s, c->stream, &c->retired_tables), "twiddle tables");
  nn_status st = xform_reserve(c, t, s);
  if (st != NN_OK) return st;
  const std::vector<nn::Pass> plan = c->passes(s);
  NN_CK(c, nn::ntt_forward(d_limbs, n, t->res, s, c->tables, c->stream, &plan), "forward NTT");
  return NN_OK;
}

nn_status inverse_save(nn_context* c, nn_transform* t, u64* d_out, u64 size, u64* written,
                       bool skip_last_pass = false) {
  if (size < 2) {
    c->err = "save: size must be at least 2";
    return NN_ERR_INVALID;
  }
  const std::vector<nn::Pass> plan = c->passes(t->scale);
  NN_CK(c, nn::ntt_inverse(t->res, t->scale, c->tables, c->stream, &plan, skip_last_pass), "inverse NTT");
  u64 w = 0;
  NN_CK(c, nn::ntt_save(t->res, t->scale, d_out, size, c->scan, &w, c->stream), "CRT/carry");
  if (written) *written = w;
  return NN_OK;
}

// inverse_save(skip_last_pass) in normal mode, with the product's limbs
// copied to h_out on the copy stream range by range as the carry scan
// finishes them, so the copy-back overlaps the scan.
constexpr int kCopyChunks = 8;
nn_status inverse_save_to_host(nn_context* c, nn_transform* t, u64* d_out, u64 size, u64* h_out) {
  const std::vector<nn::Pass> plan = c->passes(t->scale);
  NN_CK(c, nn::ntt_inverse(t->res, t->scale, c->tables, c->stream, &plan, true), "inverse NTT");
  const cudaError_t e =
      nn::ntt_save_chunks(t->res, t->scale, d_out, size, c->scan, c->stream, kCopyChunks, [&](u64 lo, u64 hi) {
        cudaError_t r = cudaEventRecord(c->ev_chunk, c->stream);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(c->copy, c->ev_chunk, 0);
        if (r == cudaSuccess)
          r = cudaMemcpyAsync(h_out + lo, d_out + lo, (hi - lo) * 8, cudaMemcpyDeviceToHost, c->copy);
        return r;
      });
  NN_CK(c, e, "CRT/carry with copy-back");
  return NN_OK;
}

nn_status pointwise(nn_context* c, nn_transform* dst, const nn_transform* a, const nn_transform* b) {
  if (a->scale != b->scale || a->scale < 2) {
    c->err = "pointwise: transforms differ in scale";
    return NN_ERR_INVALID;
  }
  nn_status st = xform_reserve(c, dst, a->scale);
  if (st != NN_OK) return st;
  NN_CK(c, nn::ntt_pointwise(dst->res, a->res, b->res, a->scale, c->tables, c->stream), "pointwise");
  return NN_OK;
}

// The second operand's transform up to its last pass, then that pass fused
// with the pointwise product by `other` (nullptr: square) and the first
// inverse pass; the caller finishes with inverse_save(skip_last_pass).
nn_status forward_fused(nn_context* c, nn_transform* t, const u64* d_limbs, u64 n, int s, const nn_transform* other) {
  NN_CK(c, nn::tables_ensure(c->tables, s, c->stream, &c->retired_tables), "twiddle tables");
  nn_status st = xform_reserve(c, t, s);
  if (st != NN_OK) return st;
  const std::vector<nn::Pass> plan = c->passes(s);
  NN_CK(c, nn::ntt_forward_head(d_limbs, n, t->res, s, c->tables, c->stream, plan), "forward NTT");
  NN_CK(c, nn::ntt_fused_last(t->res, other ? other->res : nullptr, s, c->tables, c->stream, plan),
        "fused pass");
  return NN_OK;
}

// Balanced NTT product at scale s into d_out (size limbs, or wrap).
// b_ready (optional): an event b's contents wait for; the stream waits for it
// only after a's forward transform.  h_out (optional): host memory the
// product is also copied to, overlapping the carry scan; *h_done tells
// whether that happened (fused pipelines only).
nn_status ntt_product(nn_context* c, u64* d_out, const u64* a, u64 na, const u64* b, u64 nb, int s, u64 size,
                      u64* written, cudaEvent_t b_ready = nullptr, u64* h_out = nullptr, bool* h_done = nullptr) {
  nn_transform xa, xb;
  nn_status st = forward(c, &xa, a, na, s);
  if (st == NN_OK && b_ready) {
    const cudaError_t e = cudaStreamWaitEvent(c->stream, b_ready, 0);
    if (e != cudaSuccess) st = fail(c, e, "wait for the second operand");
  }
  if (st == NN_OK && c->passes(s).size() >= 2) {
    st = forward_fused(c, &xb, b, nb, s, &xa);
    if (st == NN_OK && h_out && size - 1 <= (1ull << s)) {
      st = inverse_save_to_host(c, &xb, d_out, size, h_out);
      if (st == NN_OK && h_done) *h_done = true;
    } else if (st == NN_OK) {
      st = inverse_save(c, &xb, d_out, size, written, true);
    }
  } else {
    if (st == NN_OK) st = forward(c, &xb, b, nb, s);
    if (st == NN_OK) st = pointwise(c, &xb, &xa, &xb);
    if (st == NN_OK) st = inverse_save(c, &xb, d_out, size, written);
  }
  dev_free(c, xa.res, xa.words);
  dev_free(c, xb.res, xb.words);
  return st;
}

// Balanced NTT product of host operands (ha: na limbs, hb: nb limbs, na >=
// nb) into d_out and h_out.  a's copy to da goes a range of columns at a time
// (kInChunks ranges: a 2-D copy of the range in every full row of the first
// pass, plus its part of a last, partial row) on the copy stream, and the
// first forward pass runs each range's tiles as soon as it has arrived, so
// the copy overlaps that pass; b's copy follows on the same stream while a's
// other passes run.  *used is false, and nothing is done, when the plan's
// first pass cannot run by ranges.
constexpr int kInChunks = 8;
nn_status ntt_product_from_host(nn_context* c, u64* d_out, u64* da, const u64* ha, u64 na, u64* db, const u64* hb,
                                u64 nb, int s, u64* h_out, bool* used) {
  *used = false;
  const std::vector<nn::Pass> plan = c->passes(s);
  u64 tiles = 0;
  if (plan.size() < 2 || !nn::ntt_first_pass_tiles(s, plan[0], &tiles)) return NN_OK;
  *used = true;
  NN_CK(c, nn::tables_ensure(c->tables, s, c->stream, &c->retired_tables), "twiddle tables");
  nn_transform xa, xb;
  nn_status st = xform_reserve(c, &xa, s);
  if (st != NN_OK) return st;
  const u64 row = 1ull << (s - plan[0].R);           // limbs a row of the first pass
  const u64 full = na / row, part = na - full * row;  // full rows, limbs of the partial row
  const u64 k = std::min<u64>(kInChunks, tiles);
  cudaError_t e = cudaEventRecord(c->ev_first, c->stream);  // da and db are reused: after earlier work
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy, c->ev_first, 0);
  for (u64 j = 0; j < k && e == cudaSuccess; ++j) {
    const u64 t0 = tiles * j / k, t1 = tiles * (j + 1) / k, c0 = 16 * t0, c1 = 16 * t1;
    if (full)
      e = cudaMemcpy2DAsync(da + c0, row * 8, ha + c0, row * 8, (c1 - c0) * 8, full, cudaMemcpyHostToDevice, c->copy);
    if (e == cudaSuccess && part > c0)
      e = cudaMemcpyAsync(da + full * row + c0, ha + full * row + c0, (std::min(c1, part) - c0) * 8,
                          cudaMemcpyHostToDevice, c->copy);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_in, c->copy);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_in, 0);
    if (e == cudaSuccess) e = nn::ntt_first_pass_range(da, na, xa.res, s, c->tables, plan[0], t0, t1, c->stream);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(db, hb, nb * 8, cudaMemcpyHostToDevice, c->copy);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_second, c->copy);
  if (e == cudaSuccess) e = nn::ntt_forward_tail(xa.res, s, c->tables, c->stream, plan);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_second, 0);
  if (e != cudaSuccess) st = fail(c, e, "first operand by column ranges");
  if (st == NN_OK) st = forward_fused(c, &xb, db, nb, s, &xa);
  if (st == NN_OK) st = inverse_save_to_host(c, &xb, d_out, na + nb, h_out);
  dev_free(c, xa.res, xa.words);
  dev_free(c, xb.res, xb.words);
  return st;
}

// b_ready (optional): an event the contents of b wait for; the balanced NTT
// product waits for it after a's forward transform, the other paths at once.
nn_status mul_impl(nn_context* c, u64* d_out, const u64* a, u64 na, const u64* b, u64 nb,
                   cudaEvent_t b_ready = nullptr, u64* h_out = nullptr, bool* h_done = nullptr) {
  if (!d_out || !a || !b || na == 0 || nb == 0) {
    c->err = "mul: null pointer or empty operand";
    return NN_ERR_INVALID;
  }
  if (na < nb) {
    std::swap(a, b);
    std::swap(na, nb);
    if (b_ready) NN_CK(c, cudaStreamWaitEvent(c->stream, b_ready, 0), "wait for an operand");
    b_ready = nullptr;
  }
  const u64 a0 = (na + 1) >> 1;
  const bool balanced = nb >= kNttMulThreshold && ntt_scale(na, nb) == ntt_scale(a0, nb);
  if (b_ready && !balanced) {
    NN_CK(c, cudaStreamWaitEvent(c->stream, b_ready, 0), "wait for an operand");
    b_ready = nullptr;
  }
  if (nb < kNttMulThreshold) {  // natural.h:445-446 -> _mul_base
    NN_CK(c, nn::school_mul(a, na, b, nb, d_out, c->scan, c->stream), "base-case product");
    return NN_OK;
  }
  // natural::_mul_NTT (natural.h:391-419)
  const int s = ntt_scale(na, nb), s_opt = ntt_scale(a0, nb);
  if (s == s_opt) return ntt_product(c, d_out, a, na, b, nb, s, na + nb, nullptr, b_ready, h_out, h_done);
  // Unbalanced: b's transform is made once at s_opt and reused for both
  // halves of a (mul_save_NTT_info / mul_load_NTT_info, natural.h:452-515).
  const u64 a1 = na - a0;
  nn_transform xb, x0, x1;
  DBuf p0(c), p1(c);
  nn_status st = p0.alloc(a0 + nb);
  if (st == NN_OK) st = p1.alloc(a1 + nb);
  if (st == NN_OK) st = forward(c, &xb, b, nb, s_opt);
  if (st == NN_OK) st = forward(c, &x0, a, a0, s_opt);
  if (st == NN_OK) st = pointwise(c, &x0, &xb, &x0);
  if (st == NN_OK) st = inverse_save(c, &x0, p0.p, a0 + nb, nullptr);
  if (st == NN_OK) st = forward(c, &x1, a + a0, a1, s_opt);
  if (st == NN_OK) st = pointwise(c, &x1, &xb, &x1);
  if (st == NN_OK) st = inverse_save(c, &x1, p1.p, a1 + nb, nullptr);
  // (a1*b << a0 limbs) + a0*b  (natural.h:417)
  if (st == NN_OK) {
    cudaError_t e = nn::add_shifted(p0.p, a0 + nb, p1.p, a1 + nb, a0, d_out, na + nb, c->scan, c->stream);
    if (e != cudaSuccess) st = fail(c, e, "split combine");
  }
  dev_free(c, xb.res, xb.words);
  dev_free(c, x0.res, x0.words);
  dev_free(c, x1.res, x1.words);
  return st;
}

nn_status sqr_impl(nn_context* c, u64* d_out, const u64* a, u64 n) {
  if (!d_out || !a || n == 0) {
    c->err = "sqr: null pointer or empty operand";
    return NN_ERR_INVALID;
  }
  if (n < kNttMulThreshold) {  // natural.h:530-531 -> _sqr_base
    NN_CK(c, nn::school_mul(a, n, a, n, d_out, c->scan, c->stream), "base-case square");
    return NN_OK;
  }
  // natural::_sqr_NTT (natural.h:433-442): one transform, squared pointwise.
  const int s = ntt_scale(n, n);
  nn_transform x;
  nn_status st;
  if (c->passes(s).size() >= 2) {
    st = forward_fused(c, &x, a, n, s, nullptr);
    if (st == NN_OK) st = inverse_save(c, &x, d_out, 2 * n, nullptr, true);
  } else {
    st = forward(c, &x, a, n, s);
    if (st == NN_OK) st = pointwise(c, &x, &x, &x);
    if (st == NN_OK) st = inverse_save(c, &x, d_out, 2 * n, nullptr);
  }
  dev_free(c, x.res, x.words);
  return st;
}

// Grow-only device staging buffer `slot` of at least `words` limbs.
nn_status scratch(nn_context* c, int slot, u64 words, u64** p) {
  if (c->scratch_words[slot] < words) {
    dev_free(c, c->scratch[slot], c->scratch_words[slot]);
    c->scratch[slot] = nullptr;
    c->scratch_words[slot] = 0;
    u64 w = std::bit_ceil(std::max<u64>(words, 1024));
    nn_status st = dev_alloc(c, &c->scratch[slot], w);
    if (st != NN_OK) return st;
    c->scratch_words[slot] = w;
  }
  *p = c->scratch[slot];
  return NN_OK;
}

// ---------------------------------------------------------------------------
// Batches: a work queue over all jobs' pipeline steps (batch.cu).
// ---------------------------------------------------------------------------

// Batched transform time per word at each scale, relative (GB300: 10^9
// transform words per second of whole batched products at that scale, tiles
// merged, last pass fused; scales below 9 and above 20 estimated).
double batch_word_rate(int s) {
  static const double rate[] = {1.0, 1.0, 1.0, 1.0, 1.2, 1.4, 1.7, 2.0, 2.3, 2.57, 4.77, 6.94,
                                7.51, 6.9, 6.9, 6.66, 6.39, 6.08, 5.63, 5.66, 5.65};
  return s < (int)(sizeof rate / sizeof rate[0]) ? rate[s] : 5.0;
}

// An unbalanced product nx x ny (nx >= ny) may run as P pieces of k limbs of
// the longer operand, each through a transform of scale s2 < s sharing the
// shorter operand's: 2P + 1 transforms of 2^s2 words against 3 of 2^s.  The
// piece length is the most that keeps each piece's product within its
// transform (k + ny - 1 <= 2^s2), rounded down to a multiple of 8 (the CRT
// scan's vector loads stay within a piece), and at least ny, so that at most
// two pieces overlap at any product position.  Returns the scale; sets k, P
// (k = nx, P = 1: not split).
int batch_split(u64 nx, u64 ny, int s, u64* k, u64* P) {
  double best = 3.0 * (double)(1ull << s) / batch_word_rate(s);
  int s_best = s;
  *k = nx;
  *P = 1;
  for (int s2 = s - 1; s2 >= 2; --s2) {
    const u64 L2 = 1ull << s2;
    if (L2 + 1 < 2 * ny) break;
    const u64 kk = (L2 - ny + 1) & ~7ull;
    if (kk < ny || kk >= nx) continue;
    const u64 pieces = (nx + kk - 1) / kk;
    const double cost = (2.0 * pieces + 1.0) * (double)L2 / batch_word_rate(s2);
    if (cost < 0.95 * best) {
      best = cost;
      s_best = s2;
      *k = kk;
      *P = pieces;
    }
  }
  return s_best;
}

nn_status batch_plan(nn_context* c, nn_batch* B, const u64* na, const u64* nb, const int* square, u64 count) {
  if (count >= 0xffffffffull) {  // BatchItem::job is 32-bit
    c->err = "batch: too many products";
    return NN_ERR_INVALID;
  }
  B->count = count;
  B->na.assign(na, na + count);
  B->nb.assign(nb, nb + count);
  B->jobs.resize(count);
  B->off_a.assign(count, 0);
  B->off_b.assign(count, 0);
  B->swap.assign(count, 0);
  std::vector<int> steps(count, 0);
  std::vector<int> fused_at(count, -1);  // step of the fused items, -1 without
  int max_s = 2;
  size_t smem = 8;
  for (u64 j = 0; j < count; ++j) {
    if (!na[j] || !nb[j]) {
      c->err = "batch: empty operand";
      return NN_ERR_INVALID;
    }
    nn::BatchJob& J = B->jobs[j];
    J = nn::BatchJob{};
    J.na = na[j];
    J.nb = nb[j];
    J.piece = na[j];
    J.pieces = 1;
    J.ctr_base = B->n_ctrs;
    J.flag_base = B->n_flags;
    B->n_flags += (nn::u32)nn::scan_tiles(na[j] + nb[j]);
    const u64 mn = std::min(na[j], nb[j]), mx = std::max(na[j], nb[j]);
    if (mn < c->batch_ntt_min || (mn < c->batch_school_balanced && mx <= 2 * mn)) {
      J.s = 0;
      steps[j] = 1;
      smem = std::max(smem, nn::kColumnTileSmem);  // the item's column sums
    } else {
      J.square = square ? square[j] : 0;
      if (J.square && na[j] != nb[j]) {
        c->err = "batch: a square needs equal operand sizes";
        return NN_ERR_INVALID;
      }
      // operand 0 is the longer one; it may be split into pieces
      B->swap[j] = na[j] < nb[j];
      J.na = std::max(na[j], nb[j]);
      J.nb = std::min(na[j], nb[j]);
      J.piece = J.na;
      int s = ntt_scale(J.na, J.nb);
      if (c->batch_solo_scale > 0 && s >= c->batch_solo_scale) {
        // From this scale on the one-product passes (TMA tiles, fused last
        // pass) beat the batch kernel's generic tiles (GB300, 4 products of
        // 2^21 limbs: 4.65 ms against 5.55 ms), and one product already fills
        // the GPU: no items, no arena; the launch runs it alone.
        B->solo.push_back(j);
        continue;
      }
      if (c->batch_split && !J.square) s = batch_split(J.na, J.nb, s, &J.piece, &J.pieces);
      J.s = s;
      max_s = std::max(max_s, s);
      const std::vector<nn::Pass> plan = c->batch_passes(s);
      if (plan.size() > 4) {
        c->err = "batch: transform too long for one batch";
        return NN_ERR_INVALID;
      }
      J.n_pass = (int)plan.size();
      for (int k = 0; k < J.n_pass; ++k) {
        J.lambda0[k] = plan[k].lambda0;
        J.R[k] = plan[k].R;
        J.C[k] = plan[k].C;
        J.skip[k] = 0;
        if (c->batch_merge) {
          // Small tiles leave most of a CTA's 256 threads idle and cut the
          // levels into radix-2 and radix-4 sweeps; work on 2048 words at once:
          // pass 0's strided tiles get up to 128 columns (as many as its
          // column blocks hold), later contiguous passes take 2^skip
          // consecutive tiles as one tile of R + skip levels.
          const int lg_s = s - plan[k].lambda0 - plan[k].R;
          if (k == 0 && plan[k].C == 16)
            while ((J.C[k] << J.R[k]) < kMergedTileWords && J.C[k] < 128 && 2 * J.C[k] <= (1 << lg_s)) J.C[k] *= 2;
          if (k > 0 && plan[k].C == 2)
            while ((2 << J.R[k]) < kMergedTileWords && J.skip[k] < plan[k].lambda0) {
              ++J.skip[k];
              ++J.R[k];
              --J.lambda0[k];
            }
        }
        smem = std::max(smem, nn::tile_smem_bytes(J.C[k], J.R[k]));
      }
      const int m = J.n_pass;
      if (c->batch_fused && m >= 2 && J.C[m - 1] == 2) {
        // forward passes 0..m-2 of both operands, the second operand's last
        // pass (not for a square), the fused step, inverse passes m-2..0, CRT
        fused_at[j] = J.square ? m - 1 : m;
        steps[j] = fused_at[j] + m + 1;
      } else {
        steps[j] = 2 * m + 2;
      }
      B->off_a[j] = B->arena_words;
      B->arena_words += J.pieces * (3ull << s);
      if (!J.square) {
        B->off_b[j] = B->arena_words;
        B->arena_words += 3ull << s;
      }
    }
    B->n_ctrs += steps[j];
  }
  B->need.assign(B->n_ctrs, 0);
  const int max_steps = *std::max_element(steps.begin(), steps.end());  // 0 when every job runs alone
  B->items.clear();
  for (int st = 0; st < max_steps; ++st) {
    for (u64 j = 0; j < count; ++j) {
      if (st >= steps[j]) continue;
      const nn::BatchJob& J = B->jobs[j];
      auto push = [&](unsigned char kind, int pass, int prime, int operand, u64 tile, u64 ntile = 1) {
        nn::BatchItem it{};
        it.job = (nn::u32)j;
        it.step = (unsigned short)st;
        it.kind = kind;
        it.pass = (unsigned char)pass;
        it.prime = (unsigned char)prime;
        it.operand = (unsigned char)operand;
        it.tile = (nn::u32)tile;
        it.ntile = (unsigned short)ntile;
        B->items.push_back(it);
        B->need[J.ctr_base + st] += 1;
      };
      if (J.s == 0) {
        for (u64 t = 0; t < nn::scan_tiles(J.na + J.nb); ++t) push(nn::kItemColumn, 0, 0, 0, t);
        continue;
      }
      const int m = J.n_pass;
      const u64 L = 1ull << J.s;
      // items of pass k over operand 0's pieces (tiles numbered across them) or operand 1
      auto pass_items = [&](unsigned char kind, int k, int operand) {
        const u64 tw = (u64)J.C[k] << J.R[k], tiles = (L / tw) * (operand == 0 ? J.pieces : 1);
        const u64 per = std::clamp<u64>(c->batch_item_words / tw, 1, 0xffff);  // BatchItem::ntile is 16-bit
        for (int pr = 0; pr < 3; ++pr)
          for (u64 t = 0; t < tiles; t += per) push(kind, k, pr, operand, t, std::min(per, tiles - t));
      };
      auto crt_items = [&] {
        for (u64 t = 0; t < nn::scan_tiles(J.na + J.nb); ++t) push(nn::kItemCrt, 0, 0, 0, t);
      };
      if (const int f = fused_at[j]; f >= 0) {
        if (st < m - 1) {
          for (int op = 0; op < (J.square ? 1 : 2); ++op) pass_items(nn::kItemFwd, st, op);
        } else if (st < f) {
          pass_items(nn::kItemFwd, m - 1, 1);  // the second operand's last pass
        } else if (st == f) {
          pass_items(nn::kItemFused, m - 1, 0);
        } else if (st < f + m) {
          pass_items(nn::kItemInv, f + m - 1 - st, 0);  // inverse passes m-2 .. 0
        } else {
          crt_items();
        }
        continue;
      }
      if (st < m) {  // forward pass st of each operand
        for (int op = 0; op < (J.square ? 1 : 2); ++op) pass_items(nn::kItemFwd, st, op);
      } else if (st == m) {
        const u64 chunks = (L / 4 + nn::kBatchPointwiseChunk - 1) / nn::kBatchPointwiseChunk * J.pieces;
        for (int pr = 0; pr < 3; ++pr)
          for (u64 t = 0; t < chunks; ++t) push(nn::kItemPointwise, 0, pr, 0, t);
      } else if (st < 2 * m + 1) {  // inverse passes m-1 .. 0
        pass_items(nn::kItemInv, 2 * m - st, 0);
      } else {
        crt_items();
      }
    }
  }
  if (B->items.size() >= 0xffffffffull) {
    c->err = "batch: too many work items";
    return NN_ERR_INVALID;
  }
  B->smem = smem;
  NN_CK(c, nn::tables_ensure(c->tables, max_s, c->stream, &c->retired_tables), "twiddle tables");
  int per_sm = 0;
  NN_CK(c, nn::batch_configure(&per_sm, smem), "batch kernel attributes");
  if (c->batch_blocks_per_sm > 0) per_sm = std::min(per_sm, c->batch_blocks_per_sm);
  int sms = 0;
  NN_CK(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device), "device attributes");
  B->grid = std::max(1, per_sm) * sms;
  // device tables
  // Regions in one allocation, each rounded to 256 bytes: the residues are
  // read and written with 16-byte vector accesses.
  auto words = [](u64 bytes) { return (bytes + 255) / 256 * 32; };
  const u64 w_jobs = words(count * sizeof(nn::BatchJob)), w_items = words(B->items.size() * sizeof(nn::BatchItem));
  const u64 w_need = words(4ull * B->n_ctrs), w_state = words(4ull * (B->n_ctrs + 4)),
            w_flags = words(4ull * (B->n_flags + 2));
  u64* p = nullptr;
  B->dev_words = w_jobs + w_items + w_need + w_state + w_flags + B->arena_words;
  nn_status st = dev_alloc(c, &p, B->dev_words);
  if (st != NN_OK) return st;
  B->d_jobs = reinterpret_cast<nn::BatchJob*>(p);
  B->d_items = reinterpret_cast<nn::BatchItem*>(p + w_jobs);
  B->d_need = reinterpret_cast<nn::u32*>(p + w_jobs + w_items);
  B->d_state = reinterpret_cast<nn::u32*>(p + w_jobs + w_items + w_need);
  B->d_flags = reinterpret_cast<nn::u32*>(p + w_jobs + w_items + w_need + w_state);
  B->d_arena = p + w_jobs + w_items + w_need + w_state + w_flags;
  NN_CK(c, c->stage.upload(B->d_items, B->items.data(), B->items.size() * sizeof(nn::BatchItem), c->stream),
        "upload items");
  NN_CK(c, c->stage.upload(B->d_need, B->need.data(), B->need.size() * 4, c->stream), "upload counts");
  NN_CK(c, cudaEventCreateWithFlags(&B->ran, cudaEventDisableTiming), "event");
  return NN_OK;
}

// Records the run sequence (job table upload, counter resets, persistent
// kernel) into a CUDA graph on the context's own stream.
nn_status batch_capture(nn_context* c, nn_batch* B) {
  cudaStream_t cs = c->own;
  NN_CK(c, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
  cudaMemcpyAsync(B->d_jobs, B->h_jobs, B->count * sizeof(nn::BatchJob), cudaMemcpyHostToDevice, cs);
  cudaMemsetAsync(B->d_state, 0, (B->n_ctrs + 4) * 4, cs);
  cudaMemsetAsync(B->d_flags, 0, (B->n_flags + 2) * 4, cs);
  cudaError_t le = nn::batch_launch(B->d_jobs, B->d_items, (nn::u32)B->items.size(), B->d_need, B->d_state,
                                    B->d_state + B->n_ctrs, B->d_flags, c->scan.err, c->tables, B->grid, B->smem, cs);
  cudaError_t e = cudaStreamEndCapture(cs, &B->graph);
  if (le != cudaSuccess) return fail(c, le, "batch launch (capture)");
  NN_CK(c, e, "end capture");
  NN_CK(c, cudaGraphInstantiate(&B->exec, B->graph, 0), "graph instantiate");
  return NN_OK;
}

void batch_release(nn_context* c, nn_batch* B) {
  if (B->pending) cudaEventSynchronize(B->ran);
  if (B->exec) cudaGraphExecDestroy(B->exec);
  if (B->graph) cudaGraphDestroy(B->graph);
  if (B->ran) cudaEventDestroy(B->ran);
  if (B->h_jobs) cudaFreeHost(B->h_jobs);
  dev_free(c, reinterpret_cast<u64*>(B->d_jobs), B->dev_words);
  delete B;
}

u64 normalized(const u64* x, u64 n) {  // natural::std (natural.h:82-93)
  while (n > 1 && x[n - 1] == 0) --n;
  return n;
}

}  // namespace

// Context access for the other host translation units (context_access.h).
namespace nn {
cudaStream_t ctx_stream(nn_context* c) { return c->stream; }
Scan& ctx_scan(nn_context* c) { return c->scan; }
nn_status ctx_alloc(nn_context* c, u64** p, u64 words) { return dev_alloc(c, p, words); }
void ctx_free(nn_context* c, u64* p, u64 words) { dev_free(c, p, words); }
nn_status ctx_mul(nn_context* c, u64* out, const u64* a, u64 na, const u64* b, u64 nb) {
  return mul_impl(c, out, a, na, b, nb);
}
nn_status ctx_fail(nn_context* c, cudaError_t e, const char* what) { return fail(c, e, what); }
cudaError_t ctx_upload(nn_context* c, void* d_dst, const void* h_src, u64 bytes) {
  return c->stage.upload(d_dst, h_src, bytes, c->stream);
}
void ctx_error(nn_context* c, const char* msg) { c->err = msg; }
nn_status ctx_scratch(nn_context* c, int slot, u64 words, u64** p) { return scratch(c, slot, words, p); }
}  // namespace nn

extern "C" {

const char* nn_status_string(nn_status s) {
  switch (s) {
    case NN_OK: return "ok";
    case NN_ERR_INVALID: return "invalid argument";
    case NN_ERR_OOM: return "device out of memory";
    case NN_ERR_CUDA: return "CUDA error";
    case NN_ERR_TIMEOUT: return "device wait timed out";
    case NN_ERR_BUDGET: return "HBM budget exceeded";
    case NN_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown";
}

uint64_t nn_launch_count(void) { return nn::launch_count(); }

void nn_profile_enable(int on) { nn::profile_enable(on != 0); }

uint64_t nn_profile_report(char* buf, uint64_t cap) {
  std::string r = nn::profile_report();
  if (buf && cap) {
    u64 n = std::min<u64>(cap - 1, r.size());
    std::memcpy(buf, r.data(), n);
    buf[n] = 0;
  }
  return r.size();
}

// The tunables autotune.py measured on this GPU model (the "tunables" object
// of tuning.json: "name": integer pairs), applied to every new context, so
// that contexts made through the C ABI (the drop-in header's, the request
// server's) run the same tuned pass splits and batch shapes as Python ones.
// The file: $NN_TUNING ("off": none), else tuning.json in the directory above
// the one holding this library.  A missing or unreadable file leaves the
// defaults.
static void apply_tuning_file(nn_context* c) {
  std::string path;
  if (const char* e = std::getenv("NN_TUNING")) {
    if (std::strcmp(e, "off") == 0) return;
    path = e;
  } else {
    Dl_info info{};
    if (!dladdr(reinterpret_cast<void*>(&apply_tuning_file), &info) || !info.dli_fname) return;
    std::string lib(info.dli_fname);
    const size_t slash = lib.rfind('/');
    const std::string dir = slash == std::string::npos ? "." : lib.substr(0, slash);
    path = dir + "/../tuning.json";
  }
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return;
  std::string text;
  char buf[4096];
  for (size_t n; (n = std::fread(buf, 1, sizeof buf, f)) > 0;) text.append(buf, n);
  std::fclose(f);
  size_t at = text.find("\"tunables\"");
  if (at == std::string::npos) return;
  at = text.find('{', at);
  const size_t end = at == std::string::npos ? at : text.find('}', at);
  if (end == std::string::npos) return;
  for (size_t q = text.find('"', at); q != std::string::npos && q < end; q = text.find('"', q)) {
    const size_t q2 = text.find('"', q + 1);
    if (q2 == std::string::npos || q2 > end) break;
    const std::string key = text.substr(q + 1, q2 - q - 1);
    const size_t colon = text.find(':', q2);
    if (colon == std::string::npos || colon > end) break;
    char* stop = nullptr;
    const long long v = std::strtoll(text.c_str() + colon + 1, &stop, 10);
    if (stop != text.c_str() + colon + 1) nn_context_set_tunable(c, key.c_str(), v);
    q = stop ? (size_t)(stop - text.c_str()) : colon + 1;
  }
  c->err.clear();  // an unknown key from another version is not an error of this context
}

nn_status nn_context_create(int device, uint64_t budget, nn_context** out) {
  if (!out) return NN_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) {
    cudaGetLastError();
    return NN_ERR_NO_DEVICE;
  }
  nn_context* c = new nn_context;
  c->device = device;
  c->budget = budget;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_first, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_second, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_chunk, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming);
  if (e == cudaSuccess) e = nn::upload_primes();
  if (e == cudaSuccess) {
    cudaMemPool_t pool;
    e = cudaDeviceGetDefaultMemPool(&pool, device);
    if (e == cudaSuccess) {
      uint64_t keep = ~0ull;  // keep freed blocks cached for reuse
      e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  if (e == cudaSuccess) e = nn::scan_reserve(c->scan, 1024);
  c->tables.err = c->scan.err;
  if (e != cudaSuccess) {
    nn_status st = e == cudaErrorNoDevice || e == cudaErrorNoKernelImageForDevice ? NN_ERR_NO_DEVICE : NN_ERR_CUDA;
    cudaGetLastError();
    if (c->ev_in) cudaEventDestroy(c->ev_in);
    if (c->ev_chunk) cudaEventDestroy(c->ev_chunk);
    if (c->ev_second) cudaEventDestroy(c->ev_second);
    if (c->ev_first) cudaEventDestroy(c->ev_first);
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
    return st;
  }
  c->stream = c->own;
  apply_tuning_file(c);
  *out = c;
  return NN_OK;
}

nn_status nn_context_destroy(nn_context* c) {
  if (!c) return NN_ERR_INVALID;
  cudaSetDevice(c->device);
  // Work the caller ordered on its own stream must be finished (or that
  // stream still alive); teardown itself only uses the context's stream.
  if (c->stream != c->own) cudaStreamSynchronize(c->stream);
  c->stream = c->own;
  cudaStreamSynchronize(c->own);
  for (int i = 0; i < 3; ++i) dev_free(c, c->scratch[i], c->scratch_words[i]);
  cudaStreamSynchronize(c->own);
  nn::tables_free(c->tables);
  for (u64* p : c->retired_tables) cudaFree(p);
  c->retired_tables.clear();
  nn::scan_free(c->scan);
  c->stage.release();
  cudaStreamSynchronize(c->copy);
  cudaEventDestroy(c->ev_in);
  cudaEventDestroy(c->ev_chunk);
  cudaEventDestroy(c->ev_second);
  cudaEventDestroy(c->ev_first);
  cudaStreamDestroy(c->copy);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return NN_OK;
}

nn_status nn_context_set_stream(nn_context* c, void* s) {
  if (!c) return NN_ERR_INVALID;
  c->stream = (cudaStream_t)s;  // NULL is the legacy default stream, as in CUDA
  return NN_OK;
}

nn_status nn_context_use_own_stream(nn_context* c) {
  if (!c) return NN_ERR_INVALID;
  c->stream = c->own;
  return NN_OK;
}

void* nn_context_stream(nn_context* c) { return c ? (void*)c->stream : nullptr; }

nn_status nn_context_synchronize(nn_context* c) {
  if (!c) return NN_ERR_INVALID;
  NN_CK(c, cudaStreamSynchronize(c->stream), "synchronize");
  nn::u32 err = 0;
  NN_CK(c, cudaMemcpy(&err, c->scan.err, sizeof err, cudaMemcpyDeviceToHost), "read error flag");
  if (err) {
    cudaMemset(c->scan.err, 0, sizeof err);
    c->err = "carry lookback wait exceeded its bound";
    return NN_ERR_TIMEOUT;
  }
  return NN_OK;
}

nn_status nn_context_probe_wait(nn_context* c, int spin_limit) {
  if (!c || spin_limit < 0) return NN_ERR_INVALID;
  NN_CK(c, nn::wait_probe(c->scan, spin_limit, c->stream), "wait probe");
  return nn_context_synchronize(c);
}

const char* nn_last_error(const nn_context* c) { return c ? c->err.c_str() : "no context"; }

uint64_t nn_context_device_bytes(const nn_context* c) {
  if (!c) return 0;
  return c->held + 2 * 3 * c->tables.cap * sizeof(u64) + (c->scan.max_tiles + 1) * 4;
}

nn_status nn_transform_create(nn_context* c, nn_transform** out) {
  if (!c || !out) return NN_ERR_INVALID;
  *out = new nn_transform;
  return NN_OK;
}

nn_status nn_transform_destroy(nn_context* c, nn_transform* t) {
  if (!c || !t) return NN_ERR_INVALID;
  dev_free(c, t->res, t->words);
  delete t;
  return NN_OK;
}

int nn_transform_scale(const nn_transform* t) { return t ? t->scale : 0; }
void nn_transform_set_scale(nn_transform* t, int s) {
  if (t) t->scale = s;
}

nn_status nn_transform_forward(nn_context* c, nn_transform* t, const uint64_t* d, uint64_t n, int s) {
  if (!c || !t || !d) return NN_ERR_INVALID;
  return forward(c, t, d, n, s);
}

nn_status nn_transform_pointwise(nn_context* c, nn_transform* dst, const nn_transform* a, const nn_transform* b) {
  if (!c || !dst || !a || !b || !a->res || !b->res) return NN_ERR_INVALID;
  return pointwise(c, dst, a, b);
}

nn_status nn_transform_inverse_save(nn_context* c, nn_transform* t, uint64_t* d_out, uint64_t size,
                                    uint64_t* written) {
  if (!c || !t || !t->res || !d_out) return NN_ERR_INVALID;
  return inverse_save(c, t, d_out, size, written);
}

nn_status nn_transform_residues(nn_context* c, const nn_transform* t, uint64_t* d_out) {
  if (!c || !t || !t->res || !d_out) return NN_ERR_INVALID;
  NN_CK(c, cudaMemcpyAsync(d_out, t->res, (3ull << t->scale) * sizeof(u64), cudaMemcpyDeviceToDevice, c->stream),
        "copy residues");
  return NN_OK;
}

nn_status nn_mul(nn_context* c, uint64_t* d_out, const uint64_t* a, uint64_t na, const uint64_t* b, uint64_t nb) {
  if (!c) return NN_ERR_INVALID;
  return mul_impl(c, d_out, a, na, b, nb);
}

nn_status nn_sqr(nn_context* c, uint64_t* d_out, const uint64_t* a, uint64_t n) {
  if (!c) return NN_ERR_INVALID;
  return sqr_impl(c, d_out, a, n);
}

nn_status nn_ntt_mul(nn_context* c, uint64_t* d_out, const uint64_t* a, uint64_t na, const uint64_t* b, uint64_t nb,
                     int s, uint64_t size, uint64_t* written) {
  if (!c || !d_out || !a || !b) return NN_ERR_INVALID;
  return ntt_product(c, d_out, a, na, b, nb, s, size, written);
}

nn_status nn_mul_base(nn_context* c, uint64_t* d_out, const uint64_t* a, uint64_t na, const uint64_t* b,
                      uint64_t nb) {
  if (!c || !d_out || !a || !b || !na || !nb) return NN_ERR_INVALID;
  NN_CK(c, nn::school_mul(a, na, b, nb, d_out, c->scan, c->stream), "base-case product");
  return NN_OK;
}

nn_status nn_mul_host(nn_context* c, uint64_t* out, uint64_t* out_n, const uint64_t* a, uint64_t na,
                      const uint64_t* b, uint64_t nb) {
  if (!c || !out || !a || !b || !na || !nb) return NN_ERR_INVALID;
  if (na < nb) {  // the longer operand first: it is transformed first
    std::swap(a, b);
    std::swap(na, nb);
  }
  // Copies, not kernels reading and writing page-locked host memory in
  // place: measured on GB300 at 2^27 limbs, in-place access over the host
  // link made the product 7 to 95 ms slower than these copies.
  u64 *da, *db, *dout;
  nn_status st = scratch(c, 0, na, &da);
  if (st == NN_OK) st = scratch(c, 1, nb, &db);
  if (st == NN_OK) st = scratch(c, 2, na + nb, &dout);
  if (st != NN_OK) return st;
  const int s = ntt_scale(na, nb);
  if (nb >= kNttMulThreshold && s == ntt_scale((na + 1) >> 1, nb)) {  // balanced NTT product
    bool used = false;
    st = ntt_product_from_host(c, dout, da, a, na, db, b, nb, s, out, &used);
    if (used || st != NN_OK) {
      if (st == NN_OK) st = nn_context_synchronize(c);
      const cudaError_t e = cudaStreamSynchronize(c->copy);
      if (st == NN_OK && e != cudaSuccess) st = fail(c, e, "copy-back");
      if (st == NN_OK && out_n) *out_n = normalized(out, na + nb);
      return st;
    }
  }
  // a on the context's stream; b on the copy stream once a is in, so that
  // b's copy runs while a is transformed.
  NN_CK(c, cudaMemcpyAsync(da, a, na * 8, cudaMemcpyHostToDevice, c->stream), "H2D");
  NN_CK(c, cudaEventRecord(c->ev_first, c->stream), "event record");
  NN_CK(c, cudaStreamWaitEvent(c->copy, c->ev_first, 0), "copy stream wait");
  NN_CK(c, cudaMemcpyAsync(db, b, nb * 8, cudaMemcpyHostToDevice, c->copy), "H2D");
  NN_CK(c, cudaEventRecord(c->ev_second, c->copy), "event record");
  bool copied = false;  // the balanced NTT path copies the product back while its carry scan runs
  st = mul_impl(c, dout, da, na, db, nb, c->ev_second, out, &copied);
  if (st != NN_OK) {
    cudaStreamSynchronize(c->copy);
    return st;
  }
  if (!copied) NN_CK(c, cudaMemcpyAsync(out, dout, (na + nb) * 8, cudaMemcpyDeviceToHost, c->stream), "D2H");
  st = nn_context_synchronize(c);
  NN_CK(c, cudaStreamSynchronize(c->copy), "copy-back");
  if (st == NN_OK && out_n) *out_n = normalized(out, na + nb);
  return st;
}

nn_status nn_sqr_host(nn_context* c, uint64_t* out, uint64_t* out_n, const uint64_t* a, uint64_t n) {
  if (!c || !out || !a || !n) return NN_ERR_INVALID;
  u64 *da, *dout;
  nn_status st = scratch(c, 0, n, &da);
  if (st == NN_OK) st = scratch(c, 2, 2 * n, &dout);
  if (st != NN_OK) return st;
  NN_CK(c, cudaMemcpyAsync(da, a, n * 8, cudaMemcpyHostToDevice, c->stream), "H2D");
  st = sqr_impl(c, dout, da, n);
  if (st != NN_OK) return st;
  NN_CK(c, cudaMemcpyAsync(out, dout, 2 * n * 8, cudaMemcpyDeviceToHost, c->stream), "D2H");
  st = nn_context_synchronize(c);
  if (st == NN_OK && out_n) *out_n = normalized(out, 2 * n);
  return st;
}

nn_status nn_mul_base_host(nn_context* c, uint64_t* out, const uint64_t* a, uint64_t na, const uint64_t* b,
                           uint64_t nb) {
  if (!c || !out || !a || !b || !na || !nb) return NN_ERR_INVALID;
  u64 *da, *db, *dout;
  nn_status st = scratch(c, 0, na, &da);
  if (st == NN_OK) st = scratch(c, 1, nb, &db);
  if (st == NN_OK) st = scratch(c, 2, na + nb, &dout);
  if (st != NN_OK) return st;
  NN_CK(c, cudaMemcpyAsync(da, a, na * 8, cudaMemcpyHostToDevice, c->stream), "H2D");
  NN_CK(c, cudaMemcpyAsync(db, b, nb * 8, cudaMemcpyHostToDevice, c->stream), "H2D");
  NN_CK(c, nn::school_mul(da, na, db, nb, dout, c->scan, c->stream), "base-case product");
  NN_CK(c, cudaMemcpyAsync(out, dout, (na + nb) * 8, cudaMemcpyDeviceToHost, c->stream), "D2H");
  return nn_context_synchronize(c);
}

nn_status nn_transform_forward_host(nn_context* c, nn_transform* t, const uint64_t* limbs, uint64_t n, int s) {
  if (!c || !t || !limbs || !n) return NN_ERR_INVALID;
  u64* d;
  nn_status st = scratch(c, 0, n, &d);
  if (st != NN_OK) return st;
  NN_CK(c, cudaMemcpyAsync(d, limbs, n * 8, cudaMemcpyHostToDevice, c->stream), "H2D");
  return forward(c, t, d, n, s);
}

nn_status nn_transform_inverse_save_host(nn_context* c, nn_transform* t, uint64_t* out, uint64_t size,
                                         uint64_t* written) {
  if (!c || !t || !t->res || !out) return NN_ERR_INVALID;
  const u64 L = 1ull << t->scale;
  u64* d;
  nn_status st = scratch(c, 2, std::max<u64>(size, L), &d);
  if (st != NN_OK) return st;
  u64 w = 0;
  st = inverse_save(c, t, d, size, &w);
  if (st != NN_OK) return st;
  NN_CK(c, cudaMemcpyAsync(out, d, w * 8, cudaMemcpyDeviceToHost, c->stream), "D2H");
  st = nn_context_synchronize(c);
  if (written) *written = w;
  return st;
}

nn_status nn_context_set_tunable(nn_context* c, const char* name, int64_t v) {
  if (!c || !name) return NN_ERR_INVALID;
  std::string k(name);
  const size_t at = k.find('@');
  if (at != std::string::npos) {  // per-scale pass split: "r_last@28", "r_col@28", "batch_r_last@16"
    const std::string base = k.substr(0, at);
    const int sc = std::atoi(k.c_str() + at + 1);
    const bool rl = base == "r_last" || base == "batch_r_last";
    if (sc >= 2 && sc < 64 && ((rl && (v == 0 || (v >= 3 && v <= 12))) || (base == "r_col" && v >= 0 && v <= 9))) {
      (base == "r_last" ? c->r_last_at : base == "r_col" ? c->r_col_at : c->batch_r_last_at)[sc] = (int)v;
      return NN_OK;
    }
    c->err = "unknown tunable or value out of range: " + k;
    return NN_ERR_INVALID;
  }
  if (k == "r_last" && v >= 3 && v <= 12)
    c->r_last = (int)v;
  else if (k == "r_col" && v >= 1 && v <= 9)
    c->r_col = (int)v;
  else if (k == "batch_ntt_min" && v >= 1)
    c->batch_ntt_min = (u64)v;
  else if (k == "batch_item_words" && v >= 1 && v <= (1 << 20))
    c->batch_item_words = (u64)v;
  else if (k == "batch_fused" && (v == 0 || v == 1))
    c->batch_fused = (int)v;
  else if (k == "batch_merge" && (v == 0 || v == 1))
    c->batch_merge = (int)v;
  else if (k == "batch_split" && (v == 0 || v == 1))
    c->batch_split = (int)v;
  else if (k == "batch_blocks_per_sm" && v >= 0 && v <= 32)
    c->batch_blocks_per_sm = (int)v;
  else if (k == "batch_solo_scale" && (v == 0 || (v >= 2 && v < 64)))
    c->batch_solo_scale = (int)v;
  else if (k == "batch_school_balanced" && v >= 0)
    c->batch_school_balanced = (u64)v;
  else {
    c->err = "unknown tunable or value out of range: " + k;
    return NN_ERR_INVALID;
  }
  return NN_OK;
}

int64_t nn_context_get_tunable(const nn_context* c, const char* name) {
  if (!c || !name) return -1;
  std::string k(name);
  const size_t at = k.find('@');
  if (at != std::string::npos) {
    const int sc = std::atoi(k.c_str() + at + 1);
    if (sc < 2 || sc >= 64) return -1;
    if (k.substr(0, at) == "r_last") return c->r_last_at[sc];
    if (k.substr(0, at) == "r_col") return c->r_col_at[sc];
    if (k.substr(0, at) == "batch_r_last") return c->batch_r_last_at[sc];
    return -1;
  }
  if (k == "r_last") return c->r_last;
  if (k == "r_col") return c->r_col;
  if (k == "batch_ntt_min") return (int64_t)c->batch_ntt_min;
  if (k == "batch_item_words") return (int64_t)c->batch_item_words;
  if (k == "batch_fused") return (int64_t)c->batch_fused;
  if (k == "batch_merge") return (int64_t)c->batch_merge;
  if (k == "batch_split") return (int64_t)c->batch_split;
  if (k == "batch_blocks_per_sm") return c->batch_blocks_per_sm;
  if (k == "batch_solo_scale") return c->batch_solo_scale;
  if (k == "batch_school_balanced") return (int64_t)c->batch_school_balanced;
  return -1;
}

nn_status nn_batch_create(nn_context* c, const uint64_t* na, const uint64_t* nb, const int* square, uint64_t count,
                          nn_batch** out) {
  if (!c || !na || !nb || !count || !out) return NN_ERR_INVALID;
  *out = nullptr;
  nn_batch* B = new nn_batch;
  nn_status st = batch_plan(c, B, na, nb, square, count);
  if (st != NN_OK) {
    batch_release(c, B);
    return st;
  }
  *out = B;
  return NN_OK;
}

}  // extern "C"

namespace {  // helpers of the batch entry points, not exported

// Fills a job table (the plan's pinned one, or `into`) for one run.
nn_status batch_fill(nn_context* c, nn_batch* B, const nn_mul_job* jobs, nn::BatchJob* into = nullptr) {
  nn::BatchJob* dst = into ? into : B->h_jobs;
  for (u64 j = 0; j < B->count; ++j) {
    if (jobs[j].n_a != B->na[j] || jobs[j].n_b != B->nb[j] || !jobs[j].d_a || !jobs[j].d_b || !jobs[j].d_out) {
      c->err = "batch run: job does not match the plan";
      return NN_ERR_INVALID;
    }
    nn::BatchJob J = B->jobs[j];
    J.a = B->swap[j] ? jobs[j].d_b : jobs[j].d_a;
    J.b = B->swap[j] ? jobs[j].d_a : jobs[j].d_b;
    J.out = jobs[j].d_out;
    J.res_a = B->d_arena + B->off_a[j];
    J.res_b = B->d_arena + B->off_b[j];
    dst[j] = J;
  }
  return NN_OK;
}

// The plan's large products, one at a time on the context's stream.
nn_status batch_solo(nn_context* c, const nn_batch* B, const nn_mul_job* jobs) {
  for (u64 j : B->solo) {
    const nn_mul_job& m = jobs[j];
    const nn_status st = B->jobs[j].square ? sqr_impl(c, m.d_out, m.d_a, m.n_a)
                                           : mul_impl(c, m.d_out, m.d_a, m.n_a, m.d_b, m.n_b);
    if (st != NN_OK) return st;
  }
  return NN_OK;
}

}  // namespace

extern "C" {

nn_status nn_batch_launch(nn_context* c, nn_batch* B, const nn_mul_job* jobs) {
  if (!c || !B || !jobs) return NN_ERR_INVALID;
  if (B->pending) NN_CK(c, cudaEventSynchronize(B->ran), "previous batch run");
  // The table goes up through the context's page-locked ring: the call
  // returns without waiting for the stream's earlier work.
  std::vector<nn::BatchJob> table(B->count);
  nn_status st = batch_fill(c, B, jobs, table.data());
  if (st != NN_OK) return st;
  if (!B->items.empty()) {
    NN_CK(c, c->stage.upload(B->d_jobs, table.data(), B->count * sizeof(nn::BatchJob), c->stream), "upload jobs");
    NN_CK(c, cudaMemsetAsync(B->d_state, 0, (B->n_ctrs + 4) * 4, c->stream), "reset counters");
    NN_CK(c, cudaMemsetAsync(B->d_flags, 0, (B->n_flags + 2) * 4, c->stream), "reset flags");
    nn::launch_begin("batch_persistent", c->stream);
    cudaError_t le = nn::batch_launch(B->d_jobs, B->d_items, (nn::u32)B->items.size(), B->d_need, B->d_state,
                                      B->d_state + B->n_ctrs, B->d_flags, c->scan.err, c->tables, B->grid,
                                      B->smem, c->stream);
    nn::launch_end(c->stream);
    NN_CK(c, le, "batch launch");
  }
  st = batch_solo(c, B, jobs);
  if (st != NN_OK) return st;
  NN_CK(c, cudaEventRecord(B->ran, c->stream), "event record");
  B->pending = true;
  return NN_OK;
}

nn_status nn_batch_run(nn_context* c, nn_batch* B, const nn_mul_job* jobs) {
  if (!c || !B || !jobs) return NN_ERR_INVALID;
  if (B->pending) NN_CK(c, cudaEventSynchronize(B->ran), "previous batch run");
  if (!B->h_jobs)  // pinned, so the graph's upload node can read it at replay time
    NN_CK(c, cudaHostAlloc((void**)&B->h_jobs, B->count * sizeof(nn::BatchJob), cudaHostAllocDefault),
          "pinned jobs");
  nn_status fst = batch_fill(c, B, jobs);
  if (fst != NN_OK) return fst;
  if (!B->items.empty()) {
    if (!B->exec) {
      nn_status st = batch_capture(c, B);
      if (st != NN_OK) return st;
    }
    nn::launch_begin("batch_persistent", c->stream);
    cudaError_t ge = cudaGraphLaunch(B->exec, c->stream);
    nn::launch_end(c->stream);
    NN_CK(c, ge, "graph launch");
  }
  fst = batch_solo(c, B, jobs);
  if (fst != NN_OK) return fst;
  NN_CK(c, cudaEventRecord(B->ran, c->stream), "event record");
  B->pending = true;
  return NN_OK;
}

nn_status nn_batch_destroy(nn_context* c, nn_batch* B) {
  if (!c || !B) return NN_ERR_INVALID;
  batch_release(c, B);
  return NN_OK;
}

uint64_t nn_batch_items(const nn_batch* B) { return B ? B->items.size() : 0; }

nn_status nn_mul_each(nn_context* c, const nn_mul_job* jobs, uint64_t count) {
  if (!c || !jobs) return NN_ERR_INVALID;
  for (u64 j = 0; j < count; ++j) {
    nn_status st = mul_impl(c, jobs[j].d_out, jobs[j].d_a, jobs[j].n_a, jobs[j].d_b, jobs[j].n_b);
    if (st != NN_OK) return st;
  }
  return NN_OK;
}

nn_status nn_batch_mul(nn_context* c, const nn_mul_job* jobs, uint64_t count) {
  if (!c || !jobs || !count) return NN_ERR_INVALID;
  std::vector<u64> na(count), nb(count);
  std::vector<int> sq(count);
  for (u64 j = 0; j < count; ++j) {
    na[j] = jobs[j].n_a;
    nb[j] = jobs[j].n_b;
    sq[j] = jobs[j].d_a == jobs[j].d_b && na[j] == nb[j];
  }
  nn_batch* B = nullptr;
  nn_status st = nn_batch_create(c, na.data(), nb.data(), sq.data(), count, &B);
  if (st != NN_OK) return st;
  st = nn_batch_run(c, B, jobs);
  batch_release(c, B);
  return st;
}

nn_context* nn_default_context(void) {
  static nn_context* ctx = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    int dev = 0;
    cudaGetDevice(&dev);
    if (nn_context_create(dev, 0, &ctx) != NN_OK) ctx = nullptr;
  }
  return ctx;
}

}  // extern "C"

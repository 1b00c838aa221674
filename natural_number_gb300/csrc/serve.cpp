// serve.cpp — a request server with continuous batching over one GPU.
//
// Clients submit multiply and divide requests on host memory.  A scheduler
// thread admits requests in arrival order while their estimated device
// footprint fits the HBM budget; every pass of its loop uploads the newly
// admitted products' operands and launches them as one batch (nn_batch_launch,
// the persistent work-queue kernel) on the next of several streams, so a batch
// formed from later arrivals runs while earlier batches are still on the
// device.  Completed batches are found through events; their results are
// copied back, their memory and budget released, and more requests admitted.
// Divisions (Newton reciprocal + block division, host-orchestrated) run on
// worker threads that each own a context and stream, so they overlap with the
// batches too.  Operands stay resident on the device from admission to
// completion; the twiddle tables stay resident for the server's lifetime.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <bit>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/natural_gb300.h"
#include "../../include/natural_gb300.hpp"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id = 0;
  int kind = 0;  // 0 multiply, 1 divide
  const uint64_t *a = nullptr, *b = nullptr;
  uint64_t na = 0, nb = 0;
  uint64_t *out = nullptr, *q = nullptr, *r = nullptr;
  uint64_t bytes = 0;  // admission charge
  double t_submit = 0, t_admit = 0, t_done = 0;
  int state = 0;  // 0 waiting, 1 admitted, 2 done
  nn_status status = NN_OK;
  uint64_t out_n = 0, q_n = 0, r_n = 0;
  uint64_t *d_in = nullptr, *d_out = nullptr;  // d_in: a, then b from an even offset
  uint64_t* stage = nullptr;                  // page-locked: a|b on the way in, the product on the way out
  uint64_t stage_bytes = 0;
};

// Offset of b in a product request's input buffers (16-byte aligned).
uint64_t b_offset(const Request* R) { return (R->na + 1) & ~1ull; }

// Page-locked staging for a request's transfers, from the recycled host pool
// in power-of-two sizes (so that blocks are reused across request sizes).
uint64_t stage_size(uint64_t bytes) { return std::bit_ceil(std::max<uint64_t>(bytes, 64 << 10)); }

void release_buffers(Request* R, cudaStream_t st) {
  if (R->d_in) cudaFreeAsync(R->d_in, st);
  if (R->d_out) cudaFreeAsync(R->d_out, st);
  if (R->stage) nn_host_free(R->stage, R->stage_bytes);
  R->d_in = R->d_out = R->stage = nullptr;
}

struct InFlight {
  std::vector<Request*> reqs;
  nn_batch* batch = nullptr;
  cudaEvent_t done = nullptr;
  int stream = 0;
};

int scale_of(uint64_t n1, uint64_t n2) { return 64 - __builtin_clzll(n1 + n2 - 2 ? n1 + n2 - 2 : 1); }

// Estimated device bytes while a request is in flight.
uint64_t footprint(int kind, uint64_t na, uint64_t nb) {
  const uint64_t L = 1ull << scale_of(na, nb);
  if (kind == 0) return 16 * (na + nb) + (std::min(na, nb) >= 256 ? 48 * L : 0) + 4096;
  // division: shifted operands, reciprocal, cached transforms of the divisor and reciprocal
  return 64 * (na + nb) + 144 * L + 4096;
}

}  // namespace

struct nn_server {
  int device = 0;
  uint64_t budget = 0;
  std::atomic<uint64_t> in_use{0};
  uint64_t peak = 0;
  nn_context* ctx = nullptr;
  std::vector<cudaStream_t> streams;
  std::vector<nn_context*> div_ctx;
  std::vector<cudaStream_t> div_streams;  // the division contexts' low-priority streams
  std::mutex mu;
  std::condition_variable cv, done_cv, div_cv;
  std::deque<Request*> waiting;
  std::deque<Request*> div_queue;
  std::vector<InFlight> inflight;
  std::vector<Request*> ready;  // admitted products waiting for a free stream (scheduler thread)
  std::map<uint64_t, Request*> all;
  uint64_t next_id = 1;
  bool stop = false;
  std::thread sched;
  std::vector<std::thread> workers;
  Clock::time_point t0 = Clock::now();
  uint64_t batches = 0, max_overlap = 0, max_batch = 0;
  std::atomic<int> div_running{0};
  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void finish(nn_server* S, Request* R, nn_status st) {
  R->status = st;
  R->t_done = S->now();
  R->state = 2;
  S->in_use -= R->bytes;
}

// Launches every admitted, unlaunched multiply as one batch, on a stream
// with no batch in flight.
void launch_products(nn_server* S, std::vector<Request*>& fresh) {
  if (fresh.empty()) return;
  int k = 0;
  for (; k < (int)S->streams.size(); ++k) {
    bool busy = false;
    for (const InFlight& f : S->inflight) busy |= f.stream == k;
    if (!busy) break;
  }
  if (k == (int)S->streams.size()) k = 0;  // not reached: the caller checks for a free stream
  cudaStream_t st = S->streams[k];
  nn_context_set_stream(S->ctx, st);
  std::vector<nn_mul_job> jobs;
  std::vector<Request*> ok;
  for (Request* R : fresh) {
    // The client's (pageable) operands go through page-locked staging, filled
    // on all host cores, so the link copies run at full speed and the
    // scheduler thread is not held up by a driver-staged copy.
    const uint64_t ob = b_offset(R), n_in = ob + R->nb, n_out = R->na + R->nb;
    R->stage_bytes = stage_size(std::max(n_in, n_out) * 8);
    R->stage = static_cast<uint64_t*>(nn_host_alloc(R->stage_bytes));
    cudaError_t e = R->stage ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&R->d_in, n_in * 8, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&R->d_out, n_out * 8, st);
    if (e == cudaSuccess) {
      nn_host_copy(R->stage, R->a, R->na);
      nn_host_copy(R->stage + ob, R->b, R->nb);
      e = cudaMemcpyAsync(R->d_in, R->stage, n_in * 8, cudaMemcpyHostToDevice, st);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      release_buffers(R, st);
      std::lock_guard<std::mutex> lk(S->mu);
      finish(S, R, e == cudaErrorMemoryAllocation ? NN_ERR_OOM : NN_ERR_CUDA);
      S->done_cv.notify_all();
      continue;
    }
    jobs.push_back(nn_mul_job{R->d_in, R->na, R->d_in + ob, R->nb, R->d_out});
    ok.push_back(R);
  }
  if (ok.empty()) return;
  std::vector<uint64_t> na(ok.size()), nb(ok.size());
  for (size_t j = 0; j < ok.size(); ++j) {
    na[j] = ok[j]->na;
    nb[j] = ok[j]->nb;
  }
  InFlight f;
  nn_status bs = nn_batch_create(S->ctx, na.data(), nb.data(), nullptr, ok.size(), &f.batch);
  if (bs == NN_OK) bs = nn_batch_launch(S->ctx, f.batch, jobs.data());
  if (bs == NN_OK)  // the products come back into the staging behind the batch, on its stream
    for (Request* R : ok)
      if (cudaMemcpyAsync(R->stage, R->d_out, (R->na + R->nb) * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) {
        cudaGetLastError();
        R->status = NN_ERR_CUDA;
      }
  f.reqs = ok;
  f.stream = k;
  cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
  cudaEventRecord(f.done, st);
  if (bs != NN_OK)
    for (Request* R : ok) R->status = bs;
  S->inflight.push_back(f);
  std::lock_guard<std::mutex> lk(S->mu);
  S->batches += 1;
  S->max_batch = std::max<uint64_t>(S->max_batch, ok.size());
  S->max_overlap = std::max<uint64_t>(S->max_overlap, S->inflight.size());
}

// Retires batches whose completion event has fired (scheduler thread only;
// request states change under the lock, where waiters read them).
bool retire(nn_server* S) {
  bool any = false;
  for (size_t i = 0; i < S->inflight.size();) {
    InFlight& f = S->inflight[i];
    if (cudaEventQuery(f.done) != cudaSuccess) {
      ++i;
      continue;
    }
    cudaStream_t st = S->streams[f.stream];
    for (Request* R : f.reqs) {
      // the batch and its copies are complete: the product is in the staging
      uint64_t n = R->na + R->nb;
      if (R->status == NN_OK) {
        nn_host_copy(R->out, R->stage, n);
        while (n > 1 && R->out[n - 1] == 0) --n;
      }
      R->out_n = n;
      release_buffers(R, st);
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      for (Request* R : f.reqs) finish(S, R, R->status);
    }
    cudaEventDestroy(f.done);
    if (f.batch) nn_batch_destroy(S->ctx, f.batch);
    S->inflight.erase(S->inflight.begin() + i);
    any = true;
  }
  return any;
}

// Continuous batching: products admitted while every stream has a batch in
// flight wait, and go out together in the next batch when one retires; so
// under load the batches grow rather than the number of small launches.
void scheduler(nn_server* S) {
  cudaSetDevice(S->device);
  while (true) {
    std::vector<Request*>& fresh = S->ready;
    bool quit = false;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      // admit in arrival order while the budget allows (a lone request always fits)
      while (!S->waiting.empty()) {
        Request* R = S->waiting.front();
        if (S->budget && S->in_use + R->bytes > S->budget && (S->in_use > 0 || !S->inflight.empty())) break;
        S->waiting.pop_front();
        S->in_use += R->bytes;
        S->peak = std::max<uint64_t>(S->peak, S->in_use);
        R->state = 1;
        R->t_admit = S->now();
        if (R->kind == 0) {
          fresh.push_back(R);
        } else {
          S->div_queue.push_back(R);
          S->div_cv.notify_one();
        }
      }
      quit = S->stop && S->waiting.empty() && S->inflight.empty() && S->div_queue.empty() && S->div_running == 0 &&
             fresh.empty();
    }
    if (quit) break;
    // no lock: only this thread touches the ready and in-flight lists and the context
    bool launched = false;
    if (!fresh.empty() && S->inflight.size() < S->streams.size()) {
      launch_products(S, fresh);
      fresh.clear();
      launched = true;
    }
    const bool retired = retire(S);
    if (retired) S->done_cv.notify_all();
    if (!launched && !retired) {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv.wait_for(lk, std::chrono::microseconds(S->inflight.empty() ? 2000 : 50));
    }
  }
}

// Divisions whose divisor has at least this many limbs run with every step on
// the GPU (nn_divmod_host); shorter ones take natural::_div on the host.
constexpr uint64_t kDeviceDivLimbs = 1024;

uint64_t trimmed(const uint64_t* x, uint64_t n) {
  while (n > 1 && x[n - 1] == 0) --n;
  return n;
}

void div_worker(nn_server* S, int w) {
  cudaSetDevice(S->device);
  nn_context* c = S->div_ctx[w];
  while (true) {
    Request* R = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->div_cv.wait(lk, [&] { return S->stop || !S->div_queue.empty(); });
      if (S->div_queue.empty()) {
        if (S->stop) break;
        continue;
      }
      R = S->div_queue.front();
      S->div_queue.pop_front();
      S->div_running += 1;
    }
    nn_status st = NN_OK;
    uint64_t na = R->na, nb = R->nb;
    while (na > 1 && R->a[na - 1] == 0) --na;
    while (nb > 1 && R->b[nb - 1] == 0) --nb;
    if (nb >= kDeviceDivLimbs && na >= nb) {
      // long divisors: every step on the GPU (nn_divmod_host); normalised results
      st = nn_divmod_host(c, R->q, R->r, R->a, na, R->b, nb);
      if (st == NN_OK) {
        R->q_n = trimmed(R->q, na - nb + 1);
        R->r_n = trimmed(R->r, nb);
      }
    } else {
      uint64_t *q = nullptr, *r = nullptr, qn = 0, rn = 0;
      st = nn_div_host(c, R->a, R->na, R->b, R->nb, &q, &qn, &r, &rn);
      if (st == NN_OK) {
        std::memcpy(R->q, q, 8 * qn);
        std::memcpy(R->r, r, 8 * rn);
        R->q_n = qn;
        R->r_n = rn;
      }
      nn_free(q);
      nn_free(r);
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      finish(S, R, st);
      S->div_running -= 1;
    }
    S->cv.notify_all();
    S->done_cv.notify_all();
  }
}

nn_status submit(nn_server* S, Request* R, uint64_t* ticket) {
  R->bytes = footprint(R->kind, R->na, R->nb);
  if (S->budget && R->bytes > S->budget) {
    delete R;
    return NN_ERR_BUDGET;
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) {
      delete R;
      return NN_ERR_INVALID;
    }
    R->id = S->next_id++;
    R->t_submit = S->now();
    S->all[R->id] = R;
    S->waiting.push_back(R);
    *ticket = R->id;
  }
  S->cv.notify_all();
  return NN_OK;
}

}  // namespace

extern "C" {

nn_status nn_server_create(int device, uint64_t hbm_budget, int streams, int div_workers, nn_server** out) {
  if (!out) return NN_ERR_INVALID;
  *out = nullptr;
  nn_server* S = new nn_server;
  S->device = device;
  S->budget = hbm_budget;
  nn_status st = nn_context_create(device, 0, &S->ctx);
  if (st != NN_OK) {
    delete S;
    return st;
  }
  // Every product stays inside its batch's kernel: batches run on several
  // streams at once, and a product run on its own (the batch_solo_scale
  // route) would use the context's one carry-scan scratch from each of them.
  nn_context_set_tunable(S->ctx, "batch_solo_scale", 0);
  // Product batches run on high-priority streams and divisions (long chains
  // of dependent kernels on the worker contexts) on low-priority ones, so a
  // batch that arrives while a division runs gets the SMs as they free up.
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  streams = std::max(1, std::min(streams, 16));
  for (int i = 0; i < streams; ++i) {
    cudaStream_t s;
    cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, greatest);
    S->streams.push_back(s);
  }
  div_workers = std::max(1, std::min(div_workers, 8));
  for (int i = 0; i < div_workers; ++i) {
    nn_context* c = nullptr;
    st = nn_context_create(device, 0, &c);
    if (st != NN_OK) break;
    cudaStream_t low = nullptr;
    cudaStreamCreateWithPriority(&low, cudaStreamNonBlocking, least);
    nn_context_set_stream(c, low);
    S->div_streams.push_back(low);
    S->div_ctx.push_back(c);
  }
  if (st != NN_OK) {
    for (nn_context* c : S->div_ctx) nn_context_destroy(c);
    for (cudaStream_t s : S->div_streams) cudaStreamDestroy(s);
    for (cudaStream_t s : S->streams) cudaStreamDestroy(s);
    nn_context_destroy(S->ctx);
    delete S;
    return st;
  }
  S->sched = std::thread(scheduler, S);
  for (int i = 0; i < div_workers; ++i) S->workers.emplace_back(div_worker, S, i);
  *out = S;
  return NN_OK;
}

nn_status nn_server_submit_mul(nn_server* S, const uint64_t* a, uint64_t na, const uint64_t* b, uint64_t nb,
                               uint64_t* out, uint64_t* ticket) {
  if (!S || !a || !b || !out || !na || !nb || !ticket) return NN_ERR_INVALID;
  Request* R = new Request;
  R->kind = 0;
  R->a = a;
  R->b = b;
  R->na = na;
  R->nb = nb;
  R->out = out;
  return submit(S, R, ticket);
}

nn_status nn_server_submit_div(nn_server* S, const uint64_t* a, uint64_t na, const uint64_t* b, uint64_t nb,
                               uint64_t* q, uint64_t* r, uint64_t* ticket) {
  if (!S || !a || !b || !q || !r || !na || !nb || !ticket) return NN_ERR_INVALID;
  Request* R = new Request;
  R->kind = 1;
  R->a = a;
  R->b = b;
  R->na = na;
  R->nb = nb;
  R->q = q;
  R->r = r;
  return submit(S, R, ticket);
}

nn_status nn_server_wait(nn_server* S, uint64_t ticket, double timeout_s, nn_request_info* info) {
  if (!S) return NN_ERR_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->all.find(ticket);
  if (it == S->all.end()) return NN_ERR_INVALID;
  Request* R = it->second;
  const bool ok = S->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return R->state == 2; });
  if (!ok) return NN_ERR_TIMEOUT;
  if (info) {
    info->status = R->status;
    info->out_n = R->kind == 0 ? R->out_n : R->q_n;
    info->r_n = R->r_n;
    info->t_submit = R->t_submit;
    info->t_admit = R->t_admit;
    info->t_done = R->t_done;
  }
  nn_status st = R->status;
  S->all.erase(it);
  delete R;
  return st;
}

nn_status nn_server_get_stats(nn_server* S, nn_server_stats* out) {
  if (!S || !out) return NN_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  out->in_flight_bytes = S->in_use;
  out->peak_bytes = S->peak;
  out->waiting = S->waiting.size();
  out->batches = S->batches;
  out->max_concurrent_batches = S->max_overlap;
  out->max_batch_jobs = S->max_batch;
  return NN_OK;
}

double nn_server_clock(nn_server* S) { return S ? S->now() : 0.0; }

nn_status nn_server_destroy(nn_server* S) {
  if (!S) return NN_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv.notify_all();
  S->div_cv.notify_all();
  if (S->sched.joinable()) S->sched.join();
  {
    std::lock_guard<std::mutex> lk(S->mu);
  }
  S->div_cv.notify_all();
  for (auto& t : S->workers) t.join();
  for (auto& kv : S->all) delete kv.second;
  for (cudaStream_t s : S->streams) cudaStreamSynchronize(s);
  nn_context_use_own_stream(S->ctx);  // the context must not keep a handle to a stream destroyed below
  for (cudaStream_t s : S->streams) cudaStreamDestroy(s);
  for (nn_context* c : S->div_ctx) nn_context_destroy(c);  // waits on its stream, then drops it
  for (cudaStream_t s : S->div_streams) cudaStreamDestroy(s);
  nn_context_destroy(S->ctx);
  delete S;
  return NN_OK;
}

}  // extern "C"

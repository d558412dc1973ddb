// Serving loop: continuous batching of idfact / psvdfact requests on one
// device (lra_server_*), and the batched idfact built on it.
//
// A server owns `slots` workers, each a host thread with its own context
// (CUDA stream and workspace arena).  Requests wait in arrival order and are
// admitted as soon as a slot is free and their estimated device memory fits
// the HBM budget beside the requests already running; admitted requests run
// concurrently on the slots' streams, so the work of different requests
// overlaps on the device.  Admission is first come, first served: a request
// that does not fit holds back the ones behind it, so no request starves.
//
// Every request runs as a fresh library call: the in-library generator
// restarts from the request's own seed and nothing else of a slot's state
// reaches the arithmetic, so a result is the same whichever slot runs it and
// whatever runs beside it.

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <string>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.hpp"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Req {
  uint64_t ticket = 0;
  lra_request r{};
  int64_t est = 0;
  Clock::time_point t_submit, t_start, t_done;
  bool done = false;
  int status = LRA_OK;
  int slot = -1;
  lra_id* id = nullptr;
  lra_psvd* psvd = nullptr;
  std::string error;
};

// device memory a request may hold at its peak: the input when it comes from
// the host, the BF16 digit planes of the mixed path, the sketch at its
// largest order, the factors and the post-processing workspace
int64_t estimate_bytes(const lra_request& r) {
  const int64_t e = r.dtype == LRA_F64 ? 8 : 4;
  const int64_t m = std::max<int64_t>(r.m, 1), n = std::max<int64_t>(r.n, 1);
  const int64_t mn = m * n;
  const int64_t k = std::min(m, n);
  int64_t b = 4 * mn * e;                          // input copy, digit planes (1.5x in F64)
  b += 2 * std::min<int64_t>(2 * k + 8, k) * std::max(m, n) * e;  // sketches
  b += 6 * k * std::max(m, n) * e;                 // factors and post-processing
  return b + ((int64_t)64 << 20);
}

}  // namespace

struct lra_server {
  int device = 0;
  int nslots = 0;
  int64_t budget = 0;
  std::mutex mu;
  std::condition_variable cv_work;  // workers: a request may be admissible
  std::condition_variable cv_done;  // pollers: a request finished
  std::deque<Req*> queue;
  std::unordered_map<uint64_t, Req*> all;
  uint64_t next_ticket = 1;
  int64_t in_use = 0;
  int64_t running = 0;
  int64_t submitted = 0, completed = 0, rejected = 0;
  std::vector<double> latencies;
  Clock::time_point t_first{}, t_last{};
  bool have_first = false;
  bool stop = false;
  std::vector<lra_ctx*> ctxs;
  std::vector<std::thread> workers;

  void work(int slot) {
    lra_ctx* ctx = ctxs[slot];
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      cv_work.wait(lk, [&] { return stop || (!queue.empty() && in_use + queue.front()->est <= budget); });
      if (stop && queue.empty()) return;
      if (queue.empty() || in_use + queue.front()->est > budget) continue;
      Req* q = queue.front();
      queue.pop_front();
      in_use += q->est;
      ++running;
      // the pivoted QR's launches take this request's share of the SMs, so
      // that the requests in flight factor side by side (a column's
      // arithmetic does not depend on the CTA count: the same bits)
      const int share = std::max(16, ctx->num_sms / (int)std::max<int64_t>(running, 1));
      q->slot = slot;
      q->t_start = Clock::now();
      lk.unlock();
      ctx->tuning.qr_sms = share;
      ctx->rng_counter = 0;  // each request starts its own stream of draws
      const lra_request& r = q->r;
      int st;
      if (r.kind == LRA_REQ_IDFACT)
        st = lra_idfact(ctx, r.dtype, r.trans ? r.trans : 'n', r.m, r.n, r.A, r.lda, &r.opts, r.rand, &q->id);
      else
        st = lra_psvdfact(ctx, r.dtype, r.m, r.n, r.A, r.lda, &r.opts, r.rand, 0, &q->psvd);
      // a slot keeps at most its share of the budget cached between requests
      if ((int64_t)ctx->arena.capacity() > budget / std::max(nslots, 1)) ctx->arena.free_all(ctx->stream);
      const Clock::time_point t = Clock::now();
      lk.lock();
      q->status = st;
      if (st != LRA_OK) q->error = lra_last_error(ctx);
      q->t_done = t;
      q->done = true;
      in_use -= q->est;
      --running;
      ++completed;
      latencies.push_back(ms_between(q->t_submit, t));
      t_last = t;
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }
};

extern "C" {

int lra_server_create(int device, int slots, int64_t hbm_budget_bytes, lra_server** out) {
  if (!out) return LRA_EINVAL;
  *out = nullptr;
  if (slots < 1 || slots > 64 || hbm_budget_bytes <= 0) return LRA_EINVAL;
  lra_server* s = new (std::nothrow) lra_server();
  if (!s) return LRA_ENOMEM;
  s->device = device;
  s->nslots = slots;
  s->budget = hbm_budget_bytes;
  for (int i = 0; i < slots; ++i) {
    lra_ctx* c = nullptr;
    const int st = lra_ctx_create(device, &c);
    if (st != LRA_OK) {
      for (lra_ctx* x : s->ctxs) lra_ctx_destroy(x);
      delete s;
      return st;
    }
    s->ctxs.push_back(c);
  }
  try {
    for (int i = 0; i < slots; ++i) s->workers.emplace_back([s, i] { s->work(i); });
  } catch (...) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    for (lra_ctx* x : s->ctxs) lra_ctx_destroy(x);
    delete s;
    return LRA_ENOMEM;
  }
  *out = s;
  return LRA_OK;
}

int lra_server_submit(lra_server* s, const lra_request* req, uint64_t* ticket) {
  if (!s || !req || !ticket) return LRA_EINVAL;
  if (req->kind != LRA_REQ_IDFACT && req->kind != LRA_REQ_PSVDFACT) return LRA_EINVAL;
  if (req->dtype == LRA_C32 || req->dtype == LRA_C64) return LRA_ENOTSUP;  // complex types: single calls
  if (req->dtype != LRA_F32 && req->dtype != LRA_F64) return LRA_EINVAL;
  if (req->m < 0 || req->n < 0 || !req->A) return LRA_EDIM;
  Req* q = new (std::nothrow) Req();
  if (!q) return LRA_ENOMEM;
  q->r = *req;
  q->est = estimate_bytes(*req);
  q->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (q->est > s->budget) {
    ++s->rejected;
    delete q;
    return LRA_ENOMEM;
  }
  if (!s->have_first) {
    s->t_first = q->t_submit;
    s->have_first = true;
  }
  q->ticket = s->next_ticket++;
  s->all[q->ticket] = q;
  s->queue.push_back(q);
  ++s->submitted;
  *ticket = q->ticket;
  s->cv_work.notify_all();
  return LRA_OK;
}

int lra_server_poll(lra_server* s, uint64_t ticket, int64_t wait_ms, lra_result* out) {
  if (!s || !out) return LRA_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(ticket);
  if (it == s->all.end()) return LRA_EINVAL;
  Req* q = it->second;
  if (!q->done && wait_ms != 0) {
    if (wait_ms < 0)
      s->cv_done.wait(lk, [&] { return q->done; });
    else
      s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return q->done; });
  }
  if (!q->done) return LRA_EBUSY;
  out->kind = q->r.kind;
  out->status = q->status;
  out->id = q->id;
  out->psvd = q->psvd;
  out->queue_ms = ms_between(q->t_submit, q->t_start);
  out->run_ms = ms_between(q->t_start, q->t_done);
  out->total_ms = ms_between(q->t_submit, q->t_done);
  out->slot = q->slot;
  std::memset(out->error, 0, sizeof out->error);
  std::strncpy(out->error, q->error.c_str(), sizeof out->error - 1);
  s->all.erase(it);
  delete q;
  return LRA_OK;
}

int lra_server_get_stats(lra_server* s, lra_server_stats* out) {
  if (!s || !out) return LRA_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = lra_server_stats{};
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->rejected = s->rejected;
  out->in_flight = s->running;
  out->queued = (int64_t)s->queue.size();
  out->hbm_budget = s->budget;
  out->hbm_in_use = s->in_use;
  if (!s->latencies.empty()) {
    std::vector<double> v = s->latencies;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
      const double x = p * (double)(v.size() - 1);
      const size_t i = (size_t)x;
      const double f = x - (double)i;
      return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
    };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / (double)v.size();
    const double span = ms_between(s->t_first, s->t_last);
    out->matrices_per_s = span > 0 ? 1e3 * (double)s->completed / span : 0;
  }
  return LRA_OK;
}

void lra_server_destroy(lra_server* s) {
  if (!s) return;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    // queued requests that never started are dropped; running ones finish
    for (Req* q : s->queue) {
      s->all.erase(q->ticket);
      delete q;
    }
    s->queue.clear();
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  for (auto& kv : s->all) {
    lra_id_free(kv.second->id);
    lra_psvd_free(kv.second->psvd);
    delete kv.second;
  }
  for (lra_ctx* c : s->ctxs) lra_ctx_destroy(c);
  delete s;
}

// idfact of many independent matrices: spread over `count`-bounded worker
// contexts of a private server, so that the matrices' work overlaps on the
// device (each result identical to a single lra_idfact call on it)
int lra_idfact_batched(lra_ctx* ctx, int dtype, int64_t count, const lra_matdesc* mats, const lra_opts* opts,
                       const lra_rand* rand, lra_id** outs) {
  if (!ctx || !mats || !outs || count < 0 || !opts) return LRA_EINVAL;
  for (int64_t i = 0; i < count; ++i) outs[i] = nullptr;
  if (count == 0) return LRA_OK;
  // Float64 on the mixed path: grouped launches, a CTA per matrix
  const int g = lra::try_idfact_batched_grouped(ctx, dtype, count, mats, opts, rand, outs);
  if (g >= 0) return g;
  size_t free_b = 0, total_b = 0;
  cudaSetDevice(ctx->device);
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    return LRA_ECUDA;
  }
  const int slots = (int)std::min<int64_t>(count, 8);
  lra_server* s = nullptr;
  int st = lra_server_create(ctx->device, slots, (int64_t)(0.8 * (double)free_b), &s);
  if (st != LRA_OK) return st;
  std::vector<uint64_t> tickets((size_t)count, 0);
  for (int64_t i = 0; i < count && st == LRA_OK; ++i) {
    lra_request r{};
    r.kind = LRA_REQ_IDFACT;
    r.dtype = dtype;
    r.trans = 'n';
    r.m = mats[i].m;
    r.n = mats[i].n;
    r.lda = mats[i].lda;
    r.A = mats[i].A;
    r.opts = *opts;
    r.rand = rand ? rand + i : nullptr;
    st = lra_server_submit(s, &r, &tickets[i]);
  }
  int first_err = st;
  for (int64_t i = 0; i < count; ++i) {
    if (!tickets[i]) continue;
    lra_result res{};
    if (lra_server_poll(s, tickets[i], -1, &res) != LRA_OK) continue;
    outs[i] = res.id;
    if (res.status != LRA_OK && first_err == LRA_OK) first_err = res.status;
  }
  lra_server_destroy(s);
  if (first_err != LRA_OK) {
    for (int64_t i = 0; i < count; ++i) {
      lra_id_free(outs[i]);
      outs[i] = nullptr;
    }
    ctx->last_error = "a matrix of the batch failed";
  }
  return first_err;
}

}  // extern "C"

// Continuous-batching request loop for elliptic solves and shallow-water ensemble members on one GPU
// (self_serve_*).  No counterpart in the reference, whose drivers run one model at a time.
//
// A worker thread owns every CUDA call.  Callers submit requests from any thread (submit / poll / cancel / result /
// stats touch only the request table, under a mutex); the worker admits queued requests in arrival order while
// their device footprint fits the HBM budget and keeps them on the GPU until they finish:
//   * Helmholtz solves join one batched slot pool (self_cgbatch_*): every tick advances all of them together --
//     outer FP64 residual step, the outer decision and graph_k inner PCG iterations, all on the device -- and one
//     synchronisation per tick reads the slot states; finished solves leave their slot and free their memory.
//   * Shallow-water members each get a handle on one of a few extra streams and advance in chunks of RK3 steps
//     enqueued asynchronously, so their kernels overlap the batched solves.
// Each result depends only on its own request (per-problem arithmetic and reduction order do not depend on the
// other problems in the pool; each member runs on its own handle), so it is bit-identical alone and in the mix.
// The caller keeps every array a request's descriptor points to, and its source / initial state, alive until the
// request is done, failed or cancelled: the worker reads them when it admits the request.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.hpp"

namespace {

struct Req {
  long long ticket = 0;
  int kind = SELF_SERVE_SOLVE;
  int state = SELF_SERVE_QUEUED;
  int status = SELF_OK;
  bool cancel = false;
  double t_submit = 0, t_admit = -1, t_done = -1;
  long long bytes = 0;
  // solve
  self_cg2d_desc cg{};
  const double* source = nullptr;
  int slot = -1;
  // shallow-water member
  self_dg2d_desc dg{};
  const double* q0 = nullptr;
  int steps = 0, steps_done = 0, stream = -1;
  self_dg2d* h = nullptr;
  // outcome
  self_solve_report report{};
  std::vector<double> result;
};

using Clock = std::chrono::steady_clock;

}  // namespace

struct self_serve {
  self_ctx* ctx = nullptr;
  std::vector<self_ctx*> sw_ctx;
  self_cgbatch* pool = nullptr;
  self_serve_opts o{};
  self_solve_opts so{};
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv;
  std::thread worker;
  bool stop = false;
  long long next_ticket = 1;
  std::map<long long, std::unique_ptr<Req>> reqs;
  std::deque<Req*> queue;  // submitted, not admitted (arrival order)
  std::vector<Req*> running;
  long long used = 0;
  long long n_submitted = 0, n_admitted = 0, n_finished = 0, n_cancelled = 0, n_failed = 0;
  std::vector<double> latencies;  // finished requests, seconds
  double first_submit = -1, last_done = -1;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

long long footprint(const Req& r) {
  if (r.kind == SELF_SERVE_SOLVE) {
    long long b = 0;
    self_cgbatch_footprint(&r.cg, &b);
    return b;
  }
  const long long nn = (long long)(r.dg.N + 1) * (r.dg.N + 1);
  // state, RK register, metrics, aux, traces and staging (FP32 form; FP64 twice that)
  const long long per = nn * r.dg.nEq * 4 * 40 / 3;
  return r.dg.nEl * per * (r.dg.precision == SELF_PREC_FP32 ? 1 : 2) + 4096;
}

void finish(self_serve* s, Req* r, int state, int status) {
  r->state = state;
  r->status = status;
  r->t_done = s->now();
  if (r->bytes) s->used -= r->bytes;
  r->bytes = 0;
  if (state == SELF_SERVE_DONE) {
    ++s->n_finished;
    s->latencies.push_back(r->t_done - r->t_submit);
    s->last_done = r->t_done;
  } else if (state == SELF_SERVE_CANCELLED) {
    ++s->n_cancelled;
  } else {
    ++s->n_failed;
  }
}

// Admission of one request on the device (worker thread, without the lock).
int admit(self_serve* s, Req* r) {
  int rc;
  if (r->kind == SELF_SERVE_SOLVE) {
    rc = self_cgbatch_add(s->pool, &r->cg, r->source, &r->slot);
  } else {
    const int k = (int)(s->n_admitted % (long long)s->sw_ctx.size());
    r->stream = k;
    rc = self_dg2d_create(s->sw_ctx[k], &r->dg, &r->h);
    if (!rc) rc = self_dg2d_set_state(r->h, r->q0);
  }
  return rc;
}

void worker_loop(self_serve* s) {
  cudaSetDevice(s->ctx->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    // cancellations of queued requests
    for (auto it = s->queue.begin(); it != s->queue.end();) {
      if ((*it)->cancel) {
        finish(s, *it, SELF_SERVE_CANCELLED, SELF_OK);
        it = s->queue.erase(it);
        s->cv.notify_all();
      } else {
        ++it;
      }
    }
    // admission in arrival order while the footprint fits (and the concurrency cap allows)
    while (!s->queue.empty()) {
      Req* r = s->queue.front();
      const long long fp = footprint(*r);
      if (s->used + fp > (long long)s->o.hbm_budget_bytes && !s->running.empty()) break;
      if (s->o.max_active > 0 && (int)s->running.size() >= s->o.max_active) break;
      s->queue.pop_front();
      r->bytes = fp;
      s->used += fp;
      r->state = SELF_SERVE_RUNNING;
      r->t_admit = s->now();
      ++s->n_admitted;
      s->running.push_back(r);  // listed before the lock is released: a waiter always finds it in one list
      lk.unlock();
      const int rc = admit(s, r);
      lk.lock();
      if (rc) {
        if (r->h) self_dg2d_destroy(r->h);
        r->h = nullptr;
        s->running.erase(std::find(s->running.begin(), s->running.end(), r));
        finish(s, r, SELF_SERVE_FAILED, rc);
        s->cv.notify_all();
      }
    }
    if (s->running.empty()) {
      if (s->stop) break;
      s->cv.wait_for(lk, std::chrono::milliseconds(1));
      continue;
    }
    std::vector<Req*> run = s->running;
    lk.unlock();
    // shallow-water members: next chunk on idle streams
    bool any_solve = false;
    for (Req* r : run) {
      if (r->kind == SELF_SERVE_SOLVE) {
        any_solve = true;
        continue;
      }
      if (r->steps_done < r->steps && !r->cancel && r->status == SELF_OK &&
          self_ctx_query(s->sw_ctx[r->stream]) == 1) {
        const int k = std::min(std::max(1, s->o.sw_chunk), r->steps - r->steps_done);
        const int rc = self_dg2d_rk3_async(r->h, 0.0, k);
        if (rc == SELF_OK) r->steps_done += k;
        else r->status = rc;
      }
    }
    // batched solves: one tick (outer step, device-side decision, inner iterations), one synchronisation
    int nfin = 0, tick_rc = SELF_OK;
    if (any_solve) tick_rc = self_cgbatch_step(s->pool, &s->so, &nfin);
    // completions
    std::vector<std::pair<Req*, int>> done;  // request, final state
    for (Req* r : run) {
      if (r->kind == SELF_SERVE_SOLVE) {
        if (tick_rc) {
          r->status = tick_rc;
          self_cgbatch_remove(s->pool, r->slot);
          done.push_back({r, SELF_SERVE_FAILED});
          continue;
        }
        int fin = 0;
        self_solve_report rep{};
        self_cgbatch_report(s->pool, r->slot, &rep, &fin);
        if (fin || r->cancel) {
          r->report = rep;
          if (fin) {
            if (!(rep.rel_residual < s->so.tolerance)) r->report.ioerr = -1;
            long long nl = 0;
            self_cgbatch_problem_size(s->pool, r->slot, &nl);
            r->result.resize((size_t)nl);
            self_cgbatch_get_solution(s->pool, r->slot, r->result.data());
          }
          self_cgbatch_remove(s->pool, r->slot);
          done.push_back({r, fin ? SELF_SERVE_DONE : SELF_SERVE_CANCELLED});
        }
      } else {
        if (self_ctx_query(s->sw_ctx[r->stream]) != 1) continue;  // a chunk is still in flight
        int state = -1;
        if (r->status != SELF_OK) {
          state = SELF_SERVE_FAILED;
        } else if (r->cancel) {
          state = SELF_SERVE_CANCELLED;
        } else if (r->steps_done >= r->steps) {
          int rc = self_dg2d_rk3(r->h, 0.0, 0);  // synchronise and report a time-out recorded in flight
          r->result.resize((size_t)(r->dg.N + 1) * (r->dg.N + 1) * r->dg.nEq * r->dg.nEl);
          if (!rc) rc = self_dg2d_get_state(r->h, r->result.data());
          r->status = rc;
          state = rc ? SELF_SERVE_FAILED : SELF_SERVE_DONE;
        }
        if (state >= 0) {
          self_dg2d_destroy(r->h);
          r->h = nullptr;
          done.push_back({r, state});
        }
      }
    }
    lk.lock();
    for (auto& d : done) {
      finish(s, d.first, d.second, d.first->status);
      s->running.erase(std::find(s->running.begin(), s->running.end(), d.first));
    }
    if (!done.empty()) s->cv.notify_all();
    // only shallow-water members in flight and none finished: wait briefly instead of polling the streams hot
    if (!any_solve && done.empty()) s->cv.wait_for(lk, std::chrono::microseconds(200));
  }
}

Req* find(self_serve* s, long long ticket) {
  auto it = s->reqs.find(ticket);
  return it == s->reqs.end() ? nullptr : it->second.get();
}

int submit(self_serve* s, std::unique_ptr<Req> r, long long* ticket) {
  std::lock_guard<std::mutex> lk(s->mu);
  r->ticket = s->next_ticket++;
  r->t_submit = s->now();
  if (s->first_submit < 0) s->first_submit = r->t_submit;
  ++s->n_submitted;
  *ticket = r->ticket;
  s->queue.push_back(r.get());
  s->reqs[r->ticket] = std::move(r);
  s->cv.notify_all();
  return SELF_OK;
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int self_serve_create(self_ctx* ctx, const self_serve_opts* o, self_serve** out) {
  if (!ctx || !o || !out || !(o->hbm_budget_bytes > 0) || !(o->tolerance > 0))
    return selfgpu::set_error(ctx, SELF_ERR_INVALID, "self_serve_create: bad options");
  if (o->precision != SELF_PREC_FP32 && o->precision != SELF_PREC_FP64)
    return selfgpu::set_error(ctx, SELF_ERR_INVALID, "self_serve_create: precision %d", o->precision);
  std::unique_ptr<self_serve> s(new self_serve());
  s->ctx = ctx;
  s->o = *o;
  if (s->o.sw_streams < 1) s->o.sw_streams = 4;
  if (s->o.sw_chunk < 1) s->o.sw_chunk = 10;
  s->so.method = SELF_SOLVE_PCG_JACOBI;
  s->so.precision = o->precision;
  s->so.maxIters = o->maxIters > 0 ? o->maxIters : 100000;
  s->so.tolerance = o->tolerance;
  s->so.inner_tolerance = o->inner_tolerance > 0 ? o->inner_tolerance : 1e-4;
  s->so.max_outer = o->max_outer > 0 ? o->max_outer : 30;
  int rc = self_cgbatch_create(ctx, 0, nullptr, &s->pool);
  if (rc) return rc;
  for (int k = 0; k < s->o.sw_streams; ++k) {
    self_ctx* c = nullptr;
    if ((rc = self_ctx_create(ctx->device, &c))) {
      for (self_ctx* x : s->sw_ctx) self_ctx_destroy(x);
      self_cgbatch_destroy(s->pool);
      return rc;
    }
    s->sw_ctx.push_back(c);
  }
  s->t0 = Clock::now();
  self_serve* raw = s.get();
  s->worker = std::thread(worker_loop, raw);
  *out = s.release();
  return SELF_OK;
}

int self_serve_destroy(self_serve* s) {
  if (!s) return SELF_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (Req* r : s->queue) r->cancel = true;
    for (Req* r : s->running) r->cancel = true;
    s->cv.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  for (auto& kv : s->reqs)
    if (kv.second->h) self_dg2d_destroy(kv.second->h);
  self_cgbatch_destroy(s->pool);
  for (self_ctx* c : s->sw_ctx) self_ctx_destroy(c);
  delete s;
  return SELF_OK;
}

int self_serve_submit_solve(self_serve* s, const self_cg2d_desc* d, const double* source, long long* ticket) {
  if (!s || !d || !source || !ticket) return SELF_ERR_INVALID;
  if (d->op != 0) return selfgpu::set_error(nullptr, SELF_ERR_UNSUPPORTED, "serving: Helmholtz operator (op 0) only");
  std::unique_ptr<Req> r(new Req());
  r->kind = SELF_SERVE_SOLVE;
  r->cg = *d;
  r->source = source;
  return submit(s, std::move(r), ticket);
}

int self_serve_submit_sw(self_serve* s, const self_dg2d_desc* d, const double* q0, int steps, long long* ticket) {
  if (!s || !d || !q0 || steps < 1 || !ticket) return SELF_ERR_INVALID;
  std::unique_ptr<Req> r(new Req());
  r->kind = SELF_SERVE_SW;
  r->dg = *d;
  r->q0 = q0;
  r->steps = steps;
  return submit(s, std::move(r), ticket);
}

int self_serve_poll(self_serve* s, long long ticket, self_serve_info* info) {
  if (!s || !info) return SELF_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  Req* r = find(s, ticket);
  if (!r) return selfgpu::set_error(nullptr, SELF_ERR_INVALID, "serving: unknown ticket %lld", ticket);
  info->state = r->state;
  info->kind = r->kind;
  info->status = r->status;
  info->steps_done = r->steps_done;
  info->submit_s = r->t_submit;
  info->admit_s = r->t_admit;
  info->done_s = r->t_done;
  info->report = r->report;
  return SELF_OK;
}

int self_serve_result(self_serve* s, long long ticket, double* out, size_t n) {
  if (!s || !out) return SELF_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  Req* r = find(s, ticket);
  if (!r || r->state != SELF_SERVE_DONE)
    return selfgpu::set_error(nullptr, SELF_ERR_INVALID, "serving: ticket %lld has no result", ticket);
  if (n != r->result.size())
    return selfgpu::set_error(nullptr, SELF_ERR_INVALID, "serving: the result has %zu values, %zu asked",
                              r->result.size(), n);
  std::copy(r->result.begin(), r->result.end(), out);
  return SELF_OK;
}

int self_serve_release(self_serve* s, long long ticket) {
  if (!s) return SELF_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  Req* r = find(s, ticket);
  if (!r) return SELF_ERR_INVALID;
  if (r->state == SELF_SERVE_QUEUED || r->state == SELF_SERVE_RUNNING)
    return selfgpu::set_error(nullptr, SELF_ERR_INVALID, "serving: ticket %lld is still active", ticket);
  s->reqs.erase(ticket);
  return SELF_OK;
}

int self_serve_cancel(self_serve* s, long long ticket) {
  if (!s) return SELF_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  Req* r = find(s, ticket);
  if (!r) return SELF_ERR_INVALID;
  if (r->state == SELF_SERVE_QUEUED || r->state == SELF_SERVE_RUNNING) r->cancel = true;
  s->cv.notify_all();
  return SELF_OK;
}

int self_serve_wait(self_serve* s, double timeout_s) {
  if (!s) return SELF_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
  while (!s->queue.empty() || !s->running.empty()) {
    if (s->cv.wait_until(lk, until) == std::cv_status::timeout && (!s->queue.empty() || !s->running.empty()))
      return selfgpu::set_error(nullptr, SELF_ERR_TIMEOUT, "serving: requests still active after %g s", timeout_s);
  }
  return SELF_OK;
}

int self_serve_stats(self_serve* s, self_serve_statistics* st) {
  if (!s || !st) return SELF_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  st->submitted = s->n_submitted;
  st->admitted = s->n_admitted;
  st->finished = s->n_finished;
  st->cancelled = s->n_cancelled;
  st->failed = s->n_failed;
  st->queued = (long long)s->queue.size();
  st->running = (long long)s->running.size();
  st->bytes_in_use = s->used;
  st->p50_ms = 1e3 * percentile(s->latencies, 0.50);
  st->p99_ms = 1e3 * percentile(s->latencies, 0.99);
  double mean = 0;
  for (double v : s->latencies) mean += v;
  st->mean_ms = s->latencies.empty() ? 0.0 : 1e3 * mean / (double)s->latencies.size();
  const double span = (s->last_done >= 0 && s->first_submit >= 0) ? s->last_done - s->first_submit : 0.0;
  st->throughput_per_s = span > 0 ? (double)s->n_finished / span : 0.0;
  st->elapsed_s = s->now();
  return SELF_OK;
}

}  // extern "C"

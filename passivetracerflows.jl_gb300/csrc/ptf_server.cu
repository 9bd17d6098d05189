// Request server: continuous batching of tracer solves on one GPU.
//
// A worker thread owns a ptf_batch (square 2D solves, stepped together by
// the batched stage kernels) and a set of single-solve handles (3D
// requests).  Each loop iteration it (1) admits queued requests in arrival
// order wherever the device-memory budget and the bucket slots allow,
// (2) advances every admitted solve by one chunk of steps -- the chunk ends
// early when the nearest solve finishes, so finished solves leave promptly --
// and (3) retires finished solves: reads the tracer back, frees the slot and
// records the latency (submission to result).  Requests that arrive while
// others run are admitted between chunks, so their work overlaps on the GPU
// with the solves already in flight.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ptf.h"
#include "ptf_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

enum ReqState { REQ_QUEUED = 0, REQ_ACTIVE = 1, REQ_DONE = 2, REQ_FAILED = 3 };

struct Request {
  ptf_solve_desc desc;
  std::vector<double> c0, u, v, w;
  std::vector<double> result;
  Clock::time_point t_submit, t_done;
  int state = REQ_QUEUED;
  int64_t batch_id = -1;        // 2D: id in the batch
  ptf_handle* handle = nullptr; // 3D: its own handle
  int64_t done_steps = 0;
  double mass0 = 0.0, mass_end = 0.0;  // sum of c0 and of the result (compensated FP64)
  std::string error;
};

// Compensated (Neumaier) sum of n doubles.
double mass_of(const double* x, size_t n) {
  double s = 0.0, c = 0.0;
  for (size_t i = 0; i < n; ++i) {
    const double t = s + x[i];
    c += std::fabs(s) >= std::fabs(x[i]) ? (s - t) + x[i] : (x[i] - t) + s;
    s = t;
  }
  return s + c;
}

}  // namespace

struct ptf_server {
  ptf_server_config cfg;
  ptf_batch* batch = nullptr;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv, cv_done;
  std::map<int64_t, Request> reqs;
  std::deque<int64_t> queue;
  std::vector<int64_t> active;
  int64_t next_id = 1;
  bool stop = false;
  int64_t handle_bytes = 0;
  // statistics
  std::vector<double> latencies;
  double grid_point_steps = 0.0;
  bool started = false;
  Clock::time_point t_first, t_last;
  int64_t completed = 0, failed = 0;
  double mass_drift_max = 0.0;
  double admit_s = 0.0, chunk_s = 0.0;  // worker time in admission, and in stepping chunks to their completion
  int64_t chunks = 0;
  int inject_fail_in = -1;  // host-side fault injection: fail the chunk this many chunks ahead (-1: none)
  std::string error;
};

namespace {

double points(const ptf_solve_desc& d) {
  const double n = d.n;
  return d.dim == 3 ? n * n * n : n * n;
}

size_t handle_estimate(const ptf_server* s, const ptf_solve_desc& d) {
  const size_t n = d.n, pitch = ((n / 2 + 1) + 7) / 8 * 8;
  const size_t e = s->cfg.precision == PTF_FP32 ? 8 : 16, r = e / 2;
  // 7 spectral fields, 8 with an FP32 handle's compensated state
  return (s->cfg.precision == PTF_FP32 ? 8 : 7) * n * n * pitch * e + 5 * n * n * n * r + n * n * n * 8;
}

bool try_admit(ptf_server* s, int64_t id, Request& q) {
  if (q.desc.dim == 3) {
    const size_t need = handle_estimate(s, q.desc);
    int64_t used = 0;
    ptf_batch_info(s->batch, &used, nullptr, nullptr);
    if (s->cfg.memory_budget > 0 && (int64_t)(used + s->handle_bytes + need) > s->cfg.memory_budget) return false;
    ptf_config c;
    ptf_config_default(&c, 3);
    c.nx = c.ny = c.nz = q.desc.n;
    c.Lx = c.Ly = c.Lz = q.desc.L;
    c.kappa = q.desc.kappa; c.eta = q.desc.eta; c.iota = q.desc.eta;
    c.kappah = q.desc.kappah; c.nkappah = q.desc.nkappah;
    c.dt = q.desc.dt;
    c.stepper = PTF_RK4;
    c.precision = s->cfg.precision;
    ptf_handle* h = nullptr;
    if (ptf_create(&c, &h) != PTF_OK) { q.state = REQ_FAILED; q.error = ptf_last_error(nullptr); return true; }
    if (ptf_set_flow_arrays(h, q.u.data(), q.v.data(), q.w.data(), PTF_HOST) != PTF_OK ||
        ptf_set_c(h, q.c0.data(), PTF_HOST) != PTF_OK) {
      q.state = REQ_FAILED; q.error = ptf_last_error(h); ptf_destroy(h); return true;
    }
    int64_t hb = 0;
    ptf_device_bytes(h, &hb);
    s->handle_bytes += hb;
    q.handle = h;
  } else {
    if (!ptf_batch_can_admit(s->batch, &q.desc)) return false;
    int64_t bid = -1;
    const double* u = q.desc.flow_kind == PTF_FLOW_ARRAYS ? q.u.data() : nullptr;
    const double* v = q.desc.flow_kind == PTF_FLOW_ARRAYS ? q.v.data() : nullptr;
    const int rc = ptf_batch_add(s->batch, &q.desc, q.c0.data(), u, v, &bid);
    if (rc == PTF_ERR_MEMORY) return false;  // no room now: retry when solves retire
    if (rc != PTF_OK) { q.state = REQ_FAILED; q.error = ptf_batch_last_error(s->batch); return true; }
    q.batch_id = bid;
  }
  q.state = REQ_ACTIVE;
  q.c0.clear(); q.c0.shrink_to_fit();
  s->active.push_back(id);
  return true;
}

void finish(ptf_server* s, int64_t id, Request& q) {
  const size_t np = (size_t)points(q.desc);
  q.result.resize(np);
  int rc;
  if (q.handle) {
    rc = ptf_get_c(q.handle, q.result.data(), PTF_HOST);
    if (rc) q.error = ptf_last_error(q.handle);
    int64_t hb = 0;
    ptf_device_bytes(q.handle, &hb);
    s->handle_bytes -= hb;
    ptf_destroy(q.handle);
    q.handle = nullptr;
  } else {
    rc = ptf_batch_get_c(s->batch, q.batch_id, q.result.data());
    if (rc) q.error = ptf_batch_last_error(s->batch);
    ptf_batch_remove(s->batch, q.batch_id);
  }
  q.t_done = Clock::now();
  q.state = rc ? REQ_FAILED : REQ_DONE;
  q.u.clear(); q.v.clear(); q.w.clear();
  if (!rc) {
    q.mass_end = mass_of(q.result.data(), q.result.size());
    if (q.mass0 != 0.0) s->mass_drift_max = std::max(s->mass_drift_max, std::fabs(q.mass_end / q.mass0 - 1.0));
    s->latencies.push_back(std::chrono::duration<double>(q.t_done - q.t_submit).count());
    s->grid_point_steps += points(q.desc) * (double)q.desc.nsteps;
    s->completed++;
  } else {
    s->failed++;
  }
  s->t_last = q.t_done;
  (void)id;
}

// A request that failed in flight: release its slot or handle so that the
// memory budget and the batch's slots come back.
void drop_failed(ptf_server* s, Request& q, const std::string& why) {
  if (q.handle) {
    int64_t hb = 0;
    ptf_device_bytes(q.handle, &hb);
    s->handle_bytes -= hb;
    ptf_destroy(q.handle);
    q.handle = nullptr;
  } else if (q.batch_id >= 0) {
    ptf_batch_remove(s->batch, q.batch_id);  // deactivates the slot; a sticky CUDA error leaves nothing to free
    q.batch_id = -1;
  }
  q.state = REQ_FAILED;
  q.error = why;
  q.t_done = Clock::now();
  q.u.clear(); q.v.clear(); q.w.clear();
  s->failed++;
  s->t_last = q.t_done;
}

void worker_loop(ptf_server* s) {
  for (;;) {
    std::vector<ptf_handle*> handles;
    std::vector<int64_t> hsteps;  // each handle's steps this chunk (to its own count)
    int64_t chunk = 0;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // admission in arrival order, first fit
      const Clock::time_point ta = Clock::now();
      for (auto it = s->queue.begin(); it != s->queue.end();) {
        Request& q = s->reqs[*it];
        if (try_admit(s, *it, q)) {
          if (q.state == REQ_FAILED) { q.t_done = Clock::now(); s->failed++; s->cv_done.notify_all(); }
          it = s->queue.erase(it);
        } else {
          ++it;
        }
      }
      s->admit_s += std::chrono::duration<double>(Clock::now() - ta).count();
      if (s->active.empty()) {
        if (s->stop && s->queue.empty()) return;
        s->cv.wait_for(lk, std::chrono::milliseconds(2));
        continue;
      }
      // The batch retires each slot at its own step count on the device
      // (its clock kernel), so a chunk need not stop at the soonest
      // finishing request: 2D requests take the full chunk, 3D handles
      // step exactly to their own counts.
      chunk = s->cfg.chunk_steps > 0 ? s->cfg.chunk_steps : 50;
      for (int64_t id : s->active) {
        const Request& q = s->reqs[id];
        if (q.handle) {
          handles.push_back(q.handle);
          hsteps.push_back(std::min<int64_t>(chunk, q.desc.nsteps - q.done_steps));
        }
      }
    }
    const Clock::time_point tc = Clock::now();
    bool injected = false;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->inject_fail_in == 0) injected = true;
      if (s->inject_fail_in >= 0) s->inject_fail_in--;
    }
    // GPU work outside the lock (only this thread touches the batch and handles)
    std::string why;
    int rc = injected ? PTF_ERR_CUDA : ptf_batch_step(s->batch, chunk);
    if (injected) why = "batched step: injected failure (test)";
    else if (rc) why = std::string("batched step: ") + ptf_batch_last_error(s->batch);
    // 3D handles: enqueue every handle's chunk (their streams run beside the
    // batch's), then wait for each
    for (size_t k = 0; k < handles.size(); ++k) {
      if (rc) break;
      rc = ptf_step(handles[k], hsteps[k]);
      if (rc) why = std::string("3D step: ") + ptf_last_error(handles[k]);
    }
    for (ptf_handle* h : handles) {
      if (rc) break;
      rc = ptf_synchronize(h);
      if (rc) why = std::string("3D step: ") + ptf_last_error(h);
    }
    if (!rc) {
      rc = ptf_batch_synchronize(s->batch);
      if (rc) why = std::string("batched step: ") + ptf_batch_last_error(s->batch);
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->chunk_s += std::chrono::duration<double>(Clock::now() - tc).count();
      s->chunks++;
      if (rc) s->error = why;
      std::vector<int64_t> still;
      for (int64_t id : s->active) {
        Request& q = s->reqs[id];
        if (rc) { drop_failed(s, q, why); continue; }
        q.done_steps = std::min<int64_t>(q.desc.nsteps, q.done_steps + chunk);
        if (q.done_steps >= q.desc.nsteps) finish(s, id, q);
        else still.push_back(id);
      }
      s->active.swap(still);
      s->cv_done.notify_all();
    }
  }
}

int sfail(ptf_server* s, int code, const std::string& m) {
  if (s) s->error = m; else ptf::set_global_error(m);
  return code;
}

}  // namespace

extern "C" {

void ptf_server_config_default(ptf_server_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->precision = PTF_FP32;
  c->memory_budget = 0;
  c->chunk_steps = 50;
  c->slots_per_bucket = 0;
}

int ptf_server_create(const ptf_server_config* cfg, ptf_server** out) {
  if (!cfg || !out) return sfail(nullptr, PTF_ERR_ARG, "ptf_server_create: null argument");
  *out = nullptr;
  if (cfg->chunk_steps < 0 || cfg->memory_budget < 0) return sfail(nullptr, PTF_ERR_ARG, "invalid server limits");
  ptf_batch_config bc;
  ptf_batch_config_default(&bc);
  bc.precision = cfg->precision;
  bc.memory_budget = cfg->memory_budget;
  bc.slots_per_bucket = cfg->slots_per_bucket;
  ptf_batch* b = nullptr;
  const int rc = ptf_batch_create(&bc, &b);
  if (rc) return rc;
  ptf_server* s = new ptf_server();
  s->cfg = *cfg;
  s->batch = b;
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return PTF_OK;
}

void ptf_server_destroy(ptf_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->queue.clear();
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto& kv : s->reqs)
    if (kv.second.handle) ptf_destroy(kv.second.handle);
  ptf_batch_destroy(s->batch);
  delete s;
}

const char* ptf_server_last_error(const ptf_server* s) { return s ? s->error.c_str() : ptf_last_error(nullptr); }

int ptf_server_submit(ptf_server* s, const ptf_solve_desc* d, const double* c0, const double* u, const double* v,
                      const double* w, int64_t* id) {
  if (!s) return sfail(nullptr, PTF_ERR_ARG, "null server");
  if (!d || !c0) return sfail(s, PTF_ERR_ARG, "solve description and initial condition are required");
  const bool three = d->dim == 3;
  if (d->dim != 2 && d->dim != 3) return sfail(s, PTF_ERR_ARG, "dim must be 2 or 3");
  if (three && (d->flow_kind != PTF_FLOW_ARRAYS || !u || !v || !w))
    return sfail(s, PTF_ERR_ARG, "3D requests take flow arrays u, v, w");
  if (!three && d->flow_kind == PTF_FLOW_ARRAYS && (!u || !v)) return sfail(s, PTF_ERR_ARG, "u and v are required");
  if (!three && !(d->n == 64 || d->n == 128 || d->n == 256 || d->n == 512 || d->n == 1024))
    return sfail(s, PTF_ERR_ARG, "2D requests take n in {64, 128, 256, 512, 1024}");
  if (three && !(d->n >= 16 && d->n <= 256 && (d->n & (d->n - 1)) == 0))
    return sfail(s, PTF_ERR_ARG, "3D requests take n a power of two in [16, 256]");
  if (!(d->dt > 0) || d->nsteps < 1) return sfail(s, PTF_ERR_ARG, "dt must be positive and nsteps >= 1");
  if (s->cfg.memory_budget > 0) {
    // what this request needs in an otherwise empty server: it never fits if that exceeds the budget
    const int64_t need = three ? (int64_t)handle_estimate(s, *d) + ptf::batch_fixed_bytes(s->batch)
                               : ptf::batch_fixed_bytes(s->batch) + ptf::batch_slot_bytes(s->batch, d->n);
    if (need > s->cfg.memory_budget)
      return sfail(s, PTF_ERR_MEMORY, "request needs " + std::to_string(need) + " device bytes, more than the server's memory budget of " +
                                          std::to_string(s->cfg.memory_budget));
  }
  Request q;
  q.desc = *d;
  const size_t np = (size_t)points(*d);
  q.c0.assign(c0, c0 + np);
  q.mass0 = mass_of(c0, np);
  if (d->flow_kind == PTF_FLOW_ARRAYS) {
    q.u.assign(u, u + np);
    q.v.assign(v, v + np);
    if (three) q.w.assign(w, w + np);
  }
  q.t_submit = Clock::now();
  int64_t rid;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return sfail(s, PTF_ERR_STATE, "server is stopping");
    rid = s->next_id++;
    if (!s->started) { s->started = true; s->t_first = q.t_submit; }
    s->reqs.emplace(rid, std::move(q));
    s->queue.push_back(rid);
  }
  s->cv.notify_all();
  if (id) *id = rid;
  return PTF_OK;
}

int ptf_server_poll(ptf_server* s, int64_t id, int32_t* state, double* c) {
  if (!s) return sfail(nullptr, PTF_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return sfail(s, PTF_ERR_ARG, "unknown request id");
  Request& q = it->second;
  if (state) *state = q.state;
  if (q.state == REQ_DONE && c) {
    std::copy(q.result.begin(), q.result.end(), c);
  }
  if (q.state == REQ_FAILED) return sfail(s, PTF_ERR_CUDA, q.error);
  return PTF_OK;
}

int ptf_server_release(ptf_server* s, int64_t id) {
  if (!s) return sfail(nullptr, PTF_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return sfail(s, PTF_ERR_ARG, "unknown request id");
  if (it->second.state != REQ_DONE && it->second.state != REQ_FAILED) return sfail(s, PTF_ERR_STATE, "request not finished");
  s->reqs.erase(it);
  return PTF_OK;
}

int ptf_server_wait_all(ptf_server* s, double timeout_s) {
  if (!s) return sfail(nullptr, PTF_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
  while (!(s->queue.empty() && s->active.empty())) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) return sfail(s, PTF_ERR_STATE, "timed out");
  }
  return s->failed ? sfail(s, PTF_ERR_CUDA, "some requests failed: " + s->error) : PTF_OK;
}

int ptf_server_get_stats(ptf_server* s, ptf_server_stats* out) {
  if (!s || !out) return sfail(nullptr, PTF_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->completed = s->completed;
  out->failed = s->failed;
  out->queued = (int64_t)s->queue.size();
  out->active = (int64_t)s->active.size();
  std::vector<double> l = s->latencies;
  std::sort(l.begin(), l.end());
  if (!l.empty()) {
    auto pct = [&](double p) {
      const double idx = p * (double)(l.size() - 1);
      const size_t lo = (size_t)idx;
      const size_t hi = std::min(lo + 1, l.size() - 1);
      return l[lo] + (idx - (double)lo) * (l[hi] - l[lo]);
    };
    out->p50_s = pct(0.50);
    out->p99_s = pct(0.99);
    double sum = 0;
    for (double x : l) sum += x;
    out->mean_s = sum / (double)l.size();
  }
  out->grid_point_steps = s->grid_point_steps;
  out->mass_drift_max_abs = s->mass_drift_max;
  out->admit_s = s->admit_s;
  out->chunk_s = s->chunk_s;
  out->chunks = s->chunks;
  int64_t live = 0;
  for (const auto& kv : s->reqs) if (kv.second.handle) ++live;
  out->handles = live;
  out->wall_s = s->started && s->completed ? std::chrono::duration<double>(s->t_last - s->t_first).count() : 0.0;
  int64_t bytes = 0, solves = 0;
  ptf_batch_info(s->batch, &bytes, &solves, nullptr);
  out->device_bytes = bytes + s->handle_bytes;
  out->batch_solves = solves;
  return PTF_OK;
}

int ptf_server_result_info(ptf_server* s, int64_t id, double* latency_s, double* mass0, double* mass_end) {
  if (!s) return sfail(nullptr, PTF_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return sfail(s, PTF_ERR_ARG, "unknown request id");
  const Request& q = it->second;
  if (q.state != REQ_DONE) return sfail(s, PTF_ERR_STATE, "request not done");
  if (latency_s) *latency_s = std::chrono::duration<double>(q.t_done - q.t_submit).count();
  if (mass0) *mass0 = q.mass0;
  if (mass_end) *mass_end = q.mass_end;
  return PTF_OK;
}

int ptf_server_inject_step_failure(ptf_server* s, int32_t chunks_from_now) {
  if (!s) return sfail(nullptr, PTF_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  s->inject_fail_in = chunks_from_now < 0 ? -1 : chunks_from_now;
  return PTF_OK;
}

}  // extern "C"

// server.cpp -- cmn_server_*: continuous batching of solve requests over
// one cmn_batch per size class, each class on its own stream and cadence.
// The worker thread is the only user of the batches; submitters touch the
// request table under the mutex only.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <system_error>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/cuminlp_gb300.h"
#include "handles.hpp"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b)
{
  return std::chrono::duration<double, std::milli>(b - a).count();
}

// nearest-rank percentile of an ascending sample
double percentile(const std::vector<double>& v, double q)
{
  if (v.empty()) return 0.0;
  size_t r = (size_t)std::ceil(q * (double)v.size());
  r = std::min(std::max<size_t>(r, 1), v.size());
  return v[r - 1];
}

bool same_shared(const cmn_solve_options& a, const cmn_solve_options& b)
{
  return a.precision == b.precision && a.bisection_budget == b.bisection_budget &&
         a.batch_parents == b.batch_parents && a.frontier_cap == b.frontier_cap &&
         a.sample_points == b.sample_points && a.sample_all == b.sample_all &&
         a.relative_width == b.relative_width && a.max_cycle_size == b.max_cycle_size &&
         a.enumerate_cap == b.enumerate_cap;
}

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2 };

struct Request {
  const cmn_problem* p = nullptr;
  cmn_solve_options o{};
  int64_t n_vars = 0, n_slots = 0;
  Clock::time_point t_submit, t_admit, t_done;
  int state = kQueued;
  int cls = -1;
  uint64_t slot = 0;
  cmn_status status = CMN_OK;
  std::string error;
  cmn_outcome out{};
  std::vector<double> point;
};

}  // namespace

struct cmn_server {
  cmn_server_config conf{};
  std::vector<cmn_batch*> batches;
  std::vector<uint64_t> slot_bytes;
  std::vector<uint64_t> occupied;
  std::vector<std::vector<uint64_t>> owner;  // class -> slot -> request id (~0: free)

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, Request> reqs;
  uint64_t next_id = 1;
  bool stop = false;
  cmn_status fatal = CMN_OK;
  std::string fatal_msg;
  std::thread worker;

  // statistics
  uint64_t submitted = 0, admitted = 0, completed = 0, converged = 0, boxes = 0, rounds = 0;
  uint64_t in_use = 0, peak = 0;
  bool any_submit = false;
  Clock::time_point t_first_submit, t_last_done;
  std::vector<double> latencies, queue_waits;

  ~cmn_server()
  {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    for (cmn_batch* b : batches) cmn_batch_destroy(b);
  }

  bool fits(const Request& r, int c) const
  {
    return r.n_vars <= conf.class_max_vars[c] && r.n_slots <= conf.class_max_program_slots[c];
  }

  uint64_t running_total() const
  {
    uint64_t t = 0;
    for (uint64_t o : occupied) t += o;
    return t;
  }

  void set_fatal(cmn_status st, const char* what)
  {
    fatal = st;
    fatal_msg = std::string(what) + ": " + cmn_last_error();
    for (auto& kv : reqs) {
      if (kv.second.state == kDone) continue;
      kv.second.state = kDone;
      kv.second.status = st;
      kv.second.error = fatal_msg;
    }
    queue.clear();
    cv_done.notify_all();
  }

  // First fit over the queue: a request takes a free slot of the smallest
  // class that holds it, while the admitted pools stay within the budget.
  void admit_locked()
  {
    for (auto it = queue.begin(); it != queue.end();) {
      Request& r = reqs[*it];
      int c = -1;
      for (int k = 0; k < conf.n_classes; ++k) {
        if (!fits(r, k) || occupied[k] >= conf.class_slots[k]) continue;
        if (conf.pool_budget_bytes && in_use + slot_bytes[k] > conf.pool_budget_bytes) continue;
        c = k;
        break;
      }
      if (c < 0) {
        ++it;
        continue;
      }
      uint64_t slot = 0;
      const cmn_status st = cmn_batch_add(batches[c], r.p, &r.o, &slot);
      if (st != CMN_OK) {
        r.state = kDone;
        r.status = st;
        r.error = cmn_last_error();
        r.t_done = Clock::now();
        cv_done.notify_all();
        it = queue.erase(it);
        continue;
      }
      r.state = kRunning;
      r.cls = c;
      r.slot = slot;
      r.t_admit = Clock::now();
      owner[c][slot] = *it;
      ++occupied[c];
      ++admitted;
      in_use += slot_bytes[c];
      peak = std::max(peak, in_use);
      queue_waits.push_back(ms_between(r.t_submit, r.t_admit));
      it = queue.erase(it);
    }
  }

  // Retires the stopped requests of class c (its state freshly pulled).
  void retire_class_locked(int c)
  {
    for (uint64_t k = 0; k < owner[c].size() && occupied[c]; ++k) {
      const uint64_t id = owner[c][k];
      if (id == ~0ULL) continue;
      int32_t done = 0;
      if (cmn_batch_poll(batches[c], k, &done) != CMN_OK || !done) continue;
      Request& r = reqs[id];
      r.point.assign((size_t)r.n_vars, 0.0);
      cmn_status st = cmn_batch_outcome(batches[c], k, &r.out, r.point.data());
      if (st == CMN_OK) st = cmn_batch_release(batches[c], k);
      if (st != CMN_OK) {
        set_fatal(st, "retiring a request");
        return;
      }
      r.t_done = Clock::now();
      r.out.elapsed_ms = ms_between(r.t_submit, r.t_done);
      r.state = kDone;
      owner[c][k] = ~0ULL;
      --occupied[c];
      in_use -= slot_bytes[c];
      ++completed;
      if (r.out.stop_reason == CMN_STOP_CONVERGED) ++converged;
      boxes += r.out.counters.bounded;
      latencies.push_back(r.out.elapsed_ms);
      t_last_done = r.t_done;
    }
    cv_done.notify_all();
  }

  // Each class runs on its own: as soon as a class's iterations finish, its
  // stopped requests retire, queued requests are admitted and the class
  // launches again, without waiting for the other classes.
  void run()
  {
    const uint64_t ipr = conf.iterations_per_round ? conf.iterations_per_round : 4;
    std::vector<int> inflight(conf.n_classes, 0);
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu);
        if (stop || fatal != CMN_OK) return;
        admit_locked();
        bool busy = false;
        for (int c = 0; c < conf.n_classes; ++c) busy = busy || inflight[c] || occupied[c] > 0;
        if (!busy) {
          cv_work.wait_for(lk, std::chrono::milliseconds(2), [&] { return stop || !queue.empty(); });
          continue;
        }
      }
      // only the worker changes `occupied`, so it reads it without the lock
      cmn_status st = CMN_OK;
      for (int c = 0; c < conf.n_classes && st == CMN_OK; ++c) {
        if (inflight[c] || occupied[c] == 0) continue;
        st = cmn_batch_launch(batches[c], ipr);
        inflight[c] = 1;
      }
      bool progressed = false;
      for (int c = 0; c < conf.n_classes && st == CMN_OK; ++c) {
        if (!inflight[c]) continue;
        int32_t idle = 0;
        st = cmn_batch_query(batches[c], &idle);
        if (st != CMN_OK || !idle) continue;
        st = cmn_batch_sync(batches[c], nullptr);
        if (st != CMN_OK) break;
        inflight[c] = 0;
        progressed = true;
        std::lock_guard<std::mutex> lk(mu);
        ++rounds;
        retire_class_locked(c);
        if (fatal != CMN_OK) return;
      }
      if (st != CMN_OK) {
        std::lock_guard<std::mutex> lk(mu);
        set_fatal(st, "running the classes");
        return;
      }
      if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
  }
};

extern "C" cmn_status cmn_server_create(const cmn_server_config* config, cmn_server** out)
{
  if (!config || !out) return cmn::set_error(CMN_INVALID_CONFIGURATION, "null argument");
  *out = nullptr;
  const cmn_server_config& cf = *config;
  if (cf.n_classes < 1 || cf.n_classes > CMN_SERVER_MAX_CLASSES)
    return cmn::set_error(CMN_INVALID_CONFIGURATION, "n_classes must be within [1, 8]");
  for (int c = 0; c < cf.n_classes; ++c) {
    if (cf.class_slots[c] < 1 || cf.class_max_vars[c] < 1)
      return cmn::set_error(CMN_INVALID_CONFIGURATION, "every class needs slots and max_vars >= 1");
    if (c && cf.class_max_vars[c] < cf.class_max_vars[c - 1])
      return cmn::set_error(CMN_INVALID_CONFIGURATION, "class_max_vars must be ascending");
  }
  try {
    cmn_server* s = new cmn_server();
    s->conf = cf;
    for (int c = 0; c < cf.n_classes; ++c) {
      cmn_batch_config bc{};
      bc.slots = cf.class_slots[c];
      bc.max_vars = cf.class_max_vars[c];
      bc.max_program_slots = cf.class_max_program_slots[c];
      bc.device = cf.device;
      bc.shared = cf.shared;
      cmn_batch* b = nullptr;
      const cmn_status st = cmn_batch_create(&bc, &b);
      if (st != CMN_OK) {
        delete s;
        return st;
      }
      s->batches.push_back(b);
      s->slot_bytes.push_back(cmn_batch_slot_bytes(b));
      s->occupied.push_back(0);
      s->owner.emplace_back(cf.class_slots[c], ~0ULL);
    }
    for (int c = 0; c < cf.n_classes; ++c)
      if (cf.pool_budget_bytes && s->slot_bytes[c] > cf.pool_budget_bytes) {
        delete s;
        return cmn::set_error(CMN_OVER_BUDGET, "one slot of class " + std::to_string(c) +
                                                   " exceeds pool_budget_bytes");
      }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return CMN_OK;
  } catch (const std::bad_alloc&) {
    return cmn::set_error(CMN_INTERNAL, "host allocation failed");
  } catch (const std::system_error&) {
    return cmn::set_error(CMN_INTERNAL, "could not start the worker thread");
  }
}

extern "C" void cmn_server_destroy(cmn_server* s) { delete s; }

extern "C" cmn_status cmn_server_submit(cmn_server* s, const cmn_problem* p, const cmn_solve_options* opts,
                                        uint64_t* request_id)
{
  if (!s || !p || !opts || !request_id) return cmn::set_error(CMN_INVALID_CONFIGURATION, "null argument");
  if (!same_shared(*opts, s->conf.shared))
    return cmn::set_error(CMN_INVALID_CONFIGURATION, "the request's shared options differ from the server's");
  cmn_problem_info info{};
  cmn_status st = cmn_problem_get_info(p, &info);
  if (st != CMN_OK) return st;
  try {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->fatal != CMN_OK) return cmn::set_error(s->fatal, s->fatal_msg);
    Request r;
    r.p = p;
    r.o = *opts;
    r.n_vars = info.n_vars;
    r.n_slots = info.program_slots;
    bool any = false;
    for (int c = 0; c < s->conf.n_classes; ++c) any = any || s->fits(r, c);
    if (!any)
      return cmn::set_error(CMN_INVALID_CONFIGURATION,
                            "no size class takes a problem with " + std::to_string(info.n_vars) + " variables and " +
                                std::to_string(info.program_slots) + " program slots");
    r.t_submit = Clock::now();
    if (!s->any_submit) {
      s->any_submit = true;
      s->t_first_submit = r.t_submit;
    }
    const uint64_t id = s->next_id++;
    s->reqs.emplace(id, std::move(r));
    s->queue.push_back(id);
    ++s->submitted;
    *request_id = id;
  } catch (const std::bad_alloc&) {
    return cmn::set_error(CMN_INTERNAL, "host allocation failed");
  }
  s->cv_work.notify_one();
  return CMN_OK;
}

static cmn_status copy_result(const Request& r, cmn_outcome* out, double* best_point)
{
  if (r.status != CMN_OK) return cmn::set_error(r.status, r.error);
  if (out) *out = r.out;
  if (best_point) std::memcpy(best_point, r.point.data(), sizeof(double) * r.point.size());
  return CMN_OK;
}

extern "C" cmn_status cmn_server_poll(cmn_server* s, uint64_t id, int32_t* done, cmn_outcome* out,
                                      double* best_point)
{
  if (!s || !done) return cmn::set_error(CMN_INVALID_CONFIGURATION, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return cmn::set_error(CMN_INVALID_CONFIGURATION, "unknown request");
  *done = it->second.state == kDone ? 1 : 0;
  return *done ? copy_result(it->second, out, best_point) : CMN_OK;
}

extern "C" cmn_status cmn_server_wait(cmn_server* s, uint64_t id, uint64_t timeout_ms, cmn_outcome* out,
                                      double* best_point)
{
  if (!s) return cmn::set_error(CMN_INVALID_CONFIGURATION, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return cmn::set_error(CMN_INVALID_CONFIGURATION, "unknown request");
  // Submits made while this thread waits may rehash the table, which
  // invalidates iterators but not references to the elements.
  const Request* r = &it->second;
  auto ready = [&] { return r->state == kDone; };
  if (timeout_ms == 0) {
    s->cv_done.wait(lk, ready);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    return cmn::set_error(CMN_TIMEOUT, "request still running after " + std::to_string(timeout_ms) + " ms");
  }
  return copy_result(*r, out, best_point);
}

extern "C" cmn_status cmn_server_stats_get(cmn_server* s, cmn_server_stats* out)
{
  if (!s || !out) return cmn::set_error(CMN_INVALID_CONFIGURATION, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof *out);
  out->submitted = s->submitted;
  out->admitted = s->admitted;
  out->completed = s->completed;
  out->queued = s->queue.size();
  out->running = s->running_total();
  out->converged = s->converged;
  out->boxes = s->boxes;
  out->rounds = s->rounds;
  out->pool_bytes_in_use = s->in_use;
  out->pool_bytes_peak = s->peak;
  out->pool_budget_bytes = s->conf.pool_budget_bytes;
  std::vector<double> lat = s->latencies, q = s->queue_waits;
  std::sort(lat.begin(), lat.end());
  std::sort(q.begin(), q.end());
  out->latency_p50_ms = percentile(lat, 0.50);
  out->latency_p99_ms = percentile(lat, 0.99);
  out->latency_max_ms = lat.empty() ? 0.0 : lat.back();
  double sum = 0;
  for (double x : lat) sum += x;
  out->latency_mean_ms = lat.empty() ? 0.0 : sum / (double)lat.size();
  out->queue_p50_ms = percentile(q, 0.50);
  out->queue_p99_ms = percentile(q, 0.99);
  out->wall_ms = s->completed ? ms_between(s->t_first_submit, s->t_last_done) : 0.0;
  out->boxes_per_s = out->wall_ms > 0 ? (double)s->boxes / (out->wall_ms * 1e-3) : 0.0;
  return CMN_OK;
}

// ev_serve.cu -- continuous-batching request loop.
//
// Requests (a circuit, a seed, a shot count) are admitted in arrival order
// as slots and HBM free up: a request needs 2^n x 16 (complex128) or 8
// (complex64) bytes of state, and the sum over admitted requests stays under
// the budget.  Admitted requests run concurrently, each on its own stream:
//   - requests of at most `batch_qubits` qubits (and at most 64 classical
//     bits) that are admitted together run together as one persistent
//     batched launch (ev_batch_run), mid-circuit measurements and classical
//     control included -- the same-stage work of many small requests in one
//     kernel;
//   - every other request runs through the device-resident run loop
//     (ev_state_run: mid-circuit measurements and classical control stay on
//     the GPU), then draws its shots (ev_sample).
// A worker thread drives each running unit, so work of different requests
// overlaps on the device; a request that arrives while others run is
// admitted as soon as a worker and memory are free.  The path a request
// takes depends only on the request (qubit count and op kinds), never on
// what else is in flight, and every path is deterministic, so a request's
// result is the same alone and in the mix.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "ev_internal.h"

struct ev_server;

namespace ev {
namespace {

using clk = std::chrono::steady_clock;

struct Request {
  uint64_t id;
  uint64_t nq, ncl;
  std::vector<ev_op> ops;
  std::vector<uint64_t> pool;
  uint64_t seed, shots;
  uint64_t* shots_out;
  size_t bytes;
  bool small;  // runs in batched launches
  clk::time_point t_submit, t_admit;
  bool cancelled = false;
};

double ms_between(clk::time_point a, clk::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace
}  // namespace ev

struct ev_server {
  ev_server_options opts{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<ev::Request*> pending;
  std::vector<ev_server_result> done;
  std::map<std::pair<uint64_t, int>, std::vector<ev_state*>> free_states;
  uint64_t next_id = 1;
  uint64_t reserved = 0;
  uint64_t budget = 0;
  bool stopping = false;
  bool paused = false;
  std::vector<std::thread> workers;
  ev_server_stats stats{};
  int device = 0;
};

namespace ev {
namespace {

ev_state* acquire_state(ev_server* s, uint64_t n, int dtype) {
  {
    std::lock_guard<std::mutex> lock(s->mu);
    auto& v = s->free_states[{n, dtype}];
    if (!v.empty()) {
      ev_state* st = v.back();
      v.pop_back();
      return st;
    }
  }
  ev_state* st = nullptr;
  if (ev_state_create(n, dtype, &st) != EV_OK) return nullptr;
  return st;
}

void release_state(ev_server* s, ev_state* st) {
  uint64_t n = 0;
  int32_t dt = 0;
  ev_state_num_qubits(st, &n);
  ev_state_dtype(st, &dt);
  std::lock_guard<std::mutex> lock(s->mu);
  s->free_states[{n, dt}].push_back(st);
}

ev_server_result make_result(const Request& r, int status, const uint8_t* classical) {
  ev_server_result out{};
  out.id = r.id;
  out.status = status;
  out.num_classical = int32_t(r.ncl);
  out.shots = r.shots;
  const auto now = clk::now();
  out.queue_ms = ms_between(r.t_submit, r.t_admit);
  out.latency_ms = ms_between(r.t_submit, now);
  if (classical)
    for (uint64_t j = 0; j < r.ncl && j < 64; ++j) out.classical[j] = classical[j];
  return out;
}

ev_circuit circuit_of(const Request& r) {
  ev_circuit c{};
  c.num_qubits = r.nq;
  c.num_classical = r.ncl;
  c.ops = r.ops.empty() ? nullptr : r.ops.data();
  c.nops = r.ops.size();
  c.ctrl_pool = r.pool.empty() ? nullptr : r.pool.data();
  c.pool_len = r.pool.size();
  return c;
}

// One request through the run loop and the sampler.
int run_single(ev_server* s, Request* r, std::vector<uint8_t>* classical) {
  ev_state* st = acquire_state(s, r->nq, s->opts.dtype);
  if (!st) return EV_ERR_OOM;
  ev_run_options o{};
  o.dtype = s->opts.dtype;
  o.mode = s->opts.mode;
  o.variant = s->opts.variant;
  // a fused arithmetic of the other amplitude type runs the tile pass instead
  if (o.mode == EV_MODE_FUSED && (o.variant == EV_FUSED_OZAKI || o.variant == EV_FUSED_OZAKI6) != (o.dtype == EV_C128))
    o.mode = EV_MODE_TILED;
  const ev_circuit c = circuit_of(*r);
  classical->assign(r->ncl ? r->ncl : 1, 0);
  int rc = ev_state_run(st, &c, r->seed, &o, classical->data());
  if (rc == EV_OK && r->shots) rc = ev_sample(st, r->seed, r->shots, r->shots_out);
  release_state(s, st);
  return rc;
}

void worker_loop(ev_server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    std::vector<Request*> unit;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      for (;;) {
        // drop cancelled requests at the head
        while (!s->pending.empty() && s->pending.front()->cancelled) {
          Request* r = s->pending.front();
          s->pending.pop_front();
          r->t_admit = clk::now();
          s->done.push_back(make_result(*r, EV_ERR_CANCELLED, nullptr));
          s->stats.cancelled++;
          delete r;
          s->cv_done.notify_all();
        }
        if (!s->pending.empty() && !s->paused) {
          Request* head = s->pending.front();
          if (head->bytes > s->budget) {  // can never fit
            s->pending.pop_front();
            head->t_admit = clk::now();
            s->done.push_back(make_result(*head, EV_ERR_ADMISSION, nullptr));
            s->stats.refused++;
            delete head;
            s->cv_done.notify_all();
            continue;
          }
          if (s->reserved + head->bytes <= s->budget) {
            // admit the head; small gate-only requests admitted together
            // with it join the same batched launch
            s->pending.pop_front();
            unit.push_back(head);
            s->reserved += head->bytes;
            if (head->small && s->opts.batch_small) {
              for (auto it = s->pending.begin(); it != s->pending.end() && unit.size() < 256;) {
                Request* r = *it;
                if (!r->cancelled && r->small && s->reserved + r->bytes <= s->budget) {
                  unit.push_back(r);
                  s->reserved += r->bytes;
                  it = s->pending.erase(it);
                } else {
                  ++it;
                }
              }
            }
            break;
          }
        }
        if (s->stopping && s->pending.empty()) return;
        s->cv_work.wait(lock);
      }
      const auto now = clk::now();
      for (Request* r : unit) r->t_admit = now;
      s->stats.admitted += unit.size();
      s->stats.running += unit.size();
    }
    // run the unit outside the lock
    std::vector<ev_server_result> results;
    if (unit.size() > 1 || (unit[0]->small && s->opts.batch_small)) {
      std::vector<ev_batch_circuit> items(unit.size());
      std::vector<std::vector<uint8_t>> classical(unit.size());
      for (size_t i = 0; i < unit.size(); ++i) {
        items[i] = ev_batch_circuit{};
        items[i].circuit = circuit_of(*unit[i]);
        items[i].seed = unit[i]->seed;
        items[i].run_seed = unit[i]->seed;  // as run_single: one seed per request
        items[i].shots = unit[i]->shots;
        items[i].shots_out = unit[i]->shots_out;
        classical[i].assign(unit[i]->ncl ? unit[i]->ncl : 1, 0);
        items[i].classical_out = classical[i].data();
      }
      ev_batch_options bo{};
      bo.dtype = s->opts.dtype;
      bo.tile_bits = s->opts.batch_qubits;
      bo.threads = 256;
      const int rc = ev_batch_run(items.data(), items.size(), &bo, nullptr);
      for (size_t i = 0; i < unit.size(); ++i)
        results.push_back(make_result(*unit[i], rc, rc == EV_OK ? classical[i].data() : nullptr));
      {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stats.batched_launches++;
        s->stats.batched_requests += unit.size();
      }
    } else {
      std::vector<uint8_t> classical;
      const int rc = run_single(s, unit[0], &classical);
      results.push_back(make_result(*unit[0], rc, classical.data()));
    }
    {
      std::lock_guard<std::mutex> lock(s->mu);
      for (size_t i = 0; i < unit.size(); ++i) {
        s->reserved -= unit[i]->bytes;
        s->done.push_back(results[i]);
        if (results[i].status == EV_OK) s->stats.completed++;
        else s->stats.failed++;
        delete unit[i];
      }
      s->stats.running -= unit.size();
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

}  // namespace
}  // namespace ev

using namespace ev;

extern "C" int ev_server_create(const ev_server_options* o, ev_server** out) {
  clear_error();
  if (!out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_server_create: null output");
  ev_server* s = new ev_server();
  if (o) s->opts = *o;
  if (s->opts.dtype != EV_C128 && s->opts.dtype != EV_C64) s->opts.dtype = EV_C64;
  if (s->opts.workers <= 0) s->opts.workers = 8;
  if (s->opts.batch_qubits <= 0) s->opts.batch_qubits = s->opts.dtype == EV_C64 ? 13 : 12;
  cudaGetDevice(&s->device);
  if (s->opts.hbm_budget == 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      cudaGetLastError();
      fr = 0;
    }
    s->budget = uint64_t(double(fr) * 0.8);
  } else {
    s->budget = s->opts.hbm_budget;
  }
  s->paused = s->opts.start_paused != 0;
  for (int w = 0; w < s->opts.workers; ++w) s->workers.emplace_back(worker_loop, s);
  *out = s;
  return EV_OK;
}

extern "C" int ev_server_submit(ev_server* s, const ev_circuit* c, uint64_t seed, uint64_t shots,
                                uint64_t* shots_out, uint64_t* id) {
  clear_error();
  if (!s || !c || !id) return fail(EV_ERR_INVALID_ARGUMENT, "ev_server_submit: null argument");
  if (shots && !shots_out) return fail(EV_ERR_INVALID_ARGUMENT, "ev_server_submit: shots without output");
  EV_TRY(ev_validate(c));
  if (c->num_qubits > 40) return fail(EV_ERR_ADMISSION, "request of %llu qubits can never fit", (unsigned long long)c->num_qubits);
  Request* r = new Request();
  r->nq = c->num_qubits;
  r->ncl = c->num_classical;
  r->ops.assign(c->ops, c->ops + c->nops);
  if (c->pool_len) r->pool.assign(c->ctrl_pool, c->ctrl_pool + c->pool_len);
  r->seed = seed;
  r->shots = shots;
  r->shots_out = shots_out;
  r->bytes = (size_t(1) << r->nq) * (s->opts.dtype == EV_C128 ? 16 : 8);
  r->small = r->nq >= 1 && int(r->nq) <= s->opts.batch_qubits && r->ncl <= 64;
  r->t_submit = clk::now();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    r->id = s->next_id++;
    *id = r->id;
    s->stats.submitted++;
    if (r->bytes > s->budget) {  // can never be admitted
      r->t_admit = r->t_submit;
      s->done.push_back(make_result(*r, EV_ERR_ADMISSION, nullptr));
      s->stats.refused++;
      delete r;
      s->cv_done.notify_all();
      return EV_OK;
    }
    s->pending.push_back(r);
  }
  s->cv_work.notify_one();
  return EV_OK;
}

extern "C" int ev_server_submit_qasm(ev_server* s, const char* src, uint64_t len, uint64_t seed,
                                     uint64_t shots, uint64_t* shots_out, uint64_t* id) {
  clear_error();
  if (!s || !id) return fail(EV_ERR_INVALID_ARGUMENT, "ev_server_submit_qasm: null argument");
  ev_program* prog = nullptr;
  EV_TRY(ev_qasm_parse(src, len, &prog, nullptr, nullptr));
  ev_circuit c;
  int rc = ev_program_circuit(prog, &c);
  if (rc == EV_OK) rc = ev_server_submit(s, &c, seed, shots, shots_out, id);  // copies the records
  ev_program_free(prog);
  return rc;
}

extern "C" int ev_server_cancel(ev_server* s, uint64_t id) {
  if (!s) return fail(EV_ERR_INVALID_ARGUMENT, "null server");
  std::lock_guard<std::mutex> lock(s->mu);
  for (Request* r : s->pending)
    if (r->id == id) {
      r->cancelled = true;
      s->cv_work.notify_all();
      return EV_OK;
    }
  return fail(EV_ERR_INVALID_ARGUMENT, "request %llu is not pending", (unsigned long long)id);
}

extern "C" int ev_server_poll(ev_server* s, ev_server_result* out, int32_t max, int32_t* count,
                              int32_t wait_ms) {
  if (!s || !count || (max > 0 && !out)) return fail(EV_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_lock<std::mutex> lock(s->mu);
  if (s->done.empty() && wait_ms > 0)
    s->cv_done.wait_for(lock, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty(); });
  const int32_t n = int32_t(std::min<size_t>(s->done.size(), size_t(std::max(0, max))));
  for (int32_t i = 0; i < n; ++i) out[i] = s->done[i];
  s->done.erase(s->done.begin(), s->done.begin() + n);
  *count = n;
  return EV_OK;
}

extern "C" int ev_server_resume(ev_server* s) {
  if (!s) return fail(EV_ERR_INVALID_ARGUMENT, "null server");
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->paused = false;
  }
  s->cv_work.notify_all();
  return EV_OK;
}

extern "C" int ev_server_stats_get(ev_server* s, ev_server_stats* out) {
  if (!s || !out) return fail(EV_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  *out = s->stats;
  out->reserved_bytes = s->reserved;
  out->budget_bytes = s->budget;
  out->pending = s->pending.size();
  return EV_OK;
}

extern "C" int ev_server_destroy(ev_server* s) {
  if (!s) return EV_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stopping = true;
    s->paused = false;
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  for (auto& kv : s->free_states)
    for (ev_state* st : kv.second) ev_state_destroy(st);
  delete s;
  return EV_OK;
}

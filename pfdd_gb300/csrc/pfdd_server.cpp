// pfdd_server.cpp -- serving form (include/pfdd_serve.h).
//
// Solves that share grid, slip systems and constants form a class.  A class
// owns one batched context (its replica slots hold its solves, B(k) is built
// once), one worker thread and that context's CUDA stream.  The worker loop:
//
//   admit pending solves into free slots (upload xi, mark the slot active)
//   -> run one chunk of steps for every active slot (one pfdd_step call)
//   -> hand back gamma of the chunk, retire slots that reached their steps.
//
// Chunks end exactly where the next active solve finishes, and are otherwise
// sized to about kChunkTargetS of wall time, so queued solves are admitted
// quickly whatever the class's step time.  Classes are created when the
// device-memory budget admits them and released when idle (at once when other
// solves wait for memory).  Streams of classes of smaller solves get a more
// urgent CUDA priority, so their kernels are not queued behind the kernels of
// large grids; within a class, free slots take the shortest queued solve.
//
// A solve's results do not depend on what runs beside it: replicas never read
// each other's data, chunking does not change the arithmetic, and admitting a
// solve recomputes the spectral state of the others from their exact xi.
//
// PFDD_SERVER_TRACE=<file> writes one CSV line per scheduling event
// (t_s,class,event,a,b,c) when the server is destroyed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pfdd_converge.h"
#include "pfdd_gpu.h"
#include "pfdd_serve.h"

namespace {

using Clock = std::chrono::steady_clock;
constexpr double kChunkTargetS = 0.02;  // wall time of one chunk of steps
// An idle class keeps its memory (and its B(k)) this long unless other solves
// wait for memory: freeing device memory synchronises the whole device, which
// would stall the other classes' steps.
constexpr double kIdleReleaseS = 60.0;

struct Request {
  long long id = 0;
  pfdd_request spec{};
  std::vector<double> eps, tau_max;
  std::string key;
  std::vector<double> gamma, gamma_a;
  int progress = 0;
  pfdd::ConvergeTracker cv;  // converging solves: the loop's test
  bool stopped = false;      // converging solves: the test ended the loop
  Clock::time_point t_submit, t_done;
  bool done = false;
  pfdd_status status = PFDD_OK;
};

struct Class {
  int serial = 0;
  std::string key;
  int n[3] = {0, 0, 0}, ns = 0, nslots = 0;
  double C[3] = {0, 0, 0}, d[3] = {1, 1, 1}, cd2 = 0, asf = 0, dslip = 1, uq2 = 1;
  std::vector<double> eps;
  pfdd_ctx *ctx = nullptr;
  std::vector<long long> slot;  // request id per slot, -1 = free
  std::deque<long long> pending;
  size_t bytes = 0;
  int priority = 0;  // CUDA stream priority (lower = more urgent), see class_priority
  std::thread worker;
};

struct TraceEv {
  double t;
  int cls;
  const char *what;
  double a, b, c;
};

std::string hexd(double v) {
  char b[32];
  snprintf(b, sizeof b, "%a,", v);
  return b;
}

std::string class_key(const pfdd_request &r) {
  std::string k = std::to_string(r.n1) + "x" + std::to_string(r.n2) + "x" + std::to_string(r.n3) + "/" +
                  std::to_string(r.ns) + "/";
  for (double v : {r.C11, r.C12, r.C44, r.cd2, r.asf, r.dslip, r.uq2, r.d1, r.d2, r.d3}) k += hexd(v);
  for (int i = 0; i < r.ns * 9; ++i) k += hexd(r.eps[i]);
  return k;
}

}  // namespace

// Exclusive mode: one class's chunk of steps on the GPU at a time, the
// waiting class of the most urgent priority first (ties in arrival order).
struct TurnGate {
  std::mutex mu;
  std::condition_variable cv;
  bool busy = false;
  long long next_ticket = 0;
  std::map<std::pair<int, long long>, int> waiting;  // (priority, ticket)

  void acquire(int prio) {
    std::unique_lock<std::mutex> lk(mu);
    const auto key = std::make_pair(prio, next_ticket++);
    waiting.emplace(key, 0);
    cv.wait(lk, [&] { return !busy && waiting.begin()->first == key; });
    waiting.erase(waiting.begin());
    busy = true;
  }
  void release() {
    {
      std::lock_guard<std::mutex> lk(mu);
      busy = false;
    }
    cv.notify_all();
  }
};

struct pfdd_server {
  int prec = 0, dev = 0, max_slots = 1, chunk = 1;
  bool exclusive = false;
  TurnGate gate;
  size_t budget = 0, reserved = 0, peak = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::map<long long, std::unique_ptr<Request>> reqs;
  std::map<std::string, Class *> classes;
  std::deque<long long> waiting;     // requests whose class does not fit the budget yet
  std::vector<std::thread> retired;  // workers of released classes, joined later
  long long next_id = 1, steps_done = 0, solves_done = 0, classes_created = 0;
  bool stopping = false;
  Clock::time_point t0 = Clock::now();
  std::string trace_path;
  std::vector<TraceEv> trace;  // guarded by mu

  void log(int cls, const char *what, double a = 0, double b = 0, double c = 0) {  // under mu
    if (!trace_path.empty())
      trace.push_back({std::chrono::duration<double>(Clock::now() - t0).count(), cls, what, a, b, c});
  }
};

static void worker_main(pfdd_server *s, Class *c);

// Under s->mu: creates the class of request r if the budget admits it, with
// as many slots (up to max_slots) as fit, and at most an eighth of the budget
// unless one slot needs more: large grids gain nothing from wide batches (their
// steps are bound by memory bandwidth), and allocating tens of GB for slots
// that may stay empty delays every class created beside them.
static Class *try_make_class(pfdd_server *s, const Request &r) {
  const pfdd_request &q = r.spec;
  int slots = s->max_slots;
  size_t need = pfdd_required_bytes(q.n1, q.n2, q.n3, q.ns, slots, s->prec);
  while (slots > 1 && (s->reserved + need > s->budget || need > s->budget / 8)) {
    --slots;
    need = pfdd_required_bytes(q.n1, q.n2, q.n3, q.ns, slots, s->prec);
  }
  if (s->reserved + need > s->budget) return nullptr;
  Class *c = new Class();
  c->serial = (int)s->classes_created;
  c->key = r.key;
  c->n[0] = q.n1; c->n[1] = q.n2; c->n[2] = q.n3; c->ns = q.ns; c->nslots = slots;
  c->C[0] = q.C11; c->C[1] = q.C12; c->C[2] = q.C44;
  c->d[0] = q.d1 > 0 ? q.d1 : 1.0; c->d[1] = q.d2 > 0 ? q.d2 : 1.0; c->d[2] = q.d3 > 0 ? q.d3 : 1.0;
  c->cd2 = q.cd2; c->asf = q.asf; c->dslip = q.dslip; c->uq2 = q.uq2;
  c->eps = r.eps;
  c->slot.assign(slots, -1);
  c->bytes = need;
  s->reserved += need;
  s->peak = std::max(s->peak, s->reserved);
  s->classes[c->key] = c;
  s->classes_created++;
  s->log(c->serial, "class", (double)q.n1 * q.n2 * q.n3, q.ns, slots);
  c->worker = std::thread(worker_main, s, c);
  return c;
}

static void finish(pfdd_server *s, Request &r, pfdd_status st, int cls) {
  r.status = st;
  r.done = true;
  r.t_done = Clock::now();
  s->solves_done++;
  s->log(cls, "finish", (double)r.id, std::chrono::duration<double>(r.t_done - r.t_submit).count(), st);
}

// Under s->mu: queues request id into its class, creating the class if the
// budget admits it; otherwise the request waits for memory, or fails when it
// would not fit even into an empty server.
static void route(pfdd_server *s, long long id) {
  Request &r = *s->reqs[id];
  auto it = s->classes.find(r.key);
  Class *c = it != s->classes.end() ? it->second : try_make_class(s, r);
  if (c) {
    c->pending.push_back(id);
  } else if (pfdd_required_bytes(r.spec.n1, r.spec.n2, r.spec.n3, r.spec.ns, 1, s->prec) > s->budget) {
    finish(s, r, PFDD_ENOMEM, -1);
  } else {
    s->waiting.push_back(id);
  }
}

// CUDA stream priority of a class: one level more urgent per factor 4 less
// work in one solve's step (grid points x systems), least urgent from 2^27.5
// (256^3 x 12) on; pfdd_set_stream_priority clamps to the device's range.
// The block scheduler dispatches the CTAs of grids of equal priority in launch
// order, so without this a small solve's kernel waits behind every CTA of a
// large grid's kernel; the slot count must not enter (a class of many small
// solves is still a class of small kernels).
static int class_priority(const Class *c) {
  const double work = (double)c->n[0] * c->n[1] * c->n[2] * c->ns;
  return -std::max(0, (int)std::floor((27.6 - std::log2(std::max(work, 1.0))) / 2.0));
}

static pfdd_status setup_class(pfdd_server *s, Class *c) {
  const int ns = c->ns;
  pfdd_status st = pfdd_create_batched(&c->ctx, c->n[0], c->n[1], c->n[2], ns, c->nslots, s->prec, s->dev);
  c->priority = class_priority(c);
  if (st == PFDD_OK) st = pfdd_set_stream_priority(c->ctx, c->priority);
  if (st == PFDD_OK) st = pfdd_build_B(c->ctx, c->C[0], c->C[1], c->C[2], c->eps.data(), c->d[0], c->d[1], c->d[2]);
  if (st == PFDD_OK) {
    std::vector<double> v(ns, c->cd2), a(ns, c->asf), d(ns, c->dslip);
    st = pfdd_set_params(c->ctx, v.data(), a.data(), d.data(), c->uq2);
  }
  for (int r = 0; st == PFDD_OK && r < c->nslots; ++r) st = pfdd_set_replica_active(c->ctx, r, 0);
  return st;
}

static void worker_main(pfdd_server *s, Class *c) {
  cudaSetDevice(s->dev);
  const int R = c->nslots, ns = c->ns;
  const auto t_setup = Clock::now();
  const pfdd_status st = setup_class(s, c);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->log(c->serial, "ready", std::chrono::duration<double>(Clock::now() - t_setup).count(), st);
  }
  std::vector<double> tau, g, ga;
  std::vector<Request *> act(R, nullptr);
  double step_s = 0;  // running estimate of the wall time of one step
  auto idle_since = Clock::now();
  while (true) {
    std::vector<std::pair<int, Request *>> admit;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (st != PFDD_OK) {  // the class could not be set up: fail its solves
        for (long long id : c->pending) finish(s, *s->reqs[id], st, c->serial);
        c->pending.clear();
        s->cv.notify_all();
      }
      // free slots take the queued solves with the fewest steps first (shortest
      // job first: a short solve does not wait behind long ones of its class)
      for (int r = 0; r < R && !c->pending.empty(); ++r)
        if (c->slot[r] < 0) {
          auto best = std::min_element(c->pending.begin(), c->pending.end(), [&](long long a, long long b) {
            const int sa = s->reqs.at(a)->spec.steps, sb = s->reqs.at(b)->spec.steps;
            return sa != sb ? sa < sb : a < b;
          });
          c->slot[r] = *best;
          c->pending.erase(best);
          admit.emplace_back(r, s->reqs.at(c->slot[r]).get());
        }
      const bool busy = std::any_of(c->slot.begin(), c->slot.end(), [](long long v) { return v >= 0; });
      if (!busy) {
        const double idle = std::chrono::duration<double>(Clock::now() - idle_since).count();
        if (s->stopping || idle > kIdleReleaseS || !s->waiting.empty() || st != PFDD_OK) {
          s->classes.erase(c->key);  // new solves of this key now create a new class
          s->retired.push_back(std::move(c->worker));
          s->log(c->serial, "release", idle);
          break;
        }
        s->cv.wait_for(lk, std::chrono::milliseconds(20));
        continue;
      }
    }
    idle_since = Clock::now();
    for (auto &sa : admit) {
      Request &r = *sa.second;
      pfdd_status e = pfdd_set_replica_state(c->ctx, sa.first, r.spec.xi, r.spec.xi_bc);
      if (e == PFDD_OK) e = pfdd_set_replica_active(c->ctx, sa.first, 1);
      std::lock_guard<std::mutex> lk(s->mu);
      s->log(c->serial, "admit", (double)r.id, sa.first,
             std::chrono::duration<double>(Clock::now() - r.t_submit).count());
      if (e != PFDD_OK) {
        finish(s, r, e, c->serial);
        c->slot[sa.first] = -1;
        s->cv.notify_all();
      }
    }
    // one chunk: ends where the next active solve finishes, about kChunkTargetS long
    int chunk = std::min(s->chunk, 2);  // until the step time is known
    if (step_s > 0) chunk = std::max(1, std::min(s->chunk, (int)(kChunkTargetS / step_s)));
    int nact = 0;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (int r = 0; r < R; ++r) {
        act[r] = c->slot[r] >= 0 ? s->reqs.at(c->slot[r]).get() : nullptr;
        if (act[r]) {
          chunk = std::min(chunk, act[r]->spec.steps - act[r]->progress);
          if (act[r]->spec.converge) chunk = std::min(chunk, act[r]->cv.min_steps());  // never past a stop
          ++nact;
        }
      }
    }
    if (!nact) continue;
    tau.assign((size_t)chunk * R * ns, 0.0);
    for (int r = 0; r < R; ++r)
      if (act[r])
        for (int k = 0; k < chunk; ++k)
          for (int a = 0; a < ns; ++a)
            tau[((size_t)k * R + r) * ns + a] =
                act[r]->tau_max[a] * ((act[r]->progress + k + 1.0) / act[r]->spec.steps);
    g.assign((size_t)chunk * R, 0.0);
    ga.assign((size_t)chunk * R * ns, 0.0);
    if (s->exclusive) s->gate.acquire(c->priority);
    const auto tc = Clock::now();
    const pfdd_status e = pfdd_step(c->ctx, chunk, tau.data(), g.data(), ga.data());
    const double dt = std::chrono::duration<double>(Clock::now() - tc).count();
    if (s->exclusive) s->gate.release();
    step_s = step_s > 0 ? 0.5 * step_s + 0.5 * dt / chunk : dt / chunk;
    std::vector<int> finished;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->log(c->serial, "chunk", chunk, nact, dt);
      for (int r = 0; r < R; ++r) {
        Request *q = act[r];
        if (!q) continue;
        pfdd_status eq = e;
        for (int k = 0; k < chunk; ++k) {
          q->gamma[q->progress + k] = g[(size_t)k * R + r];
          for (int a = 0; a < ns; ++a)
            q->gamma_a[(size_t)(q->progress + k) * ns + a] = ga[((size_t)k * R + r) * ns + a];
          if (q->spec.converge && eq == PFDD_OK && q->cv.update(g[(size_t)k * R + r])) {
            if (k != chunk - 1) eq = PFDD_EINVAL;  // a stop inside a chunk: the bound failed
            q->stopped = true;
          }
        }
        q->progress += chunk;
        s->steps_done += chunk;
        if (eq != PFDD_OK || q->stopped || q->progress >= q->spec.steps) finished.push_back(r);
        if (eq != PFDD_OK) q->status = eq;
      }
    }
    for (int r : finished) {
      Request *q = act[r];
      pfdd_status e2 = e != PFDD_OK ? e : q->status;
      if (e2 == PFDD_OK && q->spec.xi_out) e2 = pfdd_get_replica_state(c->ctx, r, q->spec.xi_out);
      pfdd_set_replica_active(c->ctx, r, 0);
      std::lock_guard<std::mutex> lk(s->mu);
      finish(s, *q, e2, c->serial);
      c->slot[r] = -1;
      s->cv.notify_all();
    }
  }
  // the memory is returned before the budget is: waiting solves can then
  // create their classes
  if (c->ctx) pfdd_destroy(c->ctx);
  std::lock_guard<std::mutex> lk(s->mu);
  s->reserved -= c->bytes;
  delete c;
  std::deque<long long> retry;
  retry.swap(s->waiting);
  for (long long id : retry) route(s, id);
  s->cv.notify_all();
}

extern "C" pfdd_status pfdd_server_create(pfdd_server **out, int precision, int device, size_t hbm_budget,
                                          int max_slots, int chunk_steps) {
  if (!out || max_slots < 1 || chunk_steps < 1 ||
      (precision != PFDD_FP64 && precision != PFDD_FFT_FP32 && precision != PFDD_FFT_FP32_BFLY))
    return PFDD_EINVAL;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return PFDD_ECUDA;
  size_t freeb = 0, total = 0;
  if (cudaMemGetInfo(&freeb, &total) != cudaSuccess) return PFDD_ECUDA;
  pfdd_server *s = new pfdd_server();
  s->prec = precision; s->dev = device; s->max_slots = max_slots; s->chunk = chunk_steps;
  s->budget = hbm_budget ? std::min(hbm_budget, freeb) : (size_t)(0.9 * (double)freeb);
  if (const char *p = std::getenv("PFDD_SERVER_TRACE")) s->trace_path = p;
  if (const char *p = std::getenv("PFDD_SERVER_EXCLUSIVE")) s->exclusive = p[0] && p[0] != '0';
  *out = s;
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_server_submit(pfdd_server *s, const pfdd_request *q, long long *id) {
  if (!s || !q || !id || !q->eps || !q->tau_max || !q->xi || q->steps < 1 || q->ns < 1 || q->ns > 12)
    return PFDD_EINVAL;
  const long long N = (long long)q->n1 * q->n2 * q->n3;
  if (N < 1) return PFDD_EINVAL;
  auto r = std::make_unique<Request>();
  r->spec = *q;
  r->eps.assign(q->eps, q->eps + 9 * q->ns);
  r->tau_max.assign(q->tau_max, q->tau_max + q->ns);
  r->spec.eps = nullptr; r->spec.tau_max = nullptr;
  r->key = class_key(*q);
  r->gamma.assign(q->steps, 0.0);
  r->gamma_a.assign((size_t)q->steps * q->ns, 0.0);
  if (q->converge) r->cv.reset(q->gamma_prev);
  std::vector<std::thread> done_workers;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return PFDD_EINVAL;
    r->id = s->next_id++;
    r->t_submit = Clock::now();
    *id = r->id;
    s->log(-1, "submit", (double)r->id, (double)N, q->steps);
    s->reqs[r->id] = std::move(r);
    route(s, *id);
    s->cv.notify_all();
    if (s->retired.size() >= 8) done_workers.swap(s->retired);
  }
  for (auto &t : done_workers) t.join();  // workers of released classes, finishing their teardown
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_server_wait(pfdd_server *s, long long id, double *gamma, double *gamma_a,
                                        double *latency_s) {
  return pfdd_server_wait_run(s, id, gamma, gamma_a, latency_s, nullptr);
}

extern "C" pfdd_status pfdd_server_wait_run(pfdd_server *s, long long id, double *gamma, double *gamma_a,
                                            double *latency_s, int *steps_run) {
  if (!s) return PFDD_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return PFDD_EINVAL;
  Request &r = *it->second;
  s->cv.wait(lk, [&] { return r.done; });
  if (gamma) std::memcpy(gamma, r.gamma.data(), r.gamma.size() * sizeof(double));
  if (gamma_a) std::memcpy(gamma_a, r.gamma_a.data(), r.gamma_a.size() * sizeof(double));
  if (latency_s) *latency_s = std::chrono::duration<double>(r.t_done - r.t_submit).count();
  if (steps_run) *steps_run = r.progress;
  const pfdd_status st = r.status;
  s->reqs.erase(it);
  return st;
}

extern "C" pfdd_status pfdd_server_stats(pfdd_server *s, long long *steps_done, long long *solves_done,
                                         long long *classes_created, size_t *peak_bytes) {
  if (!s) return PFDD_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  if (steps_done) *steps_done = s->steps_done;
  if (solves_done) *solves_done = s->solves_done;
  if (classes_created) *classes_created = s->classes_created;
  if (peak_bytes) *peak_bytes = s->peak;
  return PFDD_OK;
}

extern "C" void pfdd_server_destroy(pfdd_server *s) {
  if (!s) return;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv.wait(lk, [&] {
    for (auto &kv : s->reqs)
      if (!kv.second->done) return false;
    return true;
  });
  s->stopping = true;
  s->cv.notify_all();
  s->cv.wait(lk, [&] { return s->classes.empty(); });
  std::vector<std::thread> workers;
  workers.swap(s->retired);
  lk.unlock();
  for (auto &t : workers) t.join();
  if (!s->trace_path.empty()) {
    if (FILE *f = std::fopen(s->trace_path.c_str(), "w")) {
      std::fprintf(f, "t_s,class,event,a,b,c\n");
      for (const TraceEv &e : s->trace) std::fprintf(f, "%.6f,%d,%s,%.9g,%.9g,%.9g\n", e.t, e.cls, e.what, e.a, e.b, e.c);
      std::fclose(f);
    }
  }
  delete s;
}

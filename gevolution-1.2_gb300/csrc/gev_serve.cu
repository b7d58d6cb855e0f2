// gev_serve.cu -- continuous batching of independent simulations on one GPU
// (include/gev_serve.h).  Host code: scheduler threads drive the hot-path
// library, one context (one CUDA stream) per admitted simulation.  Worker 0 also
// admits requests; each admitted simulation is handed to the worker with the
// fewest grid points in hand, and only that worker enqueues its cycles, so the
// launches of different simulations are issued from several host threads at once
// (a 64^3 cycle is some fifty short kernels: one thread cannot issue them as fast
// as the GPU runs them for dozens of small simulations).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/gev_serve.h"
#include "gev_internal.cuh"

namespace {

typedef std::chrono::steady_clock Clock;

// a pooled simulation of one grid size and precision form, with the events that
// mark its cycles in flight
struct Slot {
  gev_ctx *ctx = nullptr;
  gev_sim *sim = nullptr;
  int N = 0, prec = 0;
  size_t bytes = 0;
  std::vector<cudaEvent_t> ev;  // ring of `inflight` events
};

struct Active {
  long id = 0;
  gev_request req{};
  Slot *slot = nullptr;
  double a_target = 1., t_submit = 0., t_admit = 0.;
  int cycles = 0;
  long head = 0, tail = 0;  // events [tail, head) of the ring are in flight
  bool finishing = false;
  int worker = 0;           // the scheduler thread that enqueues its cycles
  bool need_ic = false;     // admitted; its worker generates the initial conditions first
  gev_ic_params ic{};
};

struct Pending {
  long id;
  gev_request req;
  double t_submit;
};

}  // namespace

struct gev_server {
  int device = 0, max_active = 0, inflight = 2;
  size_t budget = 0, in_use = 0, peak = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Pending> pending;
  int admitting = 0;  // taken off pending, not yet on active (drain waits for them too)
  std::vector<gev_result> done;
  std::vector<Active *> active;
  std::mutex pool_mu;  // idle (taken before mu where both are held)
  std::map<std::pair<int, int>, std::vector<Slot *>> idle;
  std::map<std::pair<int, int>, size_t> footprint;
  int workers = 1;
  std::atomic<int> graphs{0};  // 1: cycles enqueued as CUDA graphs (gev_sim_step_graph)
  std::vector<std::thread> th;
  bool stop = false;
  long next_id = 1;
  gev_server_stats st{};
  Clock::time_point t0;
  double busy_since = -1.;
  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void slot_destroy(gev_server *s, Slot *sl) {
  for (cudaEvent_t e : sl->ev) cudaEventDestroy(e);
  gev_sim_destroy(sl->sim);
  gev_ctx_destroy(sl->ctx);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->in_use -= sl->bytes;
  }
  delete sl;
}

// the slot's bytes as its context counts them (the scratch grows with the IC and
// the first cycles; the largest seen is the size's footprint)
void slot_measure(gev_server *s, Slot *sl) {
  size_t b = 0;
  gev_ctx_info(sl->ctx, nullptr, nullptr, &b);
  std::lock_guard<std::mutex> lk(s->mu);
  s->in_use += b - sl->bytes;
  sl->bytes = b;
  s->peak = std::max(s->peak, s->in_use);
  size_t &f = s->footprint[std::make_pair(sl->N, sl->prec)];
  f = std::max(f, b);
}

// a simulation slot for (N, prec): an idle one, or a new one if its bytes fit
// (idle slots of other sizes are released to make room); nullptr when it does not fit
Slot *slot_acquire(gev_server *s, int N, int prec, int *rc) {
  *rc = GEV_OK;
  auto key = std::make_pair(N, prec);
  std::unique_lock<std::mutex> pk(s->pool_mu);
  auto &pool = s->idle[key];
  if (!pool.empty()) {
    Slot *sl = pool.back();
    pool.pop_back();
    return sl;
  }
  // the bytes it needs: measured for its size, else scaled as N^3 from the largest
  // size of its form measured so far, else unknown (the first slot is the probe)
  bool known;
  size_t need;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto fp = s->footprint.find(key);
    known = fp != s->footprint.end();
    need = known ? fp->second : 0;
    if (!known) {
      int nk = 0;
      size_t bk = 0;
      for (auto &kv : s->footprint)
        if (kv.first.second == prec && kv.first.first > nk) {
          nk = kv.first.first;
          bk = kv.second;
        }
      if (nk > 0) {
        const double r = (double)N / (double)nk;
        need = (size_t)((double)bk * r * r * r);
        known = true;
      }
    }
  }
  auto fits = [&]() {
    std::lock_guard<std::mutex> lk(s->mu);
    return s->in_use + need <= s->budget;
  };
  while (!fits()) {  // release idle slots of other sizes, largest first
    Slot *victim = nullptr;
    std::vector<Slot *> *from = nullptr;
    for (auto &kv : s->idle)
      for (Slot *c : kv.second)
        if (!victim || c->bytes > victim->bytes) {
          victim = c;
          from = &kv.second;
        }
    if (!victim) return nullptr;
    from->erase(std::find(from->begin(), from->end(), victim));
    slot_destroy(s, victim);
  }
  pk.unlock();
  Slot *sl = new Slot();
  sl->N = N;
  sl->prec = prec;
  *rc = gev_ctx_create(s->device, N, prec, &sl->ctx);
  if (!*rc) *rc = gev_sim_create(sl->ctx, (long)N * N * N, &sl->sim);
  if (!*rc) {
    sl->ev.resize((size_t)s->inflight);
    for (auto &e : sl->ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) *rc = GEV_ECUDA;
  }
  if (*rc) {
    if (sl->sim) gev_sim_destroy(sl->sim);
    if (sl->ctx) gev_ctx_destroy(sl->ctx);
    for (cudaEvent_t e : sl->ev)
      if (e) cudaEventDestroy(e);
    delete sl;
    cudaGetLastError();
    return nullptr;
  }
  slot_measure(s, sl);
  if (!known && s->in_use > s->budget) {  // the first of its size: it did not fit after all
    slot_destroy(s, sl);
    return nullptr;
  }
  return sl;
}

// takes a finished simulation off the device's list
void remove_active(gev_server *s, Active *A) {
  std::lock_guard<std::mutex> lk(s->mu);
  s->active.erase(std::find(s->active.begin(), s->active.end(), A));
  if (s->active.empty() && s->busy_since >= 0.) {
    s->st.busy_seconds += s->now() - s->busy_since;
    s->busy_since = -1.;
  }
  delete A;
  s->cv.notify_all();
}

void finish(gev_server *s, Active *A, int status) {
  gev_result r;
  memset(&r, 0, sizeof(r));
  r.id = A->id;
  r.N = A->req.N;
  r.prec = A->req.prec;
  r.cycles = A->cycles;
  r.status = status;
  r.t_submit = A->t_submit;
  r.t_admit = A->t_admit;
  Slot *sl = A->slot;
  if (!status) {
    gev_sim *sim = sl->sim;
    r.a = sim->st.a;
    r.tau = sim->st.tau;
    // the power spectrum of phi (output.hpp:1922-1928): its table's k and P
    const int nb = A->req.numbins;
    std::vector<double> ks(nb), ps(nb);
    int rc = gev_fft_r2c(sl->ctx, sim->phi, sim->scalarFT);
    if (!rc)
      rc = gev_cross_spectrum(sl->ctx, sim->scalarFT, sim->scalarFT, r.kbin, r.power, ks.data(), ps.data(),
                              r.occupation, nb, 0, 1, 0, -1, -1);
    if (rc) {
      r.status = rc;
    } else {
      const double n3 = (double)A->req.N * A->req.N * A->req.N;
      for (int i = 0; i < nb; i++) {
        r.kbin[i] /= A->req.boxsize;
        r.power[i] /= n3 * n3 * 2. * M_PI * M_PI;
      }
      r.numbins = nb;
    }
  }
  r.t_done = s->now();
  slot_measure(s, sl);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->done.push_back(r);
    if (r.status)
      s->st.failed++;
    else
      s->st.completed++;
  }
  if (r.status) {
    slot_destroy(s, sl);  // a slot that failed is not reused
  } else {
    std::lock_guard<std::mutex> pk(s->pool_mu);
    s->idle[std::make_pair(sl->N, sl->prec)].push_back(sl);
  }
  s->cv.notify_all();
}

// the worker with the fewest grid points among the simulations it enqueues
int least_loaded_worker(gev_server *s) {
  std::vector<double> load((size_t)s->workers, 0.);
  for (Active *A : s->active) load[(size_t)A->worker] += (double)A->req.N * A->req.N * A->req.N;
  return (int)(std::min_element(load.begin(), load.end()) - load.begin());
}

void scheduler(gev_server *s, int worker) {
  cudaSetDevice(s->device);
  while (true) {
    // admission (worker 0): requests in arrival order while their bytes fit
    for (; worker == 0;) {
      Pending p;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop || s->pending.empty()) break;
        if (s->max_active > 0 && (int)s->active.size() >= s->max_active) break;
        p = s->pending.front();
      }
      int rc = GEV_OK;
      Slot *sl = slot_acquire(s, p.req.N, p.req.prec, &rc);
      if (!sl && !rc) {  // does not fit yet: wait for a simulation to finish
        bool alone;
        {
          std::lock_guard<std::mutex> lk(s->mu);
          alone = s->active.empty();
        }
        if (!alone) break;
        rc = GEV_ENOMEM;  // nothing else holds memory: it never fits
      }
      {
        std::lock_guard<std::mutex> lk(s->mu);
        s->pending.pop_front();
        s->admitting++;
      }
      Active *A = new Active();
      A->id = p.id;
      A->req = p.req;
      A->t_submit = p.t_submit;
      A->t_admit = s->now();
      A->slot = sl;
      if (sl) {  // the initial conditions are generated by the worker that steps it
        gev_ic_params &ic = A->ic;
        memset(&ic, 0, sizeof(ic));
        ic.h = p.req.h;
        ic.Omega_cdm = p.req.Omega_cdm;
        ic.Omega_b = p.req.Omega_b;
        ic.n_s = p.req.n_s;
        ic.sigma8 = p.req.sigma8;
        ic.z_in = p.req.z_in;
        ic.boxsize = p.req.boxsize;
        ic.Cf = 48.;
        ic.steplimit = 0.04;
        ic.seed = p.req.seed;
        ic.ksphere = 1;
        ic.correct_displacement = 1;
        A->need_ic = true;
        A->a_target = 1. / (1. + p.req.z_target);
      }
      {
        std::lock_guard<std::mutex> lk(s->mu);
        s->st.admitted++;
        if (s->active.empty() && s->busy_since < 0.) s->busy_since = s->now();
        // a failed admission is finished below by this worker
        A->worker = (sl && !rc) ? least_loaded_worker(s) : 0;
        s->active.push_back(A);
        s->admitting--;
        s->st.max_active_seen = std::max(s->st.max_active_seen, (long)s->active.size());
      }
      if (!sl || rc) {
        if (sl) {
          finish(s, A, rc);
        } else {
          gev_result r;
          memset(&r, 0, sizeof(r));
          r.id = A->id;
          r.N = A->req.N;
          r.prec = A->req.prec;
          r.status = rc ? rc : GEV_ENOMEM;
          r.t_submit = A->t_submit;
          r.t_done = s->now();
          std::lock_guard<std::mutex> lk(s->mu);
          s->done.push_back(r);
          s->st.failed++;
        }
        remove_active(s, A);
      }
    }
    // one round: each admitted simulation gets its next cycle enqueued, as far
    // as its in-flight window allows; finished ones hand back their result
    bool progressed = false;
    std::vector<Active *> act;  // this worker's own: only it removes them
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->stop) break;
      for (Active *A : s->active)
        if (A->worker == worker) act.push_back(A);
    }
    for (Active *A : act) {
      Slot *sl = A->slot;
      if (A->need_ic) {  // on this worker's thread, so that several simulations start at once
        A->need_ic = false;
        const int rc = gev_sim_ic_generate(sl->sim, &A->ic);
        if (rc) {
          cudaGetLastError();
          finish(s, A, rc);
          remove_active(s, A);
        } else {
          slot_measure(s, sl);
        }
        progressed = true;
        continue;
      }
      const long R = (long)sl->ev.size();
      while (A->tail < A->head && cudaEventQuery(sl->ev[(size_t)(A->tail % R)]) == cudaSuccess) A->tail++;
      if (A->finishing) {
        if (A->tail == A->head) {
          finish(s, A, GEV_OK);
          remove_active(s, A);
          progressed = true;
        }
        continue;
      }
      if (A->head - A->tail >= R) continue;
      // main.cpp runs cycles until the one that passes the target redshift
      if (sl->sim->st.a >= A->a_target) {
        A->finishing = true;
        progressed = true;
        continue;
      }
      const bool as_graph = s->graphs.load(std::memory_order_relaxed) != 0;
      const long g0 = sl->sim->graph_launches;
      const int rc = as_graph ? gev_sim_step_graph(sl->sim) : gev_sim_step(sl->sim);
      if (rc || cudaEventRecord(sl->ev[(size_t)(A->head % R)], sl->ctx->stream) != cudaSuccess) {
        cudaStreamSynchronize(sl->ctx->stream);
        cudaGetLastError();
        finish(s, A, rc ? rc : GEV_ECUDA);
        remove_active(s, A);
        continue;
      }
      A->head++;
      A->cycles++;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        s->st.particle_steps += (double)A->req.N * A->req.N * A->req.N;
        s->st.graph_cycles += sl->sim->graph_launches - g0;
      }
      progressed = true;
    }
    if (!progressed) {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->stop) break;
      s->cv.wait_for(lk, std::chrono::microseconds(50));
    }
  }
}

}  // namespace

extern "C" {

int gev_server_footprint(int device, int N, int prec, size_t *bytes) {
  if (!bytes) return GEV_EINVAL;
  gev_ctx *ctx = nullptr;
  gev_sim *sim = nullptr;
  int rc = gev_ctx_create(device, N, prec, &ctx);
  if (!rc) rc = gev_sim_create(ctx, (long)N * N * N, &sim);
  if (!rc) gev_ctx_info(ctx, nullptr, nullptr, bytes);
  if (sim) gev_sim_destroy(sim);
  if (ctx) gev_ctx_destroy(ctx);
  return rc;
}

int gev_server_create(int device, size_t bytes_budget, int max_active, int inflight, gev_server **out) {
  return gev_server_create_workers(device, bytes_budget, max_active, inflight, 0, out);
}

int gev_server_create_workers(int device, size_t bytes_budget, int max_active, int inflight, int workers,
                              gev_server **out) {
  if (!out || max_active < 0 || inflight < 0 || workers < 0 || workers > GEV_SERVE_MAX_WORKERS) return GEV_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return GEV_ENODEV;
  gev_server *s = new gev_server();
  s->device = device;
  s->max_active = max_active;
  s->inflight = inflight > 0 ? inflight : 2;
  if (bytes_budget == 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    bytes_budget = (size_t)(0.9 * (double)fr);
  }
  s->budget = bytes_budget;
  s->st.bytes_budget = bytes_budget;
  s->t0 = Clock::now();
  if (workers == 0) {
    const unsigned hc = std::thread::hardware_concurrency();
    workers = hc >= 16 ? 4 : hc >= 8 ? 2 : 1;
  }
  s->workers = workers;
  for (int k = 0; k < workers; ++k) s->th.emplace_back(scheduler, s, k);
  *out = s;
  return GEV_OK;
}

int gev_server_set_graphs(gev_server *s, int on) {
  if (!s) return GEV_EINVAL;
  s->graphs.store(on ? 1 : 0, std::memory_order_relaxed);
  return GEV_OK;
}

int gev_server_submit(gev_server *s, const gev_request *req, long *id) {
  if (!s || !req || req->N < 8 || req->N % 4 != 0 || req->numbins < 1 || req->numbins > GEV_SERVE_MAX_BINS ||
      req->boxsize <= 0. || req->z_target < 0. || req->z_in <= req->z_target ||
      (req->prec != GEV_PREC_FP64 && req->prec != GEV_PREC_MIXED))
    return GEV_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  Pending p{s->next_id++, *req, s->now()};
  s->pending.push_back(p);
  s->st.submitted++;
  if (id) *id = p.id;
  s->cv.notify_all();
  return GEV_OK;
}

int gev_server_poll(gev_server *s, gev_result *out, int max, int *n) {
  if (!s || !n || (max > 0 && !out)) return GEV_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  const int k = std::min(max, (int)s->done.size());
  for (int i = 0; i < k; i++) out[i] = s->done[(size_t)i];
  s->done.erase(s->done.begin(), s->done.begin() + k);
  *n = k;
  return GEV_OK;
}

int gev_server_drain(gev_server *s, double timeout_s) {
  if (!s) return GEV_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto until = Clock::now() + std::chrono::duration<double>(timeout_s > 0. ? timeout_s : 1e9);
  auto busy = [&]() { return !s->pending.empty() || s->admitting > 0 || !s->active.empty(); };
  while (busy()) {
    if (s->cv.wait_until(lk, until) == std::cv_status::timeout && busy()) return GEV_ETIMEOUT;
  }
  return GEV_OK;
}

int gev_server_stats_get(gev_server *s, gev_server_stats *out) {
  if (!s || !out) return GEV_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->st;
  out->active = (long)s->active.size();
  out->pending = (long)s->pending.size() + s->admitting;
  out->bytes_in_use = s->in_use;
  out->bytes_peak = s->peak;
  out->workers = s->workers;
  if (s->busy_since >= 0.) out->busy_seconds += s->now() - s->busy_since;
  return GEV_OK;
}

int gev_server_destroy(gev_server *s) {
  if (!s) return GEV_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  for (std::thread &t : s->th)
    if (t.joinable()) t.join();
  for (Active *A : s->active) {
    if (A->slot) {
      cudaStreamSynchronize(A->slot->ctx->stream);
      slot_destroy(s, A->slot);
    }
    delete A;
  }
  for (auto &kv : s->idle)
    for (Slot *sl : kv.second) slot_destroy(s, sl);
  delete s;
  return GEV_OK;
}

}  // extern "C"

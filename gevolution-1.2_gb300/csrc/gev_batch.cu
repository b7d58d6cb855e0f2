// gev_batch.cu -- one cycle of many simulations with one launch per kernel of the
// cycle for each cohort of simulations of one grid size (include/gev_sim.h,
// gev_batch_step).
//
// Each simulation's cycle is recorded, not enqueued: its context's recorder takes
// every launch of the cycle (gev_launch, gev_batch.cuh) while the host runs the same
// code as gev_sim_step, so the host's side of the cycle (background, dtau, the
// particle arrays' halves) advances as in a direct cycle.  The simulation's stream is
// under capture meanwhile: an operation that bypasses the recorder lands in the
// capture instead of running, and the simulation then takes a direct cycle.
// Simulations whose recorded cycles have the same launch sequence (kernels, grids,
// blocks, shared memory) form a cohort; the cohort's packed arguments go to the
// device in one copy (a ring of three pinned staging buffers), and each kernel of the
// cycle runs once for the whole cohort (gridDim.y = the cohort's size) on the batch's
// streams (one a cohort, up to four), which first wait for the work already queued on
// every batched simulation's stream; afterwards each simulation's stream waits for its
// cohort.  Every block runs the kernel's own code on its simulation's arguments; the
// results agree with gev_sim_step's to FP32 rounding (the batched forms are compiled
// apart from the kernels, gev_batch.cuh), and bit for bit from one batched run to the
// next and whatever the other members of a cohort.
#include <cstring>
#include <map>
#include <set>
#include <vector>

#include "../../include/gev_sim.h"
#include "gev_batch.cuh"

constexpr int BATCH_STREAMS = 4;

struct gev_batch {
  int device = 0;
  cudaStream_t stream = nullptr;          // the staging copies, and the join of a step
  cudaStream_t cs[BATCH_STREAMS] = {};    // cohort c runs on cs[c % BATCH_STREAMS]
  cudaEvent_t cdone[BATCH_STREAMS] = {};  // the last cohort each ran in a step
  cudaEvent_t tables = nullptr;           // a step's argument tables are on the device
  struct Staging {
    unsigned char *host = nullptr;
    size_t host_bytes = 0;
    void *dev = nullptr;
    size_t dev_bytes = 0;
    cudaEvent_t copied = nullptr;  // the staging copy of the last step that used it
    bool used = false;
  };
  Staging ring[3];
  int next = 0;
  std::vector<GevRecorder> rec;
  std::vector<cudaEvent_t> ev;  // per recorded simulation: its stream's queued work
  cudaEvent_t done = nullptr;   // the batch's work of the last step
  long batched = 0, direct = 0, launches = 0;
};

namespace {

struct Saved {
  gev_sim_state st;
  PclsArrays cur, alt;
};

// records one cycle of s into r; false (host state put back) if it cannot be batched
bool record_cycle(gev_sim *s, GevRecorder &r) {
  gev_ctx *ctx = s->ctx;
  const Saved sv{s->st, s->pcls->cur, s->pcls->alt};
  r.clear();
  if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  ctx->rec = &r;
  const int rc = gev_sim_step(s);
  ctx->rec = nullptr;
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
  size_t stray = 0;
  if (g) {
    if (cudaGraphGetNodes(g, nullptr, &stray) != cudaSuccess) stray = 1;
    cudaGraphDestroy(g);
  }
  if (rc == GEV_OK && ce == cudaSuccess && g && stray == 0 && !r.bad) return true;
  cudaGetLastError();
  s->st = sv.st;
  s->pcls->cur = sv.cur;
  s->pcls->alt = sv.alt;
  return false;
}

// the launch sequence of a recorded cycle, as integers: simulations with equal
// signatures share every launch
std::vector<unsigned long long> signature(const GevRecorder &r) {
  std::vector<unsigned long long> k;
  k.reserve(r.ops.size() * 6);
  for (const GevOp &op : r.ops) {
    k.push_back((unsigned long long)(uintptr_t)op.launch);
    k.push_back(op.grid.x);
    k.push_back(op.block.x);
    k.push_back(op.smem);
    k.push_back(op.bytes);
  }
  return k;
}

inline size_t al16(size_t b) { return (b + 15) & ~(size_t)15; }

}  // namespace

extern "C" {

int gev_batch_create(int device, gev_batch **out) {
  if (!out) return GEV_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return GEV_ENODEV;
  }
  gev_batch *b = new gev_batch();
  b->device = device;
  bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->tables, cudaEventDisableTiming) == cudaSuccess;
  for (int c = 0; c < BATCH_STREAMS; ++c)
    ok = ok && cudaStreamCreateWithFlags(&b->cs[c], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&b->cdone[c], cudaEventDisableTiming) == cudaSuccess;
  for (auto &r : b->ring) ok = ok && cudaEventCreateWithFlags(&r.copied, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    gev_batch_destroy(b);
    return GEV_ECUDA;
  }
  *out = b;
  return GEV_OK;
}

int gev_batch_destroy(gev_batch *b) {
  if (!b) return GEV_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto &r : b->ring) {
    if (r.host) cudaFreeHost(r.host);
    cudaFree(r.dev);
    if (r.copied) cudaEventDestroy(r.copied);
  }
  for (int c = 0; c < BATCH_STREAMS; ++c) {
    if (b->cs[c]) {
      cudaStreamSynchronize(b->cs[c]);
      cudaStreamDestroy(b->cs[c]);
    }
    if (b->cdone[c]) cudaEventDestroy(b->cdone[c]);
  }
  for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
  if (b->done) cudaEventDestroy(b->done);
  if (b->tables) cudaEventDestroy(b->tables);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return GEV_OK;
}

int gev_batch_info(gev_batch *b, long *batched, long *direct, long *launches) {
  if (!b) return GEV_EINVAL;
  if (batched) *batched = b->batched;
  if (direct) *direct = b->direct;
  if (launches) *launches = b->launches;
  return GEV_OK;
}

int gev_batch_step(gev_batch *b, gev_sim *const *sims, int n) {
  // (a cohort's size is gridDim.y of its launches: at most 65535)
  if (!b || n < 0 || n > 65535 || (n > 0 && !sims)) return GEV_EINVAL;
  {
    std::set<const gev_sim *> seen;
    for (int i = 0; i < n; ++i)
      if (!sims[i] || !sims[i]->ctx || sims[i]->ctx->device != b->device || !seen.insert(sims[i]).second)
        return GEV_EINVAL;  // null, foreign device, or the same simulation twice
  }
  if (cudaSetDevice(b->device) != cudaSuccess) return GEV_ENODEV;
  // the simulations that are batched: the mixed form past the cycles that tune and
  // allocate on first use (the first two), with the timers off; the rest, and any
  // whose recording fails, take a direct cycle on their own stream
  std::vector<int> idx;
  if (b->rec.size() < (size_t)n) b->rec.resize((size_t)n);
  for (int i = 0; i < n; ++i) {
    gev_sim *s = sims[i];
    const bool batchable = s->ctx->prec == GEV_PREC_MIXED && s->st.cycle >= 2 && s->st.dtau_old > 0. &&
                           !s->ctx->timing && !s->ctx->rec;
    if (batchable && record_cycle(s, b->rec[idx.size()])) {
      idx.push_back(i);
      continue;
    }
    b->direct++;
    const int rc = gev_sim_step(s);
    if (rc) return rc;
  }
  if (idx.empty()) return GEV_OK;
  // cohorts: equal launch sequences
  std::map<std::vector<unsigned long long>, std::vector<int>> cohorts;  // -> positions in idx
  for (size_t k = 0; k < idx.size(); ++k) cohorts[signature(b->rec[k])].push_back((int)k);
  // the batch's stream starts after each simulation's queued work
  while (b->ev.size() < idx.size()) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return GEV_ECUDA;
    b->ev.push_back(e);
  }
  for (size_t k = 0; k < idx.size(); ++k) {
    if (cudaEventRecord(b->ev[k], sims[idx[k]]->ctx->stream) != cudaSuccess ||
        cudaStreamWaitEvent(b->stream, b->ev[k], 0) != cudaSuccess)
      return GEV_ECUDA;
  }
  // argument tables: for each cohort and kernel, the cohort's packed arguments as an
  // array (row s = the cohort's s-th simulation), each table 16-byte aligned
  size_t total = 0;
  for (auto &c : cohorts) {
    const GevRecorder &r0 = b->rec[(size_t)c.second[0]];
    for (const GevOp &op : r0.ops)
      if (op.launch) total = al16(total) + op.bytes * c.second.size();
  }
  total = al16(total) + 16;
  gev_batch::Staging &sg = b->ring[b->next];
  if (sg.used && cudaEventSynchronize(sg.copied) != cudaSuccess) return GEV_ECUDA;
  if (sg.host_bytes < total) {
    if (sg.host) cudaFreeHost(sg.host);
    sg.host = nullptr;
    sg.host_bytes = 0;
    if (cudaMallocHost((void **)&sg.host, total * 2) != cudaSuccess) return GEV_ENOMEM;
    sg.host_bytes = total * 2;
  }
  if (sg.dev_bytes < total) {
    // the old table may still be read by an earlier step's kernels on this stream
    if (sg.dev && cudaStreamSynchronize(b->stream) != cudaSuccess) return GEV_ECUDA;
    cudaFree(sg.dev);
    sg.dev = nullptr;
    sg.dev_bytes = 0;
    if (cudaMalloc(&sg.dev, total * 2) != cudaSuccess) return GEV_ENOMEM;
    sg.dev_bytes = total * 2;
  }
  std::vector<std::vector<size_t>> table_off;
  size_t off = 0;
  for (auto &c : cohorts) {
    const GevRecorder &r0 = b->rec[(size_t)c.second[0]];
    std::vector<size_t> offs(r0.ops.size(), 0);
    for (size_t j = 0; j < r0.ops.size(); ++j) {
      const GevOp &op = r0.ops[j];
      if (!op.launch) continue;
      off = al16(off);
      offs[j] = off;
      for (size_t m = 0; m < c.second.size(); ++m) {
        const GevRecorder &r = b->rec[(size_t)c.second[m]];
        memcpy(sg.host + off + m * op.bytes, r.args.data() + r.ops[j].off, op.bytes);
      }
      off += op.bytes * c.second.size();
    }
    table_off.push_back(offs);
  }
  if (cudaMemcpyAsync(sg.dev, sg.host, off, cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
      cudaEventRecord(sg.copied, b->stream) != cudaSuccess || cudaEventRecord(b->tables, b->stream) != cudaSuccess)
    return GEV_ECUDA;
  sg.used = true;
  b->next = (b->next + 1) % 3;
  // each cohort's cycle, one launch per kernel, cohorts on their own streams (after the
  // tables, and so after every batched simulation's queued work); each simulation's
  // stream then waits for its cohort
  const int nstreams = (int)cohorts.size() < BATCH_STREAMS ? (int)cohorts.size() : BATCH_STREAMS;
  for (int c = 0; c < nstreams; ++c)
    if (cudaStreamWaitEvent(b->cs[c], b->tables, 0) != cudaSuccess) return GEV_ECUDA;
  size_t ci = 0;
  for (auto &c : cohorts) {
    const GevRecorder &r0 = b->rec[(size_t)c.second[0]];
    const unsigned ns = (unsigned)c.second.size();
    cudaStream_t st = b->cs[ci % BATCH_STREAMS];
    for (size_t j = 0; j < r0.ops.size(); ++j) {
      const GevOp &op = r0.ops[j];
      if (op.launch) {
        op.launch((const unsigned char *)sg.dev + table_off[ci][j], ns, op.grid, op.block, op.smem, st);
        b->launches++;
      } else {
        for (int m : c.second) {
          const GevOp &cp = b->rec[(size_t)m].ops[j];
          if (cudaMemcpyAsync(cp.dst, cp.src, cp.bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return GEV_ECUDA;
        }
      }
    }
    if (cudaGetLastError() != cudaSuccess) return GEV_ECUDA;
    cudaEvent_t e = b->cdone[ci % BATCH_STREAMS];
    if (cudaEventRecord(e, st) != cudaSuccess) return GEV_ECUDA;
    for (int m : c.second)
      if (cudaStreamWaitEvent(sims[idx[(size_t)m]]->ctx->stream, e, 0) != cudaSuccess) return GEV_ECUDA;
    ++ci;
  }
  // the staging stream joins the cohorts: the next copy into a table slot comes after
  // every kernel that read it
  for (int c = 0; c < nstreams; ++c)
    if (cudaStreamWaitEvent(b->stream, b->cdone[c], 0) != cudaSuccess) return GEV_ECUDA;
  if (cudaEventRecord(b->done, b->stream) != cudaSuccess) return GEV_ECUDA;
  b->batched += (long)idx.size();
  return GEV_OK;
}

int gev_batch_run(gev_batch *b, gev_sim *const *sims, int n, const double *a_target, int *cycles) {
  if (!b || n < 0 || (n > 0 && (!sims || !a_target || !cycles))) return GEV_EINVAL;
  for (int i = 0; i < n; ++i) cycles[i] = 0;
  std::vector<gev_sim *> active;
  std::vector<int> which;
  while (true) {
    active.clear();
    which.clear();
    for (int i = 0; i < n; ++i)
      if (sims[i] && sims[i]->st.a < a_target[i]) {  // main.cpp runs cycles until one passes the target
        active.push_back(sims[i]);
        which.push_back(i);
      }
    if (active.empty()) break;
    const int rc = gev_batch_step(b, active.data(), (int)active.size());
    if (rc) return rc;
    for (int i : which) cycles[i]++;
  }
  for (int i = 0; i < n; ++i)
    if (sims[i] && cudaStreamSynchronize(sims[i]->ctx->stream) != cudaSuccess) return GEV_ECUDA;
  return GEV_OK;
}

}  // extern "C"

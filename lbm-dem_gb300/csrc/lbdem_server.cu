// Impact-run server: many independent runs resident on one GPU at once.
//
// Jobs (a configuration and a number of goCycles) queue in submission order
// and are admitted while their device footprint (lbdem_estimate_device_bytes)
// fits the memory budget and a run slot is free. Each admitted job is one
// lbdem context with its own stream; a job that ends frees its memory
// (stream-ordered, no device-wide wait) for the next one in the queue.
// Results carry the submit, start and end times for latency statistics.
//
// Runs advance by slices of cycles, each on its own stream with its own
// graphs. On request (batch_runs > 0), runs in their steady cycle with the
// same switches form batch groups of up to batch_runs runs instead: one launch per kernel
// advances all runs of a group (grid z = run, each run's records in a device
// array), two cycles captured in one CUDA graph, rebuilt whenever the
// group's members change. Each group has its own stream, so the phases of
// different groups overlap on the device (a group's latency-bound phases,
// such as the DEM gather, leave room for another group's lattice step). A
// run is taken into or out of a group only while neither it nor the group
// has work in flight (a new run's initialisation counts as its first work in
// flight), so no cross-stream ordering is needed. Runs outside
// the groups (their first cycles, an odd last cycle) advance on their own
// streams.
//
// Every slice (and a run's initialisation) ends with a copy of the run's
// device error bits into a pinned word; when the slice is seen complete, a
// set bit (a non-finite value, a sphere driven out of the domain, a list
// overflow) ends that run there with its status and message, and the others
// carry on.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <string>
#include <thread>
#include <vector>

#include "kernels_decl.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  int64_t id = 0;
  lbdem_config cfg{};
  std::vector<lbdem_particle_in> parts;
  std::vector<lbdem_object_in> objs;
  std::string restartFile;
  int32_t cycles = 0;
  int32_t done = 0;
  int64_t bytes = 0;
  double submitTime = 0.0, startTime = 0.0;
  lbdem_ctx* ctx = nullptr;
  cudaEvent_t sliceDone = nullptr;
  int* err = nullptr;  // its device error bits, read back after each slice
  int errSlot = -1;    // (a slot of the server's pinned error words)
  bool inFlight = false;
  bool counted = false;  // its bytes are part of the server's memory in use
  bool batched = false;  // a member of a batch group
  int32_t batchedCycles = 0;
};

}  // namespace

struct lbdem_server {
  lbdem_server_options opt{};
  std::string err;
  Clock::time_point origin;
  int64_t budget = 0, used = 0, nextId = 1;
  std::deque<Job*> pending;
  std::vector<Job*> active;
  std::deque<lbdem_job_result> finished;
  // batch groups
  struct Group {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    lbdem::JobArgs* dJobs = nullptr;  // 2 records per member: cycle 1, cycle 2
    std::vector<lbdem::JobArgs> hJobs;
    cudaGraphExec_t graph = nullptr;
    std::vector<Job*> members;
    bool inFlight = false;
  };
  std::vector<Group> groups;
  int groupRuns = 0;
  // one pinned word per run slot: a run's device error bits, copied after
  // each of its slices, so that a diverged run ends at that slice
  int* errPool = nullptr;
  std::vector<int> errFree;
  double now() const {
    return std::chrono::duration<double>(Clock::now() - origin).count();
  }
};

namespace {

// the message of the last failed lbdem_server_tune of this thread
thread_local std::string t_tuneErr;

int serverErr(lbdem_server* s, int code, const std::string& msg) {
  s->err = msg;
  return code;
}

void releaseJob(lbdem_server* s, Job* j) {
  if (j->errSlot >= 0) s->errFree.push_back(j->errSlot);
  if (j->sliceDone) cudaEventDestroy(j->sliceDone);
  if (j->ctx) lbdem_destroy(j->ctx);
  if (j->counted) s->used -= j->bytes;
  delete j;
}

// End a job: its state after the last slice (or the failing status, whose
// description becomes the server's last error).
void finishJob(lbdem_server* s, Job* j, int status, const char* where = nullptr) {
  if (status != LBDEM_OK) {
    std::string m = "job " + std::to_string(j->id) + " failed";
    if (where) m += std::string(" in ") + where;
    if (j->ctx && !j->ctx->err.empty()) m += ": " + j->ctx->err;
    const cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) m += std::string(" (CUDA: ") + cudaGetErrorString(e) + ")";
    s->err = m;
  }
  lbdem_job_result r;
  std::memset(&r, 0, sizeof r);
  r.job_id = j->id;
  r.status = status;
  r.cycles = j->done;
  r.batched_cycles = j->batchedCycles;
  r.submit_time = j->submitTime;
  r.start_time = j->startTime;
  r.device_bytes = j->bytes;
  if (status == LBDEM_OK && j->ctx) {
    int rc = lbdem_sync(j->ctx);
    if (rc == LBDEM_OK && j->cfg.n_objects > 0) {
      std::vector<double> x0(3 * j->cfg.n_objects), x1(3 * j->cfg.n_objects);
      lbdem_object_view v;
      std::memset(&v, 0, sizeof v);
      v.x0 = x0.data();
      v.x1 = x1.data();
      rc = lbdem_download_objects(j->ctx, &v);
      for (int c = 0; c < 3; ++c) {
        r.impactor_x0[c] = x0[c];
        r.impactor_x1[c] = x1[c];
      }
    }
    if (rc == LBDEM_OK) {
      int64_t ni = 0, na = 0;
      rc = lbdem_mass_summary(j->ctx, &r.fluid_mass, &ni, &na);
    }
    if (rc == LBDEM_OK) {
      lbdem_profile p;
      rc = lbdem_profile_read(j->ctx, &p, 0);
      r.active_node_updates = p.active_node_updates;
    }
    r.status = rc;
    if (rc != LBDEM_OK)
      s->err = "job " + std::to_string(j->id) + " failed at its end: " + j->ctx->err;
  }
  r.end_time = s->now();
  s->finished.push_back(r);
  releaseJob(s, j);
}

// Admit queued jobs, in order, while memory and run slots allow. Creating a
// run blocks the host for its initialisation (about a millisecond for a
// small run), so while runs are in progress admission stops after 2 ms of a
// turn and the resident runs get their next slices.
void admit(lbdem_server* s) {
  const bool busy = !s->active.empty();
  const double t0 = s->now();
  int admitted = 0;
  while (!s->pending.empty() && (int)s->active.size() < s->opt.max_active &&
         !(busy && admitted >= 1 && s->now() - t0 > 2e-3)) {
    Job* j = s->pending.front();
    if (s->used + j->bytes > s->budget && !s->active.empty()) break;
    s->pending.pop_front();
    lbdem_options o;
    std::memset(&o, 0, sizeof o);
    o.precision = s->opt.precision;
    o.device = s->opt.device;
    o.chunks_per_block = s->opt.chunks_per_block;
    // the run's initialisation overlaps the other runs' work; its device
    // errors are read back behind it and end the run when it completes
    o.async_init = 1;
    j->startTime = s->now();
    int rc = lbdem_create(&j->cfg, &o, &j->ctx);
    if (rc == LBDEM_OK && cudaEventCreateWithFlags(&j->sliceDone, cudaEventDisableTiming) !=
                              cudaSuccess)
      rc = LBDEM_ERR_CUDA;
    if (rc == LBDEM_OK) {  // a free error word (max_active of them, one per resident run)
      j->errSlot = s->errFree.back();
      s->errFree.pop_back();
      j->err = s->errPool + j->errSlot;
      *j->err = 0;
      rc = lbdemEnqueueErrorRead(j->ctx, j->err, j->ctx->stream);
    }
    // the run's initialisation is work in flight on its own stream: until it
    // completes the run neither joins a group (whose launches run on the
    // group's stream, unordered with the run's own) nor gets a slice
    if (rc == LBDEM_OK && cudaEventRecord(j->sliceDone, j->ctx->stream) != cudaSuccess)
      rc = LBDEM_ERR_CUDA;
    if (rc != LBDEM_OK) {
      finishJob(s, j, rc, "its initialisation");
      continue;
    }
    j->inFlight = true;
    s->used += j->bytes;
    j->counted = true;
    s->active.push_back(j);
    ++admitted;
  }
}

// Capture two batched cycles of group g's members (their records uploaded
// first) into g.graph.
int buildGroupGraph(lbdem_server* s, lbdem_server::Group& g) {
  if (g.graph) {
    cudaGraphExecDestroy(g.graph);
    g.graph = nullptr;
  }
  const size_t n = g.members.size();
  g.hJobs.resize(2 * n);
  std::vector<lbdem_ctx*> runs;
  for (size_t i = 0; i < n; ++i) {
    lbdem_ctx* c = g.members[i]->ctx;
    runs.push_back(c);
    lbdemJobArgs(c, c->cur, &g.hJobs[i]);
    lbdemJobArgs(c, 1 - c->cur, &g.hJobs[n + i]);
  }
  if (cudaMemcpyAsync(g.dJobs, g.hJobs.data(), 2 * n * sizeof(lbdem::JobArgs),
                      cudaMemcpyHostToDevice, g.stream) != cudaSuccess)
    return serverErr(s, LBDEM_ERR_CUDA, "batch records upload");
  cudaGraph_t graph = nullptr;
  if (cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return serverErr(s, LBDEM_ERR_CUDA, "batch graph capture");
  int rc = lbdemEnqueueBatchCycle(runs, g.dJobs, g.stream);
  if (rc == LBDEM_OK) rc = lbdemEnqueueBatchCycle(runs, g.dJobs + n, g.stream);
  const cudaError_t e = cudaStreamEndCapture(g.stream, &graph);
  if (rc != LBDEM_OK || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return serverErr(s, rc ? rc : LBDEM_ERR_CUDA, "batch graph capture");
  }
  const cudaError_t ei = cudaGraphInstantiate(&g.graph, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) return serverErr(s, LBDEM_ERR_CUDA, "batch graph instantiate");
  return LBDEM_OK;
}

void dropJob(lbdem_server* s, Job* j, int status, const char* where = nullptr) {
  j->batched = false;
  for (size_t q = 0; q < s->active.size(); ++q)
    if (s->active[q] == j) {
      s->active.erase(s->active.begin() + q);
      break;
    }
  finishJob(s, j, status, where);
}

// A group's turn: when its last slice is done, members that cannot take two
// more steady cycles leave, idle batchable runs join (up to groupRuns, with
// the group's switches), and the next slice (an even number of cycles) is
// enqueued as graph replays on the group's stream.
bool progressGroup(lbdem_server* s, lbdem_server::Group& g) {
  if (g.inFlight) {
    const cudaError_t e = cudaEventQuery(g.done);
    if (e == cudaErrorNotReady) return false;
    g.inFlight = false;
    if (e != cudaSuccess) {
      const std::string where = "a shared-launch group of " + std::to_string(g.members.size()) +
                                " runs (" + cudaGetErrorString(e) + ")";
      for (Job* j : g.members) dropJob(s, j, LBDEM_ERR_CUDA, where.c_str());
      g.members.clear();
      return true;
    }
  }
  // members whose error bits came back set end at this slice; the group's
  // graph is then rebuilt without them
  bool dropped = false;
  for (size_t q = 0; q < g.members.size();) {
    Job* j = g.members[q];
    if (!*j->err) {
      ++q;
      continue;
    }
    g.members.erase(g.members.begin() + q);
    dropJob(s, j, lbdemErrorStatus(j->ctx, *j->err, " after a slice"), "a shared-launch slice");
    dropped = true;
  }
  auto fits = [&](Job* j, int key) {
    return j->cycles - j->done >= 2 && lbdemBatchable(j->ctx) &&
           lbdemBatchKey(j->ctx) == key;
  };
  std::vector<Job*> next;
  int key = g.members.empty() ? -1 : lbdemBatchKey(g.members[0]->ctx);
  for (Job* j : g.members)
    if (fits(j, key)) next.push_back(j);
  if (next.empty()) key = -1;
  for (Job* j : g.members) j->batched = false;
  for (Job* j : s->active) {
    if ((int)next.size() >= s->groupRuns) break;
    if (j->batched || j->inFlight || j->cycles - j->done < 2 || !lbdemBatchable(j->ctx) ||
        std::find(next.begin(), next.end(), j) != next.end())
      continue;
    if (key < 0) key = lbdemBatchKey(j->ctx);
    if (lbdemBatchKey(j->ctx) == key) next.push_back(j);
  }
  const bool changed = dropped || next != g.members;
  g.members = next;
  for (Job* j : g.members) j->batched = true;
  if (changed && !g.members.empty() && buildGroupGraph(s, g) != LBDEM_OK) {
    for (Job* j : g.members) j->batched = false;
    g.members.clear();
    return true;
  }
  if (g.members.empty()) return changed;
  int slice = s->opt.slice_cycles & ~1;
  if (slice < 2) slice = 2;
  for (Job* j : g.members) slice = std::min(slice, (j->cycles - j->done) & ~1);
  for (int c = 0; c < slice; c += 2)
    if (cudaGraphLaunch(g.graph, g.stream) != cudaSuccess) {
      serverErr(s, LBDEM_ERR_CUDA, "batch graph launch");
      break;
    }
  for (Job* j : g.members) lbdemEnqueueErrorRead(j->ctx, j->err, g.stream);
  cudaEventRecord(g.done, g.stream);
  for (Job* j : g.members) {
    j->done += slice;
    j->batchedCycles += slice;
    lbdemAdvanceCounters(j->ctx, slice);
  }
  g.inFlight = true;
  return true;
}

// One pass over the running jobs: the groups' turns, then the runs outside
// them: finished slices are noticed, jobs that reached their cycle count end,
// the others get their next slice. Returns whether anything changed.
bool progress(lbdem_server* s) {
  bool changed = false;
  for (auto& g : s->groups) changed = progressGroup(s, g) || changed;
  for (size_t q = 0; q < s->active.size();) {
    Job* j = s->active[q];
    if (j->batched) {
      ++q;
      continue;
    }
    // a run that fits a group waits for a group's next turn
    if (!s->groups.empty() && !j->inFlight && j->cycles - j->done >= 2 &&
        lbdemBatchable(j->ctx)) {
      ++q;
      continue;
    }
    if (j->inFlight) {
      const cudaError_t e = cudaEventQuery(j->sliceDone);
      if (e == cudaErrorNotReady) {
        ++q;
        continue;
      }
      j->inFlight = false;
      changed = true;
      if (e != cudaSuccess) {
        s->active.erase(s->active.begin() + q);
        const std::string where = std::string("its own slice (") + cudaGetErrorString(e) + ")";
        finishJob(s, j, LBDEM_ERR_CUDA, where.c_str());
        continue;
      }
      if (*j->err) {  // diverged (or overflowed): the run ends at this slice
        s->active.erase(s->active.begin() + q);
        finishJob(s, j, lbdemErrorStatus(j->ctx, *j->err, " after a slice"), "a slice");
        continue;
      }
      // now idle: a run that fits a group waits for the group's next turn
      if (!s->groups.empty() && j->cycles - j->done >= 2 && lbdemBatchable(j->ctx)) {
        ++q;
        continue;
      }
    }
    if (j->done >= j->cycles) {
      s->active.erase(s->active.begin() + q);
      finishJob(s, j, LBDEM_OK);
      changed = true;
      continue;
    }
    const int32_t n = std::min(s->opt.slice_cycles, j->cycles - j->done);
    int rc = lbdem_cycle(j->ctx, n);
    if (rc == LBDEM_OK) rc = lbdemEnqueueErrorRead(j->ctx, j->err, j->ctx->stream);
    if (rc == LBDEM_OK && cudaEventRecord(j->sliceDone, j->ctx->stream) != cudaSuccess)
      rc = LBDEM_ERR_CUDA;
    if (rc != LBDEM_OK) {
      s->active.erase(s->active.begin() + q);
      finishJob(s, j, rc, "enqueueing its slice");
      changed = true;
      continue;
    }
    j->done += n;
    j->inFlight = true;
    changed = true;
    ++q;
  }
  return changed;
}

}  // namespace

extern "C" int lbdem_server_create(const lbdem_server_options* opt, lbdem_server** out) {
  if (!opt || !out) return LBDEM_ERR_INVALID;
  *out = nullptr;
  if (opt->precision != LBDEM_PLAIN_FP64 && opt->precision != LBDEM_MIXED)
    return LBDEM_ERR_INVALID;
  if (opt->max_active < 1 || opt->slice_cycles < 1) return LBDEM_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return LBDEM_ERR_NO_DEVICE;
  if (opt->device < 0 || opt->device >= ndev) return LBDEM_ERR_INVALID;
  if (cudaSetDevice(opt->device) != cudaSuccess) return LBDEM_ERR_CUDA;
  lbdem_server* s = new lbdem_server();
  s->opt = *opt;
  s->origin = Clock::now();
  if (opt->batch_runs > 0) {
    s->groupRuns = opt->batch_runs;
    const int ng = (opt->max_active + s->groupRuns - 1) / s->groupRuns;
    s->groups.resize(ng);
    for (auto& g : s->groups) {
      lbdemNoteDeviceAllocation();
      if (cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming) != cudaSuccess ||
          cudaMalloc(&g.dJobs, 2 * (size_t)s->groupRuns * sizeof(lbdem::JobArgs)) !=
              cudaSuccess) {
        lbdem_server_destroy(s);
        return LBDEM_ERR_CUDA;
      }
    }
  }
  if (cudaHostAlloc(&s->errPool, sizeof(int) * (size_t)opt->max_active, cudaHostAllocDefault) !=
      cudaSuccess) {
    s->errPool = nullptr;
    lbdem_server_destroy(s);
    return LBDEM_ERR_CUDA;
  }
  for (int i = opt->max_active - 1; i >= 0; --i) s->errFree.push_back(i);
  s->budget = opt->device_budget_bytes;
  if (s->budget <= 0) {
    size_t freeB = 0, totalB = 0;
    if (cudaMemGetInfo(&freeB, &totalB) != cudaSuccess) {
      lbdem_server_destroy(s);
      return LBDEM_ERR_CUDA;
    }
    s->budget = (int64_t)(0.9 * (double)freeB);
  }
  *out = s;
  return LBDEM_OK;
}

extern "C" int lbdem_server_submit(lbdem_server* s, const lbdem_config* cfg, int32_t cycles,
                                   int64_t* job_id) {
  if (!s || !cfg || cycles < 0) return LBDEM_ERR_INVALID;
  if (cfg->n_particles < 0 || (cfg->n_particles > 0 && !cfg->particles) ||
      cfg->n_objects < 0 || (cfg->n_objects > 0 && !cfg->objects))
    return serverErr(s, LBDEM_ERR_INVALID, "configuration tables missing");
  int64_t bytes = 0;
  int rc = lbdem_estimate_device_bytes(cfg, s->opt.precision, &bytes);
  if (rc) return serverErr(s, rc, "cannot size the run's lattice");
  if (bytes > s->budget)
    return serverErr(s, LBDEM_ERR_OOM,
                     "run needs " + std::to_string(bytes) + " device bytes, budget is " +
                         std::to_string(s->budget));
  Job* j = new Job();
  j->id = s->nextId++;
  j->cfg = *cfg;
  j->parts.assign(cfg->particles, cfg->particles + cfg->n_particles);
  j->objs.assign(cfg->objects, cfg->objects + cfg->n_objects);
  j->cfg.particles = j->parts.empty() ? nullptr : j->parts.data();
  j->cfg.objects = j->objs.empty() ? nullptr : j->objs.data();
  j->restartFile = cfg->lbRestartFile ? cfg->lbRestartFile : "";
  j->cfg.lbRestartFile = cfg->lbRestartFile ? j->restartFile.c_str() : nullptr;
  j->cycles = cycles;
  j->bytes = bytes;
  j->submitTime = s->now();
  s->pending.push_back(j);
  if (job_id) *job_id = j->id;
  return LBDEM_OK;
}

extern "C" int lbdem_server_poll(lbdem_server* s, double wait_seconds, lbdem_job_result* out,
                                 int32_t max_out, int32_t* n_out) {
  if (!s || (max_out > 0 && !out) || !n_out) return LBDEM_ERR_INVALID;
  *n_out = 0;
  if (cudaSetDevice(s->opt.device) != cudaSuccess) return LBDEM_ERR_CUDA;
  const double until = s->now() + (wait_seconds > 0.0 ? wait_seconds : 0.0);
  for (;;) {
    admit(s);
    const bool changed = progress(s);
    if (!s->finished.empty() || (s->pending.empty() && s->active.empty()) || s->now() >= until)
      break;
    if (!changed) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  while (*n_out < max_out && !s->finished.empty()) {
    out[(*n_out)++] = s->finished.front();
    s->finished.pop_front();
  }
  return LBDEM_OK;
}

extern "C" int lbdem_server_status(const lbdem_server* s, int32_t* queued, int32_t* running,
                                   int32_t* unread, int64_t* device_bytes_in_use) {
  if (!s) return LBDEM_ERR_INVALID;
  if (queued) *queued = (int32_t)s->pending.size();
  if (running) *running = (int32_t)s->active.size();
  if (unread) *unread = (int32_t)s->finished.size();
  if (device_bytes_in_use) *device_bytes_in_use = s->used;
  return LBDEM_OK;
}

extern "C" const char* lbdem_server_last_error(const lbdem_server* s) {
  return s ? s->err.c_str() : t_tuneErr.c_str();
}

extern "C" void lbdem_server_destroy(lbdem_server* s) {
  if (!s) return;
  cudaSetDevice(s->opt.device);
  for (auto& g : s->groups) {
    if (g.stream) cudaStreamSynchronize(g.stream);
    if (g.graph) cudaGraphExecDestroy(g.graph);
    if (g.done) cudaEventDestroy(g.done);
    if (g.dJobs) cudaFree(g.dJobs);
    if (g.stream) cudaStreamDestroy(g.stream);
  }
  for (Job* j : s->active) releaseJob(s, j);
  for (Job* j : s->pending) delete j;
  if (s->errPool) cudaFreeHost(s->errPool);
  delete s;
}

extern "C" int lbdem_server_tune(lbdem_server_options* opt, const lbdem_config* const* cfgs,
                                 int32_t n, int32_t cycles, double* best_seconds) {
  if (!opt || !cfgs || n < 1 || cycles < 1) return LBDEM_ERR_INVALID;
  t_tuneErr.clear();
  const int32_t batchC[] = {0, 2, 4, 8};
  const int32_t chunkC[] = {8, 32};
  double best = -1.0;
  int32_t bestB = 0, bestC = 8;
  for (int32_t b : batchC)
    for (int32_t c : chunkC) {
      lbdem_server_options o = *opt;
      o.batch_runs = b;
      o.chunks_per_block = c;
      if (o.max_active < n) o.max_active = n;
      lbdem_server* s = nullptr;
      int rc = lbdem_server_create(&o, &s);
      if (rc != LBDEM_OK) return rc;
      const auto t0 = Clock::now();
      for (int32_t i = 0; i < n && rc == LBDEM_OK; ++i)
        rc = lbdem_server_submit(s, cfgs[i], cycles, nullptr);
      int32_t done = 0;
      std::vector<lbdem_job_result> res(n);
      while (rc == LBDEM_OK && done < n) {
        int32_t got = 0;
        rc = lbdem_server_poll(s, 0.05, res.data() + done, n - done, &got);
        for (int32_t i = done; i < done + got; ++i)
          if (res[i].status != LBDEM_OK) rc = res[i].status;
        done += got;
      }
      const double t = std::chrono::duration<double>(Clock::now() - t0).count();
      if (rc != LBDEM_OK)
        t_tuneErr = "schedule batch_runs " + std::to_string(b) + ", chunks_per_block " +
                    std::to_string(c) + ": " + s->err;
      lbdem_server_destroy(s);
      if (rc != LBDEM_OK) return rc;
      if (best < 0.0 || t < best) {
        best = t;
        bestB = b;
        bestC = c;
      }
    }
  opt->batch_runs = bestB;
  opt->chunks_per_block = bestC;
  if (best_seconds) *best_seconds = best;
  return LBDEM_OK;
}

// Render server: continuous batching of render jobs over one batch engine.
//
// No counterpart in the reference, which renders one job at a time.  Callers
// on any thread submit jobs (a scene already resident in device memory, the
// render parameters, a camera and a pass); a worker thread admits them in
// arrival order while the device memory budget (the batch's path state plus
// the films of the admitted jobs) and the job table allow, gives each a film,
// merges its samples into the shared wavefront (bling_batch_submit), runs
// a few wavefront iterations at a time, and hands every finished film back to
// its waiter.  Jobs that arrive while others run join the queues at the next
// admission round, between two steps.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "handles.h"

using namespace bgpu;

namespace {

enum JobState { J_PENDING = 0, J_RUNNING = 1, J_DONE = 2, J_FAILED = 3 };

struct ServerJob {
  int64_t ticket = 0;
  bling_scene* scene = nullptr;
  bling_render_params params{};
  bling_camera_desc camera{};
  uint64_t pass = 0;
  uint64_t bytes = 0;    // film bytes on the device
  uint64_t samples = 0;  // path samples of the job
  int state = J_PENDING;
  int rc = BLING_OK;
  std::string err;
  float* d_film = nullptr;
  int scene_idx = -1;          // the scene's batch table index
  uint64_t sent = 0;           // samples of the pass handed to the batch, in slices
  std::vector<int64_t> slices; // batch job ids of the slices
  std::vector<float> result;  // (w, X, Y, Z) per pixel once done
  double t_submit = 0, t_admit = 0, t_done = 0;
};

}  // namespace

struct bling_server {
  bling_ctx* ctx = nullptr;
  BatchEngine* eng = nullptr;
  uint64_t budget = 0;      // bytes for path state + films
  uint64_t base_bytes = 0;  // the batch's path state
  uint64_t in_use = 0;      // base_bytes + films of admitted jobs
  int iters_per_step = 4;
  int max_jobs = 1024;
  int64_t fail_after = -1;  // test hook: the step after this many more steps fails (-1: none)
  uint64_t slice = 1 << 20;    // samples per slice handed to the batch
  uint64_t backlog = 1 << 21;  // submitted but unstarted samples kept queued
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::deque<ServerJob*> pending;
  std::vector<ServerJob*> running;
  std::unordered_map<int64_t, std::unique_ptr<ServerJob>> jobs;
  int64_t next_ticket = 0;
  bling_server_stats stats{};
  std::string err;
  std::thread worker;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

uint64_t samplesOf(const bling_render_params& p) {
  // the filter-padded sample extent (imageWindow', Image.hs:170-176)
  float fw = p.filter_kind == BLING_FILTER_BOX ? 0.5f : p.filter_params[0];
  float fh = p.filter_kind == BLING_FILTER_BOX ? 0.5f : p.filter_params[1];
  int64_t nx = (int64_t)floorf(0.5f + (float)p.width + fw) - (int64_t)floorf(0.5f - fw) + 1;
  int64_t ny = (int64_t)floorf(0.5f + (float)p.height + fh) - (int64_t)floorf(0.5f - fh) + 1;
  return (uint64_t)(nx * ny) * (uint64_t)(p.strata_x * p.strata_y);
}

void failJob(ServerJob* j, int rc, const std::string& msg) {
  j->state = J_FAILED;
  j->rc = rc;
  j->err = msg;
}

// the job with the fewest samples left to hand out, or null
ServerJob* shortestUnsent(const std::vector<ServerJob*>& running) {
  ServerJob* best = nullptr;
  for (ServerJob* j : running) {
    if (j->state != J_RUNNING || j->sent >= j->samples) continue;
    if (!best || j->samples - j->sent < best->samples - best->sent) best = j;
  }
  return best;
}

// one admission round and one step of the batch; called without S->mu held.
// Admitted jobs get a film and their scene's batch index; their samples go
// to the batch in slices of at most S->slice, shortest remaining job first,
// while fewer than S->backlog submitted samples wait for a free path slot.
// A job that arrives while a long one runs therefore starts within about
// one backlog of samples, and its work shares the wavefront with the rest.
void serveRound(bling_server* S, std::vector<ServerJob*>& admit, std::vector<ServerJob*>& running,
                std::vector<ServerJob*>& finished) {
  bling_ctx* c = S->ctx;
  std::lock_guard<std::mutex> g(c->mu);
  cudaSetDevice(c->device);
  std::string err;
  for (ServerJob* j : admit) {
    j->t_admit = S->now();
    cudaError_t e = cudaMalloc(&j->d_film, j->bytes);
    if (e != cudaSuccess) {
      j->d_film = nullptr;
      failJob(j, BLING_ERR_OOM, std::string("film allocation: ") + cudaGetErrorString(e));
      finished.push_back(j);
      continue;
    }
    e = cudaMemsetAsync(j->d_film, 0, j->bytes, c->stream);
    int rc = e == cudaSuccess ? BLING_OK : BLING_ERR_CUDA;
    if (rc == BLING_OK)
      rc = batch_scene(S->eng, j->scene->serial, j->scene->accel, j->scene->shading, j->scene->lo,
                       j->scene->hi, j->scene_idx, err);
    if (rc != BLING_OK) {
      cudaFree(j->d_film);
      j->d_film = nullptr;
      failJob(j, rc, err.empty() ? cudaGetErrorString(e) : err);
      finished.push_back(j);
      continue;
    }
    j->state = J_RUNNING;
    running.push_back(j);
  }
  if (running.empty()) return;
  BatchStats bs;
  batch_stats(S->eng, bs);
  uint64_t queued = bs.samples_submitted - bs.samples_started;
  while (queued < S->backlog) {
    ServerJob* j = shortestUnsent(running);
    if (!j) break;
    uint64_t n = std::min<uint64_t>(S->slice, j->samples - j->sent);
    int64_t id = -1;
    int rc = batch_submit(S->eng, j->scene_idx, j->camera, j->d_film, j->params.width,
                          j->params.height, j->params, j->pass, id, err, j->sent, n);
    if (rc == BLING_ERR_STATE) break;  // job table full until slices complete
    if (rc != BLING_OK) {
      // no further slices; the job fails once its slices in flight are done
      j->rc = rc;
      j->err = err;
      j->sent = j->samples;
      continue;
    }
    j->slices.push_back(id);
    j->sent += n;
    queued += n;
  }
  int rc;
  bool inject = false;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->fail_after == 0) inject = true;
    if (S->fail_after >= 0) S->fail_after -= 1;
  }
  if (inject) {
    rc = BLING_ERR_CUDA;
    err = "injected step failure (bling_server_debug_fail_step)";
  } else {
    rc = batch_step(S->eng, S->iters_per_step, err);
  }
  if (rc != BLING_OK) {
    // the engine's job table and paths in flight still point at the running
    // jobs' films: drop them before the films are released, so that no later
    // step writes into freed (and possibly reused) memory
    std::string cerr;
    if (batch_cancel(S->eng, cerr) != BLING_OK) err += "; cancelling the batch: " + cerr;
    for (ServerJob* j : running) {
      failJob(j, rc, err);
      if (j->d_film) cudaFree(j->d_film);
      j->d_film = nullptr;
      finished.push_back(j);
    }
    running.clear();
    return;
  }
  std::vector<ServerJob*> still;
  for (ServerJob* j : running) {
    bool done = j->sent >= j->samples;
    for (size_t k = 0; done && k < j->slices.size(); k++) {
      uint64_t d = 0, t = 0;
      batch_job_status(S->eng, j->slices[k], d, t, err);
      done = d >= t;
    }
    if (!done) {
      still.push_back(j);
      continue;
    }
    if (j->rc != BLING_OK) {
      failJob(j, j->rc, j->err);
    } else {
      j->result.resize(j->bytes / sizeof(float));
      cudaError_t e = cudaMemcpy(j->result.data(), j->d_film, j->bytes, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess)
        failJob(j, BLING_ERR_CUDA, std::string("film copy: ") + cudaGetErrorString(e));
      else
        j->state = J_DONE;
    }
    cudaFree(j->d_film);
    j->d_film = nullptr;
    j->t_done = S->now();
    finished.push_back(j);
  }
  running.swap(still);
}

void workerLoop(bling_server* S) {
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_work.wait(lk, [&] { return S->stop || !S->pending.empty() || !S->running.empty(); });
    if (S->stop && S->running.empty()) break;
    std::vector<ServerJob*> admit;
    if (!S->stop) {
      // smallest jobs first (ties in arrival order)
      std::stable_sort(S->pending.begin(), S->pending.end(),
                       [](const ServerJob* a, const ServerJob* b) { return a->samples < b->samples; });
      while (!S->pending.empty()) {
        ServerJob* j = S->pending.front();
        if (S->in_use + j->bytes > S->budget) break;
        if (S->running.size() + admit.size() >= (size_t)S->max_jobs) break;
        S->in_use += j->bytes;
        admit.push_back(j);
        S->pending.pop_front();
      }
    }
    std::vector<ServerJob*> running = S->running;
    lk.unlock();
    std::vector<ServerJob*> finished;
    serveRound(S, admit, running, finished);
    lk.lock();
    S->running = running;
    for (ServerJob* j : finished) {
      S->in_use -= j->bytes;
      if (j->state == J_DONE) {
        S->stats.jobs_done += 1;
        S->stats.samples_done += j->samples;
      } else {
        S->stats.jobs_failed += 1;
      }
    }
    S->stats.jobs_admitted += (int64_t)admit.size();
    S->stats.jobs_running = (int64_t)S->running.size();
    S->stats.jobs_pending = (int64_t)S->pending.size();
    S->stats.bytes_in_use = S->in_use;
    S->stats.peak_bytes_in_use = std::max(S->stats.peak_bytes_in_use, S->in_use);
    if (!finished.empty()) S->cv_done.notify_all();
  }
  // stopped: pending jobs are not run
  for (ServerJob* j : S->pending) failJob(j, BLING_ERR_STATE, "server stopped");
  S->pending.clear();
  S->cv_done.notify_all();
}

}  // namespace

extern "C" {

int bling_server_create(bling_ctx* c, const bling_server_opts* o, bling_server** out) {
  if (!c || !out) return BLING_ERR_INVALID_ARG;
  *out = nullptr;
  std::unique_ptr<bling_server> S(new bling_server());
  S->ctx = c;
  BatchConfig cfg;
  cfg.graph_mode = BLING_BATCH_GRAPH;
  uint64_t budget = uint64_t(40) << 30;
  if (o) {
    const bling_batch_opts& b = o->batch;
    if (b.slots) cfg.slots = b.slots;
    if (b.block_size) cfg.block = b.block_size;
    if (b.max_jobs) cfg.max_jobs = b.max_jobs;
    cfg.sort_rays = b.sort_rays != 0;
    if (b.graph_mode) cfg.graph_mode = b.graph_mode;
    if (b.iters_per_launch) cfg.iters_per_launch = b.iters_per_launch;
    cfg.max_run_iterations = b.max_run_iterations > 0 ? b.max_run_iterations : 0;
    if (o->hbm_budget_bytes) budget = o->hbm_budget_bytes;
    if (o->iters_per_step > 0) S->iters_per_step = o->iters_per_step;
  }
  S->max_jobs = cfg.max_jobs;
  // slices of half the path slots; queued ahead of the wavefront, enough
  // samples to refill every slot in each iteration of a step
  S->slice = std::max<uint64_t>(uint64_t(1) << 12, (uint64_t)cfg.slots / 2);
  S->backlog = std::max<uint64_t>(S->slice, (uint64_t)cfg.slots * (uint64_t)S->iters_per_step);
  {
    std::lock_guard<std::mutex> g(c->mu);
    if (!c->stream) {
      c->err = "context has no device";
      return BLING_ERR_STATE;
    }
    cudaSetDevice(c->device);
    int rc = batch_create(c->device, c->stream, cfg, &S->eng, c->err);
    if (rc) return rc;
    BatchStats bs;
    batch_stats(S->eng, bs);
    S->base_bytes = (uint64_t)bs.device_bytes;
    if (S->base_bytes >= budget) {
      batch_destroy(S->eng);
      c->err = "the budget does not cover the batch's path state";
      return BLING_ERR_BOUNDS;
    }
  }
  S->budget = budget;
  S->in_use = S->base_bytes;
  S->stats.budget_bytes = budget;
  S->stats.bytes_in_use = S->in_use;
  S->stats.peak_bytes_in_use = S->in_use;
  S->t0 = std::chrono::steady_clock::now();
  bling_server* raw = S.get();
  S->worker = std::thread(workerLoop, raw);
  *out = S.release();
  return BLING_OK;
}

void bling_server_destroy(bling_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  {
    std::lock_guard<std::mutex> g(S->ctx->mu);
    cudaSetDevice(S->ctx->device);
    batch_destroy(S->eng);
  }
  delete S;
}

int bling_server_submit(bling_server* S, bling_scene* s, const bling_render_params* p,
                        const bling_camera_desc* camera, uint64_t pass, int64_t* ticket) {
  if (!S || !s || !p || !ticket) return BLING_ERR_INVALID_ARG;
  if (s->ctx != S->ctx) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->err = "scene belongs to another context";
    return BLING_ERR_INVALID_ARG;
  }
  // validation touches no shared state: a submission never waits for the
  // worker, which holds the context lock while the device runs a step
  std::string perr;
  int prc = validate_render_params(p, perr);
  if (prc) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->err = perr;
    return prc;
  }
  std::unique_ptr<ServerJob> j(new ServerJob());
  j->scene = s;
  j->params = *p;
  j->camera = camera ? *camera : s->shading.camera;
  j->pass = pass;
  j->bytes = (uint64_t)p->width * (uint64_t)p->height * 16;
  j->samples = samplesOf(*p);
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stop) {
    S->err = "server stopped";
    return BLING_ERR_STATE;
  }
  if (S->base_bytes + j->bytes > S->budget) {
    S->err = "the job's film does not fit the budget";
    return BLING_ERR_BOUNDS;
  }
  j->ticket = S->next_ticket++;
  j->t_submit = S->now();
  *ticket = j->ticket;
  S->pending.push_back(j.get());
  S->jobs[j->ticket] = std::move(j);
  S->stats.jobs_submitted += 1;
  S->stats.jobs_pending = (int64_t)S->pending.size();
  S->cv_work.notify_one();
  return BLING_OK;
}

int bling_server_wait(bling_server* S, int64_t ticket, int32_t timeout_ms, float* host_wxyz,
                      bling_job_times* times) {
  if (!S) return BLING_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->jobs.find(ticket);
  if (it == S->jobs.end()) {
    S->err = "unknown ticket";
    return BLING_ERR_INVALID_ARG;
  }
  ServerJob* j = it->second.get();
  auto ready = [&] { return j->state == J_DONE || j->state == J_FAILED; };
  if (timeout_ms < 0) {
    S->cv_done.wait(lk, ready);
  } else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    S->err = "job not finished within the timeout";
    return BLING_ERR_TIMEOUT;
  }
  int rc = j->rc;
  if (j->state == J_DONE && host_wxyz)
    memcpy(host_wxyz, j->result.data(), j->result.size() * sizeof(float));
  if (times) {
    times->submitted = j->t_submit;
    times->admitted = j->t_admit;
    times->finished = j->t_done;
    times->samples = j->samples;
  }
  if (rc != BLING_OK) S->err = j->err;
  S->jobs.erase(it);
  return rc;
}

int bling_server_stats_get(bling_server* S, bling_server_stats* out) {
  if (!S || !out) return BLING_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    *out = S->stats;
  }
  BatchStats bs;
  {
    std::lock_guard<std::mutex> g(S->ctx->mu);
    batch_stats(S->eng, bs);
  }
  out->rays_closest = bs.rays_closest;
  out->rays_any = bs.rays_any;
  out->iterations = bs.iterations;
  return BLING_OK;
}

int bling_server_debug_fail_step(bling_server* S, int32_t after_steps) {
  if (!S || after_steps < -1) return BLING_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  S->fail_after = after_steps;
  return BLING_OK;
}

const char* bling_server_last_error(bling_server* S) {
  if (!S) return "null server";
  std::lock_guard<std::mutex> lk(S->mu);
  thread_local std::string copy;
  copy = S->err;
  return copy.c_str();
}

}  // extern "C"

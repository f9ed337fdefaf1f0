// fdtd_server.cu -- continuous batching of FDTD jobs on one GPU.
//
// The reference runs one simulation per MPI job.  A server here keeps many
// jobs resident on one GPU and advances them together:
//   * submitted jobs (built but not committed) wait in a FIFO queue;
//   * a job is admitted -- committed, i.e. its device memory allocated and
//     its tables uploaded -- when an active slot is free and its footprint
//     (fdtd_estimate_bytes) fits in what the server's HBM budget has left;
//   * every active job runs on its own stream and advances in chunks of
//     chunk_steps time steps (CUDA-graph replays of 32-step rings), so the
//     kernels of different jobs overlap on the device, and jobs join and
//     leave between chunks without stopping the others;
//   * small 2D jobs (at most pack_cells cells) of one precision and layout
//     are packed: one launch per part of a half step covers all of them
//     (fdtd::Pack), as each alone would leave most of the GPU idle; a packed
//     job leaves its pack when less than a ring of steps is left and
//     finishes on its own stream;
//   * a finished job keeps its memory until the caller has read its results
//     and released it.
// One host thread runs the loop.  It never waits on the device except
// through event queries, so a slow job does not hold up the others; commits
// (host set-up and uploads) run on worker threads, so they overlap the
// running jobs' GPU work.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "fdtd_gb300.h"
#include "fdtd_internal.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
  int64_t ticket = 0;
  fdtd_job *job = nullptr;
  int32_t n_steps = 0;
  uint64_t est = 0, bytes = 0;  // footprint: estimate before commit, held after
  int state = FDTD_REQ_QUEUED;
  int rc = FDTD_OK;
  char err[256] = {};
  int next_n = 1;
  bool inflight = false;
  long long key = -1;  // pack group, -1: runs alone
  bool in_pack = false;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  double t_submit = 0, t_admit = 0, t_done = 0;
};

}  // namespace

struct PackGroup {
  fdtd::Pack *pack = nullptr;
  std::vector<Req *> members;
  cudaEvent_t ev = nullptr;
  bool inflight = false;
};

struct fdtd_server {
  fdtd_server_desc d{};
  std::map<long long, PackGroup> groups;
  int device = 0;
  uint64_t budget = 0;
  double t0 = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::map<int64_t, Req *> reqs;
  std::deque<Req *> queue;
  std::vector<Req *> active;
  uint64_t held = 0, held_max = 0;
  int64_t next_ticket = 1;
  int64_t done_count = 0;
  int64_t packed_rings = 0, pack_builds = 0;
  double pack_build_s = 0;
  bool stop = false;
  std::thread th;
  // admitted jobs waiting for a commit worker
  std::deque<Req *> to_commit;
  int committing = 0;
  std::condition_variable cv_commit;
  std::vector<std::thread> workers;
};

namespace {

void finish(fdtd_server *S, Req *r, int rc, const char *why) {
  r->state = rc ? FDTD_REQ_FAILED : FDTD_REQ_DONE;
  r->rc = rc;
  if (rc && why) snprintf(r->err, sizeof r->err, "%s", why);
  r->t_done = now_s();
  ++S->done_count;
  S->cv_done.notify_all();
}

// admit queued jobs in order while slots and memory allow (lock held); a
// commit worker then sets them up
void admit(fdtd_server *S) {
  while (!S->queue.empty() && (int)S->active.size() + S->committing < S->d.max_active && !S->stop) {
    Req *r = S->queue.front();
    if (r->est > S->budget) {
      S->queue.pop_front();
      finish(S, r, FDTD_ENOMEM, "job footprint exceeds the server's HBM budget");
      continue;
    }
    if (S->held + r->est > S->budget) return;  // wait for memory to be released
    S->queue.pop_front();
    S->held += r->est;
    S->held_max = std::max(S->held_max, S->held);
    r->state = FDTD_REQ_RUNNING;
    ++S->committing;
    S->to_commit.push_back(r);
    S->cv_commit.notify_one();
  }
}

// commit worker: allocate and upload an admitted job, then hand it to the loop
void commit_worker(fdtd_server *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_commit.wait(lk, [S] { return S->stop || !S->to_commit.empty(); });
    if (S->stop) return;
    Req *r = S->to_commit.front();
    S->to_commit.pop_front();
    lk.unlock();
    char msg[256] = {};
    int rc = fdtd_set_stream(r->job, r->stream);
    if (!rc) rc = fdtd_commit(r->job);
    uint64_t real = r->est;
    if (!rc) rc = fdtd_device_bytes(r->job, &real);
    long long key = -1;
    if (!rc && S->d.pack_cells >= 0 && r->n_steps >= fdtd::kStageSteps && fdtd::pack_key(r->job) >= 0) {
      int64_t cells = 0;
      fdtd_kernel_cells(r->job, FDTD_KERNEL_E, &cells);
      if (cells <= (S->d.pack_cells ? S->d.pack_cells : (1 << 20)) && !fdtd::job_reserve(r->job, r->n_steps))
        key = fdtd::pack_key(r->job);
    }
    if (rc) fdtd_last_error(msg, sizeof msg);
    lk.lock();
    --S->committing;
    S->held -= r->est;
    if (rc) {
      finish(S, r, rc, msg);
    } else {
      r->bytes = std::max(real, r->est);
      S->held += r->bytes;
      S->held_max = std::max(S->held_max, S->held);
      r->t_admit = now_s();
      r->key = key;
      S->active.push_back(r);
    }
    S->cv_work.notify_one();
  }
}

// Advance the pack groups (lock held).  A group whose pack is idle takes in
// the packable active jobs with at least a ring of steps left, lets go of
// the others, rebuilds its pack when its members changed, and queues whole
// rings up to chunk_steps.
bool advance_packs(fdtd_server *S, std::unique_lock<std::mutex> &lk) {
  bool progressed = false;
  for (Req *r : S->active)
    if (r->key >= 0 && !r->in_pack && !r->inflight && r->n_steps - r->next_n + 1 >= fdtd::kStageSteps &&
        S->groups[r->key].members.size() < (size_t)fdtd::kMaxPack && !S->groups[r->key].inflight) {
      S->groups[r->key].members.push_back(r);
      r->in_pack = true;
      if (S->groups[r->key].pack) {  // membership changed: rebuild below
        lk.unlock();
        fdtd::pack_destroy(S->groups[r->key].pack);
        lk.lock();
        S->groups[r->key].pack = nullptr;
      }
    }
  for (auto &kv : S->groups) {
    PackGroup &G = kv.second;
    if (G.inflight) {
      const cudaError_t q = cudaEventQuery(G.ev);
      if (q == cudaErrorNotReady) continue;
      G.inflight = false;
      if (q != cudaSuccess) {
        for (Req *r : G.members) {
          r->in_pack = false;
          r->key = -1;
          r->next_n = r->n_steps + 1;
          finish(S, r, FDTD_ECUDA, cudaGetErrorString(q));
          S->active.erase(std::find(S->active.begin(), S->active.end(), r));
        }
        G.members.clear();
      }
    }
    // members with less than a ring left finish alone
    bool changed = false;
    for (size_t i = 0; i < G.members.size();) {
      Req *r = G.members[i];
      if (r->n_steps - r->next_n + 1 < fdtd::kStageSteps) {
        r->in_pack = false;
        r->key = -1;
        G.members.erase(G.members.begin() + i);
        changed = true;
      } else {
        ++i;
      }
    }
    if (changed && G.pack) {
      lk.unlock();
      fdtd::pack_destroy(G.pack);
      lk.lock();
      G.pack = nullptr;
    }
    if (G.members.empty()) continue;
    if (!G.ev && cudaEventCreateWithFlags(&G.ev, cudaEventDisableTiming) != cudaSuccess) continue;
    int rings = S->d.chunk_steps / fdtd::kStageSteps;
    for (Req *r : G.members) rings = std::min(rings, (r->n_steps - r->next_n + 1) / fdtd::kStageSteps);
    std::vector<fdtd_job *> jobs;
    for (Req *r : G.members) jobs.push_back(r->job);
    lk.unlock();
    int rc = FDTD_OK;
    char msg[256] = {};
    double tb = 0;
    if (!G.pack) {
      tb = now_s();
      rc = fdtd::pack_create(jobs.data(), (int)jobs.size(), &G.pack);
      tb = now_s() - tb;
    }
    if (!rc) rc = fdtd::pack_run(G.pack, rings, G.ev);
    if (rc) fdtd_last_error(msg, sizeof msg);
    lk.lock();
    if (tb > 0) {
      ++S->pack_builds;
      S->pack_build_s += tb;
    }
    if (rc) {  // the members go on alone
      for (Req *r : G.members) {
        r->in_pack = false;
        r->key = -1;
      }
      G.members.clear();
      continue;
    }
    for (Req *r : G.members) r->next_n += rings * fdtd::kStageSteps;
    S->packed_rings += rings;
    G.inflight = true;
    progressed = true;
  }
  return progressed;
}

void serve(fdtd_server *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    admit(S);
    if (S->stop) break;
    bool progressed = advance_packs(S, lk);
    for (size_t i = 0; i < S->active.size();) {
      Req *r = S->active[i];
      if (r->key >= 0) { ++i; continue; }  // in a pack, or waiting for its group to be idle
      if (r->inflight) {
        const cudaError_t q = cudaEventQuery(r->ev);
        if (q == cudaErrorNotReady) { ++i; continue; }
        r->inflight = false;
        if (q != cudaSuccess) {
          finish(S, r, FDTD_ECUDA, cudaGetErrorString(q));
          S->active.erase(S->active.begin() + i);
          continue;
        }
      }
      char msg[256] = {};
      int rc;
      if (r->next_n > r->n_steps) {  // all steps queued and complete: fold the last ring
        lk.unlock();
        rc = fdtd_sync(r->job);
        if (rc) fdtd_last_error(msg, sizeof msg);
        lk.lock();
        finish(S, r, rc, msg);
        S->active.erase(S->active.begin() + i);
        progressed = true;
        continue;
      }
      const int k = std::min(S->d.chunk_steps, r->n_steps - r->next_n + 1);
      lk.unlock();
      rc = fdtd_step(r->job, r->next_n, k);
      if (!rc && cudaEventRecord(r->ev, r->stream) != cudaSuccess) rc = FDTD_ECUDA;
      if (rc) fdtd_last_error(msg, sizeof msg);
      lk.lock();
      if (rc) {
        finish(S, r, rc, msg);
        S->active.erase(S->active.begin() + i);
        continue;
      }
      r->next_n += k;
      r->inflight = true;
      progressed = true;
      ++i;
    }
    if (!progressed) S->cv_work.wait_for(lk, std::chrono::microseconds(50));
  }
  // stopping: let the chunks in flight end, then leave the jobs to the destructor
  for (auto &kv : S->groups) {
    lk.unlock();
    if (kv.second.pack) fdtd::pack_destroy(kv.second.pack);  // waits for its rings
    if (kv.second.ev) cudaEventDestroy(kv.second.ev);
    lk.lock();
    kv.second.pack = nullptr;
  }
  for (Req *r : S->active)
    if (r->inflight) {
      lk.unlock();
      cudaEventSynchronize(r->ev);
      lk.lock();
      r->inflight = false;
    }
}

Req *find(fdtd_server *S, int64_t ticket) {
  auto it = S->reqs.find(ticket);
  return it == S->reqs.end() ? nullptr : it->second;
}

void drop(Req *r) {
  if (r->job) fdtd_destroy(r->job);
  if (r->ev) cudaEventDestroy(r->ev);
  if (r->stream) cudaStreamDestroy(r->stream);
  delete r;
}

}  // namespace

extern "C" {

int fdtd_server_create(const fdtd_server_desc *desc, fdtd_server **out) {
  if (!desc || !out) return fdtd::report_error(FDTD_EINVAL, "null argument");
  *out = nullptr;
  int count = 0;
  if (fdtd_device_count(&count) != FDTD_OK || count < 1)
    return fdtd::report_error(FDTD_ENODEV, "no sm_103a device for the server");
  if (desc->max_active < 1 || desc->chunk_steps < 1)
    return fdtd::report_error(FDTD_EINVAL, "max_active and chunk_steps must be >= 1");
  fdtd_server *S = new fdtd_server;
  S->d = *desc;
  // chunks of whole 32-step rings replay the ring graph with no eager steps
  S->d.chunk_steps = (desc->chunk_steps + 31) / 32 * 32;
  cudaGetDevice(&S->device);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  S->budget = desc->hbm_budget ? desc->hbm_budget : (uint64_t)(0.9 * (double)free_b);
  S->t0 = now_s();
  S->th = std::thread(serve, S);
  for (int w = 0; w < 2; ++w) S->workers.emplace_back(commit_worker, S);
  *out = S;
  return FDTD_OK;
}

int fdtd_server_submit(fdtd_server *S, fdtd_job *job, int32_t n_steps, int64_t *ticket) {
  if (!S || !job || !ticket) return fdtd::report_error(FDTD_EINVAL, "null argument");
  if (n_steps < 1) return fdtd::report_error(FDTD_EINVAL, "n_steps must be >= 1");
  uint64_t est = 0;
  int rc = fdtd_estimate_bytes(job, &est);
  if (rc) return rc;
  Req *r = new Req;
  r->job = job;
  r->n_steps = n_steps;
  r->est = est;
  r->t_submit = now_s();
  if (cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&r->ev, cudaEventDisableTiming) != cudaSuccess) {
    r->job = nullptr;  // the caller keeps the job on failure
    drop(r);
    return fdtd::report_error(FDTD_ECUDA, "stream or event creation failed");
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    r->ticket = S->next_ticket++;
    S->reqs[r->ticket] = r;
    S->queue.push_back(r);
  }
  S->cv_work.notify_one();
  *ticket = r->ticket;
  return FDTD_OK;
}

int fdtd_server_wait(fdtd_server *S, int64_t ticket, int32_t timeout_ms, int32_t *state) {
  if (!S || !state) return fdtd::report_error(FDTD_EINVAL, "null argument");
  std::unique_lock<std::mutex> lk(S->mu);
  Req *r = find(S, ticket);
  if (!r) return fdtd::report_error(FDTD_EINVAL, "unknown ticket %lld", (long long)ticket);
  auto ended = [&] { return r->state == FDTD_REQ_DONE || r->state == FDTD_REQ_FAILED; };
  if (timeout_ms < 0) S->cv_done.wait(lk, ended);
  else S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ended);
  *state = r->state;
  if (r->state == FDTD_REQ_FAILED) return fdtd::report_error(r->rc ? r->rc : FDTD_ECUDA, "job failed: %s", r->err);
  return FDTD_OK;
}

int fdtd_server_job(fdtd_server *S, int64_t ticket, fdtd_job **job) {
  if (!S || !job) return fdtd::report_error(FDTD_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  Req *r = find(S, ticket);
  if (!r) return fdtd::report_error(FDTD_EINVAL, "unknown ticket %lld", (long long)ticket);
  if (r->state != FDTD_REQ_DONE) return fdtd::report_error(FDTD_ESTATE, "job %lld has not finished", (long long)ticket);
  *job = r->job;
  return FDTD_OK;
}

int fdtd_server_times(fdtd_server *S, int64_t ticket, double *t_submit, double *t_admit, double *t_done) {
  if (!S) return fdtd::report_error(FDTD_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  Req *r = find(S, ticket);
  if (!r) return fdtd::report_error(FDTD_EINVAL, "unknown ticket %lld", (long long)ticket);
  if (t_submit) *t_submit = r->t_submit - S->t0;
  if (t_admit) *t_admit = r->t_admit > 0 ? r->t_admit - S->t0 : -1.0;
  if (t_done) *t_done = r->t_done > 0 ? r->t_done - S->t0 : -1.0;
  return FDTD_OK;
}

int fdtd_server_release(fdtd_server *S, int64_t ticket) {
  if (!S) return fdtd::report_error(FDTD_EINVAL, "null argument");
  Req *r = nullptr;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    r = find(S, ticket);
    if (!r) return fdtd::report_error(FDTD_EINVAL, "unknown ticket %lld", (long long)ticket);
    if (r->state != FDTD_REQ_DONE && r->state != FDTD_REQ_FAILED)
      return fdtd::report_error(FDTD_ESTATE, "job %lld is still queued or running", (long long)ticket);
    S->reqs.erase(ticket);
    S->held -= std::min(S->held, r->bytes);
  }
  drop(r);  // frees queue behind the job's own work; no device-wide sync
  S->cv_work.notify_one();
  return FDTD_OK;
}

int fdtd_server_stats(fdtd_server *S, fdtd_server_status *st) {
  if (!S || !st) return fdtd::report_error(FDTD_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  memset(st, 0, sizeof *st);
  st->queued = (int32_t)S->queue.size();
  st->active = (int32_t)S->active.size();
  st->finished = S->done_count;
  st->held_bytes = S->held;
  st->held_bytes_max = S->held_max;
  st->budget_bytes = S->budget;
  st->packed_rings = S->packed_rings;
  st->pack_builds = S->pack_builds;
  st->pack_build_s = S->pack_build_s;
  return FDTD_OK;
}

int fdtd_server_destroy(fdtd_server *S) {
  if (!S) return FDTD_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  S->cv_commit.notify_all();
  for (auto &w : S->workers)
    if (w.joinable()) w.join();
  if (S->th.joinable()) S->th.join();
  for (auto &kv : S->reqs) drop(kv.second);
  delete S;
  return FDTD_OK;
}

}  // extern "C"

// Serving loop over one batch (umcp_server_* in include/umcp_gpu.h). Host
// code on the public ABI only: worker threads build plans, one server thread
// owns every device call of the server (mesh creation, the batch, results).
//
// A job moves queued -> building -> ready -> running -> done. Admission is
// first come, first served: the head of the ready queue waits until its
// footprint fits the budget, so a large job is not starved by small ones.
// The server thread alternates
//   run a chunk (queued on the stream, returns at once)
//   admit ready jobs (plan upload overlaps the chunk; they join the next one)
//   poll (waits for the chunk), copy out finished jobs, free their memory
// and sizes the next chunk from the last one's time per step.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/umcp_gpu.h"

namespace {

using Clock = std::chrono::steady_clock;

struct SJob {
  uint64_t id = 0;
  std::string path, lipids;
  umcp_params prm{};
  umcp_integrator it{};
  uint64_t step0 = 0;
  int64_t n_steps = 0;
  bool keep_energies = false;
  int state = UMCP_JOB_QUEUED;
  int status = UMCP_OK;
  std::string msg;
  umcp_plan *plan = nullptr;
  size_t bytes = 0;
  int nv = 0;
  umcp_mesh *mesh = nullptr;
  int64_t steps_done = 0;
  double t_submit = -1, t_admit = -1, t_done = -1;
  double h2d = 0, d2h = 0;
  std::vector<double> r, energies;
};

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t lo = (size_t)std::floor(pos), hi = std::min(lo + 1, v.size() - 1);
  return v[lo] + (pos - (double)lo) * (v[hi] - v[lo]);
}

}  // namespace

struct umcp_server {
  umcp_ctx *ctx = nullptr;
  umcp_server_opts o{};
  umcp_batch *batch = nullptr;
  Clock::time_point t0;
  double budget = 0;

  std::mutex mu;
  std::condition_variable cv_loop, cv_build, cv_done;
  std::unordered_map<uint64_t, std::unique_ptr<SJob>> jobs;
  std::deque<SJob *> build_q, ready_q;
  std::vector<SJob *> running;  // the batch's job order
  std::vector<std::thread> builders;
  std::thread loop;
  bool stop = false;
  uint64_t next_id = 1;

  double hbm_used = 0, hbm_peak = 0;
  long long n_submitted = 0, n_completed = 0, n_failed = 0, chunks = 0;
  double vertex_steps = 0, busy = 0;
  std::vector<double> latencies;
  int chunk_steps = 32;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  // Marks j done (mu held).
  void finish_locked(SJob *j, int status, const std::string &msg) {
    j->state = UMCP_JOB_DONE;
    j->status = status;
    j->msg = msg;
    j->t_done = now();
    latencies.push_back(j->t_done - j->t_submit);
    ++n_completed;
    if (status != UMCP_OK) ++n_failed;
    cv_done.notify_all();
  }

  void builder_main();
  void server_main();
  void admit_pass();
  void harvest(const std::vector<int64_t> &done, const std::vector<int> &st);
};

void umcp_server::builder_main() {
  for (;;) {
    SJob *j;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_build.wait(lk, [&] { return stop || !build_q.empty(); });
      if (stop) return;
      j = build_q.front();
      build_q.pop_front();
      j->state = UMCP_JOB_BUILDING;
    }
    umcp_plan *plan = nullptr;
    size_t bytes = 0;
    umcp_plan_info info{};
    umcp_status st = umcp_plan_from_file(j->path.c_str(), &j->prm, &plan);
    // the footprint includes the run's energy record, which the batch keeps on the device
    if (st == UMCP_OK) st = umcp_plan_device_bytes(plan, ctx, o.precision, j->n_steps, &bytes);
    if (st == UMCP_OK) st = umcp_plan_info_get(plan, &info);
    const std::string err = st == UMCP_OK ? std::string() : std::string(umcp_last_error());
    std::lock_guard<std::mutex> lk(mu);
    if (st != UMCP_OK || (double)bytes > budget) {
      if (plan) umcp_plan_destroy(plan);
      finish_locked(j, st != UMCP_OK ? st : UMCP_ERR_NOMEM,
                    st != UMCP_OK ? err : "job footprint exceeds the server's device-memory budget");
      continue;
    }
    j->plan = plan;
    j->bytes = bytes;
    j->nv = info.nv;
    j->state = UMCP_JOB_READY;
    ready_q.push_back(j);
    cv_loop.notify_one();
  }
}

// Creates the meshes of the ready jobs that fit and adds them to the batch.
// Jobs are taken first come, first served while their footprint fits (up to
// kAdmitWave at a time); their meshes are created on parallel threads (host
// tables and uploads; the error text is per thread) and joined to the batch
// in the order taken.
void umcp_server::admit_pass() {
  constexpr size_t kAdmitWave = 16;
  for (;;) {
    std::vector<SJob *> take;
    {
      std::lock_guard<std::mutex> lk(mu);
      while (!stop && !ready_q.empty() && take.size() < kAdmitWave) {
        SJob *j = ready_q.front();
        if (hbm_used + (double)j->bytes > budget) break;
        if (o.max_jobs > 0 && (int)(running.size() + take.size()) >= o.max_jobs) break;
        ready_q.pop_front();
        hbm_used += (double)j->bytes;
        hbm_peak = std::max(hbm_peak, hbm_used);
        take.push_back(j);
      }
    }
    if (take.empty()) return;
    struct Made {
      umcp_mesh *m = nullptr;
      umcp_status st = UMCP_OK;
      std::string err;
    };
    std::vector<Made> made(take.size());
    auto create = [&](size_t i) {
      made[i].st = umcp_mesh_create(ctx, take[i]->plan, &take[i]->prm, &made[i].m);
      if (made[i].st != UMCP_OK) made[i].err = umcp_last_error();
    };
    {
      std::vector<std::thread> th;
      for (size_t i = 1; i < take.size(); ++i) th.emplace_back(create, i);
      create(0);
      for (auto &t : th) t.join();
    }
    for (size_t i = 0; i < take.size(); ++i) {
      SJob *j = take[i];
      umcp_mesh *m = made[i].m;
      umcp_status st = made[i].st;
      std::string err = made[i].err;
      umcp_mesh_info mi{};
      if (st == UMCP_OK) st = umcp_mesh_info_get(m, &mi);
      if (st == UMCP_OK) st = umcp_batch_add(batch, m, &j->it, j->step0, j->n_steps);
      if (st != UMCP_OK && err.empty()) err = umcp_last_error();
      j->h2d = (double)mi.h2d_bytes;
      umcp_plan_destroy(j->plan);
      j->plan = nullptr;
      std::lock_guard<std::mutex> lk(mu);
      if (st != UMCP_OK) {
        if (m) umcp_mesh_destroy(m);
        hbm_used -= (double)j->bytes;
        finish_locked(j, st, err);
        continue;
      }
      j->mesh = m;
      j->state = UMCP_JOB_RUNNING;
      j->t_admit = now();
      running.push_back(j);
    }
  }
}

// Counts the chunk's steps and retires finished jobs (server thread; the
// batch is idle after the poll).
void umcp_server::harvest(const std::vector<int64_t> &done, const std::vector<int> &st) {
  std::vector<SJob *> keep;
  std::vector<std::pair<SJob *, int>> fin;
  double vs = 0;
  for (size_t k = 0; k < running.size(); ++k) {
    SJob *j = running[k];
    vs += (double)j->nv * (double)(done[k] - j->steps_done);
    j->steps_done = done[k];
    if (done[k] >= j->n_steps || st[k] != UMCP_OK) fin.emplace_back(j, st[k]);
    else keep.push_back(j);
  }
  std::vector<std::string> errs(fin.size());
  for (size_t i = 0; i < fin.size(); ++i) {
    SJob *j = fin[i].first;
    j->r.assign(3 * (size_t)j->nv + 3, 0.0);
    umcp_status s = umcp_state_get(j->mesh, j->r.data(), nullptr);
    if (s == UMCP_OK && j->keep_energies) {
      j->energies.assign((size_t)j->steps_done, 0.0);
      s = umcp_mesh_energies(j->mesh, j->energies.data(), j->steps_done);
    }
    if (s != UMCP_OK) {
      errs[i] = umcp_last_error();
      fin[i].second = s;
    }
    j->d2h = (double)((j->r.size() + j->energies.size()) * sizeof(double));
    umcp_mesh_destroy(j->mesh);  // leaves the batch
    j->mesh = nullptr;
  }
  std::lock_guard<std::mutex> lk(mu);
  vertex_steps += vs;
  running.swap(keep);
  for (size_t i = 0; i < fin.size(); ++i) {
    hbm_used -= (double)fin[i].first->bytes;
    finish_locked(fin[i].first, fin[i].second, errs[i]);
  }
}

void umcp_server::server_main() {
  std::vector<int64_t> done;
  std::vector<int> st;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_loop.wait(lk, [&] { return stop || !ready_q.empty() || !running.empty(); });
      if (stop) return;
    }
    if (running.empty()) admit_pass();  // nothing on the device: admit before running
    if (running.empty()) continue;
    // Chunk: the target wall time at the last measured time per step, in
    // whole captured 32-step pieces, and no longer than the job closest to
    // its end needs (its result is then picked up without delay).
    int64_t least = INT64_MAX;
    for (SJob *j : running) least = std::min<int64_t>(least, j->n_steps - j->steps_done);
    const int64_t need = std::max<int64_t>(32, (least + 31) / 32 * 32);
    const int steps = (int)std::min<int64_t>(chunk_steps, need);
    const double t_a = now();
    umcp_status s = umcp_batch_run(batch, steps);
    admit_pass();  // overlaps the chunk; new jobs join the next one
    done.assign(running.size() + 0, 0);
    st.assign(running.size(), 0);
    if (s == UMCP_OK) {
      // poll covers every job in the batch, including those admitted just now
      std::vector<int64_t> d(running.size());
      std::vector<int> t(running.size());
      s = umcp_batch_poll(batch, d.data(), t.data());
      done.swap(d);
      st.swap(t);
    }
    const double t_b = now();
    if (s != UMCP_OK) {
      // a device error ends every running job
      const std::string err = umcp_last_error();
      std::lock_guard<std::mutex> lk(mu);
      for (SJob *j : running) {
        hbm_used -= (double)j->bytes;
        finish_locked(j, s, err);
      }
      running.clear();
      continue;
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      busy += t_b - t_a;
      ++chunks;
    }
    const double per_step = (t_b - t_a) / steps;
    const double target = (o.chunk_ms > 0 ? o.chunk_ms : 25.0) * 1e-3;
    chunk_steps = (int)std::min(8192.0, std::max(32.0, std::floor(target / std::max(per_step, 1e-7) / 32) * 32));
    harvest(done, st);
  }
}

extern "C" umcp_status umcp_server_create(umcp_ctx *ctx, const umcp_server_opts *opts, umcp_server **out) {
  if (!ctx || !out) return UMCP_ERR_INVALID;
  auto s = std::make_unique<umcp_server>();
  s->ctx = ctx;
  if (opts) s->o = *opts;
  else s->o.precision = UMCP_FP32_CENTRED;
  if (s->o.precision != UMCP_FP64 && s->o.precision != UMCP_FP32_CENTRED) return UMCP_ERR_INVALID;
  if (s->o.hbm_budget_bytes > 0) {
    s->budget = s->o.hbm_budget_bytes;
  } else {
    size_t f = 0, t = 0;
    umcp_status st = umcp_ctx_mem_info(ctx, &f, &t);
    if (st != UMCP_OK) return st;
    s->budget = 0.8 * (double)f;
  }
  umcp_batch_opts bo{s->o.tile_faces, 0, 0, nullptr};
  umcp_status st = umcp_batch_create(ctx, s->o.precision, &bo, &s->batch);
  if (st != UMCP_OK) return st;
  s->t0 = Clock::now();
  int nb = s->o.builder_threads;
  if (nb <= 0) nb = (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
  umcp_server *raw = s.get();
  for (int i = 0; i < nb; ++i) s->builders.emplace_back([raw] { raw->builder_main(); });
  s->loop = std::thread([raw] { raw->server_main(); });
  *out = s.release();
  return UMCP_OK;
}

extern "C" void umcp_server_destroy(umcp_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_loop.notify_all();
  s->cv_build.notify_all();
  s->loop.join();
  for (auto &t : s->builders) t.join();
  for (auto &kv : s->jobs) {
    SJob *j = kv.second.get();
    if (j->mesh) umcp_mesh_destroy(j->mesh);
    if (j->plan) umcp_plan_destroy(j->plan);
  }
  umcp_batch_destroy(s->batch);
  s->cv_done.notify_all();
  delete s;
}

extern "C" umcp_status umcp_server_submit(umcp_server *s, const umcp_job_desc *d, uint64_t *job_id) {
  if (!s || !d || !d->mesh_path || d->n_steps < 0 || d->it.use_mass) return UMCP_ERR_INVALID;
  auto j = std::make_unique<SJob>();
  j->path = d->mesh_path;
  j->prm = d->params;
  j->prm.precision = s->o.precision;
  if (d->params.lipid_directives) j->lipids = d->params.lipid_directives;
  j->it = d->it;
  j->step0 = d->step0;
  j->n_steps = d->n_steps;
  j->keep_energies = d->keep_energies != 0;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return UMCP_ERR_INVALID;
  j->prm.lipid_directives = j->lipids.empty() ? nullptr : j->lipids.c_str();
  j->id = s->next_id++;
  j->t_submit = s->now();
  SJob *raw = j.get();
  s->jobs.emplace(raw->id, std::move(j));
  s->build_q.push_back(raw);
  ++s->n_submitted;
  if (job_id) *job_id = raw->id;
  s->cv_build.notify_one();
  return UMCP_OK;
}

extern "C" umcp_status umcp_server_wait(umcp_server *s, uint64_t id, double timeout_s) {
  if (!s) return UMCP_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return UMCP_ERR_INVALID;
  SJob *j = it->second.get();
  auto pred = [&] { return j->state == UMCP_JOB_DONE || s->stop; };
  if (timeout_s < 0) s->cv_done.wait(lk, pred);
  else s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
  return j->state == UMCP_JOB_DONE ? UMCP_OK : UMCP_ERR_TIMEOUT;
}

extern "C" umcp_status umcp_server_wait_all(umcp_server *s, double timeout_s) {
  if (!s) return UMCP_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto pred = [&] { return s->n_completed == s->n_submitted || s->stop; };
  if (timeout_s < 0) s->cv_done.wait(lk, pred);
  else s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
  return s->n_completed == s->n_submitted ? UMCP_OK : UMCP_ERR_TIMEOUT;
}

extern "C" umcp_status umcp_server_job(umcp_server *s, uint64_t id, umcp_job_info *info) {
  if (!s || !info) return UMCP_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return UMCP_ERR_INVALID;
  const SJob *j = it->second.get();
  memset(info, 0, sizeof(*info));
  info->state = j->state;
  info->status = j->status;
  info->nv = j->nv;
  info->steps_done = j->steps_done;
  info->t_submit = j->t_submit;
  info->t_admit = j->t_admit;
  info->t_done = j->t_done;
  info->device_bytes = (double)j->bytes;
  info->h2d_bytes = j->h2d;
  info->d2h_bytes = j->d2h;
  snprintf(info->message, sizeof(info->message), "%s", j->msg.c_str());
  return UMCP_OK;
}

extern "C" umcp_status umcp_server_fetch(umcp_server *s, uint64_t id, double *r, double *energies) {
  if (!s) return UMCP_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end() || it->second->state != UMCP_JOB_DONE) return UMCP_ERR_INVALID;
  const SJob *j = it->second.get();
  if (r && !j->r.empty()) memcpy(r, j->r.data(), j->r.size() * sizeof(double));
  if (energies && !j->energies.empty()) memcpy(energies, j->energies.data(), j->energies.size() * sizeof(double));
  return UMCP_OK;
}

extern "C" umcp_status umcp_server_release(umcp_server *s, uint64_t id) {
  if (!s) return UMCP_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end() || it->second->state != UMCP_JOB_DONE) return UMCP_ERR_INVALID;
  s->jobs.erase(it);
  return UMCP_OK;
}

extern "C" umcp_status umcp_server_stats_get(umcp_server *s, umcp_server_stats *o) {
  if (!s || !o) return UMCP_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  memset(o, 0, sizeof(*o));
  o->submitted = s->n_submitted;
  o->completed = s->n_completed;
  o->failed = s->n_failed;
  o->queued = (long long)(s->build_q.size() + s->ready_q.size());
  o->running = (long long)s->running.size();
  o->chunks = s->chunks;
  o->p50_latency_s = percentile(s->latencies, 0.50);
  o->p99_latency_s = percentile(s->latencies, 0.99);
  double sum = 0, mx = 0;
  for (double l : s->latencies) { sum += l; mx = std::max(mx, l); }
  o->mean_latency_s = s->latencies.empty() ? 0 : sum / (double)s->latencies.size();
  o->max_latency_s = mx;
  o->vertex_steps = s->vertex_steps;
  o->busy_s = s->busy;
  o->vertex_steps_per_s = s->busy > 0 ? s->vertex_steps / s->busy : 0;
  o->hbm_budget_bytes = s->budget;
  o->hbm_in_use_bytes = s->hbm_used;
  o->hbm_peak_bytes = s->hbm_peak;
  o->chunk_steps = s->chunk_steps;
  return UMCP_OK;
}

extern "C" double umcp_server_now(const umcp_server *s) { return s ? s->now() : 0.0; }

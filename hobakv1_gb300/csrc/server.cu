// Continuous-batching server for scene-timestep jobs, native (host C++ over
// the batch ABI): jobs are admitted FIFO while their estimated device
// footprint fits a memory budget; the jobs admitted together form one batch
// (a cohort) that steps on its own CUDA stream.  pump() relaunches each
// cohort as soon as its own step has completed (hobak_batch_query), so
// cohorts never wait for one another; tick() is the lock-step variant.
// Finished jobs are parked (hobak_batch_set_active) and read back.  A cohort
// whose finished jobs hold at least merge_fraction of it, or any cohort with
// a finished job while arrivals wait, is re-packed: a new batch of its
// running jobs plus the queued arrivals that fit the budget is built (on a
// builder thread with async_build) while the old one keeps stepping, and at
// the old cohort's next step boundary the running jobs' state (x, v and
// NEWMARK's acceleration) is copied over and the old batch freed.  A job
// carries no other state between steps and every scene keeps its own
// reduction tiles, so each result is bitwise the same as the job run alone.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <future>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "hobak_gpu.h"

namespace hobak {
int record_error(int code, const std::string& msg);  // sets hobak_last_error() (api.cu)
}

namespace {

int fail(int code, const std::string& msg) { return hobak::record_error(code, msg); }

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Cohort;

struct Job {
  int id = 0;
  std::vector<double> rest, x0, v0;
  std::vector<int> tets, pinned;
  hobak_scene_desc desc{};
  int nsteps = 0;
  bool contact = false;
  double eps = 0, mu = 0, beta = 0;
  long long footprint = 0;
  int state = HOBAK_JOB_QUEUED;
  double submitted = -1, admitted = -1, finished = -1;
  int done = 0;
  std::vector<double> stepMs;
  std::vector<double> rx, rv;
  Cohort* cohort = nullptr;
  int slot = -1;
};

// A cohort being built, or built: the batch, or the build's error.
struct Built;

struct Cohort {
  std::vector<Job*> jobs;
  hobak_batch batch = nullptr;
  long long bytes = 0;
  int running = 0;
  bool inFlight = false;
  double tLaunch = 0;
  std::shared_future<std::shared_ptr<Built>> repl;  // its re-pack being built
  long long replReserved = 0;
  bool hasRepl = false;
};

struct Built {
  std::unique_ptr<Cohort> cohort;
  std::vector<Job*> jobs;  // the jobs it was built for
  int rc = HOBAK_OK;
  std::string error;
};

// Device bytes of one scene in a batch, an upper estimate: the common
// buffers plus those of the precision, at most 16 blocks per vertex row,
// sliced in 32-vertex slices, plus 1 MB.
long long footprint_bytes(const hobak_scene_desc& s, int precision) {
  const long long nv = s.nv, nt = s.nt, nb = 16 * nv;
  const long long w = precision == HOBAK_PRECISION_MIXED ? 4 : 8;
  const long long perTet = 16 + 72 + 8 + 4 + 96 + 64 + 16 + 8 + 92 * w;  // element Hessians: 92 values per tet
  const long long perBlock = 4 + 4 + 4 + 4 + 9 * w;
  const long long perVertex = 5 * 24 + 8 + 1 + 4 + 4 + 4 + 3 * 24 + 9 * w + (w == 4 ? 6 : 4) * 3 * w;
  return nt * perTet + nb * perBlock + nv * perVertex + (1LL << 20);
}

// One builder thread running build tasks in submission order, on the
// device that was current where the server was created.
class Builder {
 public:
  Builder() {
    if (cudaGetDevice(&device_) != cudaSuccess) device_ = 0;
    worker_ = std::thread([this] { run(); });
  }
  ~Builder() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    cv_.notify_all();
    worker_.join();
  }
  std::shared_future<std::shared_ptr<Built>> submit(std::function<std::shared_ptr<Built>()> f) {
    auto task = std::make_shared<std::packaged_task<std::shared_ptr<Built>()>>(std::move(f));
    std::shared_future<std::shared_ptr<Built>> fut = task->get_future().share();
    {
      std::lock_guard<std::mutex> lk(m_);
      q_.push_back([task] { (*task)(); });
    }
    cv_.notify_all();
    return fut;
  }

 private:
  void run() {
    cudaSetDevice(device_);
    for (;;) {
      std::function<void()> f;
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [this] { return stop_ || !q_.empty(); });
        if (q_.empty()) return;
        f = std::move(q_.front());
        q_.pop_front();
      }
      f();
    }
  }
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<std::function<void()>> q_;
  bool stop_ = false;
  int device_ = 0;
  std::thread worker_;
};

bool ready(const std::shared_future<std::shared_ptr<Built>>& f) {
  return f.wait_for(std::chrono::seconds(0)) == std::future_status::ready;
}

}  // namespace

struct hobak_server_t {
  hobak_server_opts opts{};
  hobak_solver_opts solver{};
  std::vector<std::unique_ptr<Job>> jobs;  // by id
  std::deque<Job*> queue;
  std::vector<std::unique_ptr<Cohort>> cohorts;
  std::vector<std::pair<std::shared_future<std::shared_ptr<Built>>, long long>> building;
  std::unique_ptr<Builder> builder;
  long long used = 0;
  long long ticks = 0;
  int merges = 0, mergedArrivals = 0, finished = 0;

  // A cohort of `js` (their initial state), built now on this thread.
  std::shared_ptr<Built> build_now(const std::vector<Job*>& js) const {
    auto out = std::make_shared<Built>();
    out->jobs = js;
    std::vector<hobak_scene_desc> descs;
    for (Job* j : js) descs.push_back(j->desc);
    auto c = std::make_unique<Cohort>();
    c->jobs = js;
    int rc = hobak_batch_create(descs.data(), (int)descs.size(), &solver, &c->batch);
    if (rc == HOBAK_OK && opts.use_tuning) rc = hobak_batch_set_tuning(c->batch, &opts.tuning);
    for (size_t k = 0; rc == HOBAK_OK && k < js.size(); k++)
      if (js[k]->contact) rc = hobak_batch_set_collisions(c->batch, (int)k, 1, js[k]->eps, js[k]->mu, js[k]->beta);
    if (rc == HOBAK_OK) rc = hobak_batch_device_bytes(c->batch, &c->bytes);
    if (rc != HOBAK_OK) {
      out->rc = rc;
      out->error = hobak_last_error();
      if (c->batch) hobak_batch_destroy(c->batch);
      c->batch = nullptr;
      return out;
    }
    c->running = (int)js.size();
    out->cohort = std::move(c);
    return out;
  }

  std::shared_future<std::shared_ptr<Built>> build(const std::vector<Job*>& js) {
    if (!builder) {
      std::promise<std::shared_ptr<Built>> p;
      p.set_value(build_now(js));
      return p.get_future().share();
    }
    return builder->submit([this, js] { return build_now(js); });
  }

  static void attach(Cohort* c) {
    for (size_t k = 0; k < c->jobs.size(); k++) {
      c->jobs[k]->cohort = c;
      c->jobs[k]->slot = (int)k;
    }
  }

  void join(std::unique_ptr<Cohort> c, long long reserved) {
    const double t = now_s();
    for (Job* j : c->jobs) j->admitted = t;
    attach(c.get());
    used += c->bytes - reserved;
    cohorts.push_back(std::move(c));
  }

  static void destroy(std::unique_ptr<Cohort>& c) {
    if (c && c->batch) hobak_batch_destroy(c->batch);
    c.reset();
  }

  // A build that failed: its jobs will not run (HOBAK_JOB_FAILED) and the
  // bytes reserved for it are returned; the error is reported once.
  int drop_failed(const std::shared_ptr<Built>& b, long long reserved, bool arrivalsOnly, const Cohort* from) {
    for (Job* j : b->jobs)
      if (!arrivalsOnly || j->cohort != from) j->state = HOBAK_JOB_FAILED;
    used -= reserved;
    return fail(b->rc, "server: building a cohort: " + b->error);
  }

  int collect_built(bool block) {
    std::vector<std::pair<std::shared_future<std::shared_ptr<Built>>, long long>> keep;
    int err = HOBAK_OK;
    for (auto& b : building) {
      if (block || ready(b.first)) {
        std::shared_ptr<Built> r = b.first.get();
        if (r->rc != HOBAK_OK) {
          if (!err) err = drop_failed(r, b.second, false, nullptr);
          continue;
        }
        join(std::move(r->cohort), b.second);
      } else {
        keep.push_back(b);
      }
    }
    building = std::move(keep);
    return err;
  }

  void plan_merges() {
    if (!opts.merge) return;
    for (auto& cp : cohorts) {
      Cohort* c = cp.get();
      if (c->hasRepl || c->running == 0) continue;
      const int parked = (int)c->jobs.size() - c->running;
      if (parked == 0) continue;
      std::vector<Job*> keep;
      long long estKeep = 0;
      for (Job* j : c->jobs)
        if (j->state != HOBAK_JOB_FINISHED) {
          keep.push_back(j);
          estKeep += j->footprint;
        }
      std::vector<Job*> takeJobs;
      long long est = 0;
      while (!queue.empty() && (int)(keep.size() + takeJobs.size()) < opts.max_cohort) {
        const long long need = queue.front()->footprint;
        if (used + estKeep + est + need > opts.budget_bytes) break;
        est += need;
        takeJobs.push_back(queue.front());
        queue.pop_front();
      }
      if (parked < opts.merge_fraction * (double)c->jobs.size() && takeJobs.empty()) continue;
      if (used + estKeep + est > opts.budget_bytes) {  // no room for both batches at once yet
        for (auto it = takeJobs.rbegin(); it != takeJobs.rend(); ++it) queue.push_front(*it);
        continue;
      }
      for (Job* j : takeJobs) j->state = HOBAK_JOB_RUNNING;
      used += estKeep + est;
      std::vector<Job*> all = keep;
      all.insert(all.end(), takeJobs.begin(), takeJobs.end());
      c->repl = build(all);
      c->replReserved = estKeep + est;
      c->hasRepl = true;
    }
  }

  // The carried jobs' state (x, v and NEWMARK's acceleration) copied from c
  // into its re-pack nb; the jobs that finished meanwhile parked there.
  int carry_over(Cohort* c, Cohort* nb) {
    const bool newmark = solver.integrator == HOBAK_INTEGRATOR_NEWMARK;
    std::vector<double> x, v, a;
    for (size_t k = 0; k < nb->jobs.size(); k++) {
      Job* j = nb->jobs[k];
      if (j->cohort != c) continue;  // a merged arrival starts from its initial state
      const size_t n = 3 * (size_t)j->desc.nv;
      x.resize(n);
      v.resize(n);
      if (int rc = hobak_batch_get_state(c->batch, j->slot, x.data(), v.data())) return rc;
      if (int rc = hobak_batch_set_state(nb->batch, (int)k, x.data(), v.data())) return rc;
      if (newmark) {
        a.resize(n);
        if (int rc = hobak_batch_get_acceleration(c->batch, j->slot, a.data())) return rc;
        if (int rc = hobak_batch_set_acceleration(nb->batch, (int)k, a.data())) return rc;
      }
      if (j->state == HOBAK_JOB_FINISHED) {  // finished while the re-pack was built
        if (int rc = hobak_batch_set_active(nb->batch, (int)k, 0)) return rc;
        nb->running -= 1;
      }
    }
    return HOBAK_OK;
  }

  // At c's step boundary: its re-pack, if built, with the carried jobs'
  // state copied in; c is freed.  Returns the new cohort, or null while the
  // build is still running, or on error (*rc set): then the carried jobs go
  // on in c, the merged arrivals fail and the re-pack is freed.
  Cohort* swap_ready(Cohort* c, int* rc) {
    *rc = HOBAK_OK;
    if (!c->hasRepl || c->inFlight || !ready(c->repl)) return nullptr;
    std::shared_ptr<Built> r = c->repl.get();
    c->hasRepl = false;
    if (r->rc != HOBAK_OK) {
      *rc = drop_failed(r, c->replReserved, true, c);
      return nullptr;
    }
    std::unique_ptr<Cohort> nb = std::move(r->cohort);
    if ((*rc = carry_over(c, nb.get()))) {
      for (Job* j : nb->jobs)
        if (j->cohort != c) j->state = HOBAK_JOB_FAILED;
      destroy(nb);
      used -= c->replReserved;
      return nullptr;
    }
    const double t = now_s();
    for (Job* j : nb->jobs)
      if (j->cohort != c) {  // a merged arrival
        j->admitted = t;
        mergedArrivals += 1;
      }
    attach(nb.get());
    used += nb->bytes - c->replReserved - c->bytes;
    Cohort* out = nb.get();
    for (auto& cp : cohorts)
      if (cp.get() == c) {
        destroy(cp);
        cp = std::move(nb);
        break;
      }
    merges += 1;
    return out;
  }

  int admit() {
    if (builder)
      if (int rc = collect_built(cohorts.empty())) return rc;  // nothing running: wait for the build
    // arrivals join running cohorts that have finished jobs first (a
    // re-pack), the rest form a new cohort
    plan_merges();
    std::vector<Job*> takeJobs;
    long long est = 0;
    while (!queue.empty() && (int)takeJobs.size() < opts.max_admit) {
      const long long need = queue.front()->footprint;
      if (used + est + need > opts.budget_bytes) break;
      est += need;
      takeJobs.push_back(queue.front());
      queue.pop_front();
    }
    if (takeJobs.empty()) return HOBAK_OK;
    for (Job* j : takeJobs) j->state = HOBAK_JOB_RUNNING;
    used += est;  // reserved until the cohort reports its real size
    building.emplace_back(build(takeJobs), est);
    if (!builder || cohorts.empty()) return collect_built(true);
    return HOBAK_OK;
  }

  int step_done(Cohort* c, double ms, double t, int* done) {
    for (Job* j : c->jobs) {
      if (j->state == HOBAK_JOB_FINISHED) continue;
      j->done += 1;
      j->stepMs.push_back(ms);
      *done += 1;
      if (j->done >= j->nsteps) {
        j->finished = t;
        j->state = HOBAK_JOB_FINISHED;
        if (opts.keep_results) {
          const size_t n = 3 * (size_t)j->desc.nv;
          j->rx.resize(n);
          j->rv.resize(n);
          if (int rc = hobak_batch_get_state(c->batch, j->slot, j->rx.data(), j->rv.data())) return rc;
        }
        if (int rc = hobak_batch_set_active(c->batch, j->slot, 0)) return rc;
        c->running -= 1;
        finished += 1;
      }
    }
    return HOBAK_OK;
  }

  // c has no running jobs left but its re-pack is being built: wait for it
  // and swap it in when it holds arrivals, else drop it.
  int finish_replacement(Cohort* c, Cohort** next) {
    *next = nullptr;
    c->repl.wait();
    std::shared_ptr<Built> b = c->repl.get();
    if (b->rc != HOBAK_OK) {
      c->hasRepl = false;
      return drop_failed(b, c->replReserved, true, c);
    }
    bool arrivals = false;
    for (Job* j : b->cohort->jobs) arrivals = arrivals || j->cohort != c;
    if (arrivals) {
      int rc;
      *next = swap_ready(c, &rc);
      return rc;
    }
    destroy(b->cohort);
    used -= c->replReserved;
    c->hasRepl = false;
    return HOBAK_OK;
  }

  int retire() {
    for (size_t i = 0; i < cohorts.size();) {
      Cohort* c = cohorts[i].get();
      if (c->running == 0 && !c->inFlight) {
        if (c->hasRepl) {
          Cohort* nxt = nullptr;
          if (int rc = finish_replacement(c, &nxt)) return rc;
          if (nxt) {
            i++;
            continue;
          }
        }
        used -= c->bytes;
        destroy(cohorts[i]);
        cohorts.erase(cohorts.begin() + (long)i);
        continue;
      }
      i++;
    }
    return HOBAK_OK;
  }

  int tick(int* done) {
    *done = 0;
    if (int rc = admit()) return rc;
    std::vector<Cohort*> live;
    for (auto& c : cohorts)
      if (c->running > 0 && !c->inFlight) live.push_back(c.get());
    if (live.empty()) return HOBAK_OK;
    const double t0 = now_s();
    for (Cohort* c : live)
      if (int rc = hobak_batch_step_async(c->batch, 1)) return rc;
    for (Cohort* c : live) {
      const int rc = hobak_batch_wait(c->batch, nullptr);
      if (rc < 0) return rc;
    }
    const double t = now_s(), ms = (t - t0) * 1e3;
    ticks += 1;
    for (Cohort* c : live)
      if (int rc = step_done(c, ms, t, done)) return rc;
    if (int rc = retire()) return rc;
    plan_merges();
    std::vector<Cohort*> all;
    for (auto& c : cohorts) all.push_back(c.get());
    for (Cohort* c : all) {
      int rc;
      swap_ready(c, &rc);
      if (rc) return rc;
    }
    return HOBAK_OK;
  }

  int pump(int* done) {
    *done = 0;
    if (int rc = admit()) return rc;
    std::vector<Cohort*> all;
    for (auto& c : cohorts) all.push_back(c.get());
    for (Cohort* c : all) {
      if (c->inFlight) {
        const int q = hobak_batch_query(c->batch);
        if (q < 0) return q;
        if (q == 0) continue;
        const int rc = hobak_batch_wait(c->batch, nullptr);
        if (rc < 0) return rc;
        const double t = now_s();
        c->inFlight = false;
        ticks += 1;
        if (int e = step_done(c, (t - c->tLaunch) * 1e3, t, done)) return e;
      }
      if (c->running > 0 && c->hasRepl) {
        int rc;
        Cohort* nb = swap_ready(c, &rc);
        if (rc) return rc;
        if (nb) c = nb;
      }
      if (c->running > 0) {
        if (int rc = hobak_batch_step_async(c->batch, 1)) return rc;
        c->inFlight = true;
        c->tLaunch = now_s();
      }
    }
    if (int rc = retire()) return rc;
    plan_merges();
    return HOBAK_OK;
  }

  void close() {
    if (builder) {
      for (auto& b : building) {
        std::shared_ptr<Built> r = b.first.get();
        destroy(r->cohort);
      }
      for (auto& c : cohorts)
        if (c->hasRepl) destroy(c->repl.get()->cohort);
      builder.reset();  // joins the builder thread
    } else {
      for (auto& c : cohorts)
        if (c->hasRepl) destroy(c->repl.get()->cohort);
    }
    for (auto& c : cohorts) {
      if (c->inFlight) hobak_batch_wait(c->batch, nullptr);
      destroy(c);
    }
    cohorts.clear();
    building.clear();
  }
};

extern "C" {

void hobak_default_server_opts(hobak_server_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->budget_bytes = 64LL << 30;
  o->max_admit = 64;
  o->max_cohort = 64;
  o->merge = 1;
  o->merge_fraction = 0.5;
  o->async_build = 0;
  o->keep_results = 1;
  o->use_tuning = 0;
}

int hobak_server_create(const hobak_server_opts* opts, const hobak_solver_opts* solver, hobak_server* out) {
  if (!out) return fail(HOBAK_ERR_INVALID, "null output handle");
  *out = nullptr;
  auto s = std::make_unique<hobak_server_t>();
  hobak_default_server_opts(&s->opts);
  if (opts) s->opts = *opts;
  hobak_default_solver_opts(&s->solver);
  if (solver) s->solver = *solver;
  if (s->opts.budget_bytes <= 0 || s->opts.max_admit < 1 || s->opts.max_cohort < 1 ||
      !(s->opts.merge_fraction >= 0.0 && s->opts.merge_fraction <= 1.0))
    return fail(HOBAK_ERR_INVALID, "server options: budget_bytes > 0, max_admit and max_cohort >= 1, "
                                   "merge_fraction in [0, 1]");
  if (s->opts.async_build) s->builder = std::make_unique<Builder>();
  *out = s.release();
  return HOBAK_OK;
}

int hobak_server_submit(hobak_server s, const hobak_scene_desc* scene, int nsteps, const double* contact, int* job) {
  if (!s || !scene || !job) return fail(HOBAK_ERR_INVALID, "null argument");
  if (nsteps < 1) return fail(HOBAK_ERR_INVALID, "nsteps < 1");
  if (scene->nv < 1 || scene->nt < 1 || !scene->rest || !scene->tets || (scene->npinned > 0 && !scene->pinned))
    return fail(HOBAK_ERR_INVALID, "empty or incomplete scene");
  auto j = std::make_unique<Job>();
  j->id = (int)s->jobs.size();
  const size_t n = 3 * (size_t)scene->nv;
  j->rest.assign(scene->rest, scene->rest + n);
  j->tets.assign(scene->tets, scene->tets + 4 * (size_t)scene->nt);
  if (scene->npinned > 0) j->pinned.assign(scene->pinned, scene->pinned + scene->npinned);
  if (scene->x0) j->x0.assign(scene->x0, scene->x0 + n);
  if (scene->v0) j->v0.assign(scene->v0, scene->v0 + n);
  j->desc = *scene;
  j->desc.rest = j->rest.data();
  j->desc.tets = j->tets.data();
  j->desc.pinned = j->pinned.empty() ? nullptr : j->pinned.data();
  j->desc.x0 = j->x0.empty() ? nullptr : j->x0.data();
  j->desc.v0 = j->v0.empty() ? nullptr : j->v0.data();
  j->nsteps = nsteps;
  if (contact) {
    j->contact = true;
    j->eps = contact[0];
    j->mu = contact[1];
    j->beta = contact[2];
  }
  j->footprint = footprint_bytes(*scene, s->solver.precision);
  if (j->footprint > s->opts.budget_bytes)  // can never fit: refuse instead of blocking the queue
    return fail(HOBAK_ERR_INVALID, "the job needs more than the whole memory budget");
  j->submitted = now_s();
  *job = j->id;
  s->queue.push_back(j.get());
  s->jobs.push_back(std::move(j));
  return HOBAK_OK;
}

int hobak_server_pump(hobak_server s, int* job_steps) {
  if (!s) return fail(HOBAK_ERR_INVALID, "null handle");
  int done = 0;
  const int rc = s->pump(&done);
  if (job_steps) *job_steps = done;
  return rc;
}

int hobak_server_tick(hobak_server s, int* job_steps) {
  if (!s) return fail(HOBAK_ERR_INVALID, "null handle");
  int done = 0;
  const int rc = s->tick(&done);
  if (job_steps) *job_steps = done;
  return rc;
}

int hobak_server_idle(hobak_server s) {
  if (!s) return fail(HOBAK_ERR_INVALID, "null handle");
  return s->queue.empty() && s->cohorts.empty() && s->building.empty() ? 1 : 0;
}

int hobak_server_get_stats(hobak_server s, hobak_server_stats* out) {
  if (!s || !out) return fail(HOBAK_ERR_INVALID, "null argument");
  out->used_bytes = s->used;
  out->cohorts = (int)s->cohorts.size();
  out->queued = (int)s->queue.size();
  out->building = (int)s->building.size();
  out->ticks = s->ticks;
  out->merges = s->merges;
  out->merged_arrivals = s->mergedArrivals;
  out->finished = s->finished;
  out->now_s = now_s();
  return HOBAK_OK;
}

int hobak_server_job(hobak_server s, int job, hobak_job_info* info, double* step_ms, double* x, double* v) {
  if (!s || job < 0 || job >= (int)s->jobs.size()) return fail(HOBAK_ERR_INVALID, "bad handle or job id");
  const Job& j = *s->jobs[job];
  if (info) {
    info->state = j.state;
    info->done_steps = j.done;
    info->nsteps = j.nsteps;
    info->nv = j.desc.nv;
    info->submitted_s = j.submitted;
    info->admitted_s = j.admitted;
    info->finished_s = j.finished;
  }
  if (step_ms && !j.stepMs.empty()) std::memcpy(step_ms, j.stepMs.data(), sizeof(double) * j.stepMs.size());
  if (x || v) {
    if (j.state != HOBAK_JOB_FINISHED || j.rx.empty())
      return fail(HOBAK_ERR_INVALID, "the job has no result (not finished, or keep_results off)");
    if (x) std::memcpy(x, j.rx.data(), sizeof(double) * j.rx.size());
    if (v) std::memcpy(v, j.rv.data(), sizeof(double) * j.rv.size());
  }
  return HOBAK_OK;
}

int hobak_server_destroy(hobak_server s) {
  if (!s) return HOBAK_OK;
  s->close();
  delete s;
  return HOBAK_OK;
}

}  // extern "C"

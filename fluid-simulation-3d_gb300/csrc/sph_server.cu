// Native serving loop (sph_server_*): continuous batching of scene jobs over
// one batch engine, on a worker thread. Any thread submits a job (a scene of
// n particles to advance K steps), cancels it or waits for its result; the
// worker admits waiting jobs in submission order while the HBM budget has
// room (later, smaller jobs may backfill), advances every resident scene one
// step per batched launch, and retires a job after its K-th step with its
// state read back. The engine is only touched by the worker, and the job
// queue only under the server's mutex. Results equal the job run alone, bit
// for bit: a batched step runs every particle's arithmetic in the same order
// as a single-scene step.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sph_gb300.h"
#include "sph_engine.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  uint64_t id = 0;
  sph_params prm{};
  uint32_t n = 0;
  float dt = 0.0f;
  uint32_t steps_left = 0;
  std::vector<float> pos, vel, dens;  // inputs, then the results
  uint32_t scene = 0;
  bool resident = false, done = false;
  std::atomic<bool> cancel{false};  // set under mu, read by the worker outside it
  bool admitting = false;  // the worker is loading its inputs (outside mu)
  int status = SPH_OK;  // SPH_OK, or why the job ended without a result
  std::string why;
};

double Seconds(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

// Step latencies in a fixed log-spaced histogram, so a long-running server
// keeps constant memory: bin b holds [1 us * kRatio^b, 1 us * kRatio^(b+1)),
// 0.5% wide, up to about 1,000 s; a percentile reports its bin's geometric
// centre (within 0.25% of the step time it stands for).
struct LatencyHistogram {
  static constexpr int kBins = 4200;
  static constexpr double kRatio = 1.005;
  static constexpr double kLowMs = 1e-3;
  std::vector<uint64_t> weight = std::vector<uint64_t>(kBins, 0);
  uint64_t total = 0;

  void Add(double ms, uint32_t w) {
    int b = 0;
    if (ms > kLowMs) b = static_cast<int>(std::log(ms / kLowMs) / std::log(kRatio));
    weight[std::min(std::max(b, 0), kBins - 1)] += w;
    total += w;
  }
  // the smallest bin centre at or below which a fraction q of the weight lies
  double Percentile(double q) const {
    const double want = q * static_cast<double>(total);
    uint64_t acc = 0;
    int b = 0;
    for (; b < kBins - 1; ++b) {
      acc += weight[b];
      if (weight[b] && static_cast<double>(acc) >= want) break;
    }
    return kLowMs * std::pow(kRatio, b + 0.5);
  }
};

}  // namespace

struct sph_server {
  sph::Engine eng;
  int substeps;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  std::deque<std::shared_ptr<Job>> waiting;
  std::map<uint32_t, std::shared_ptr<Job>> resident;  // scene id -> job
  std::map<uint64_t, std::shared_ptr<Job>> jobs;      // not yet collected
  uint64_t next_id = 1;
  bool stop = false;
  std::thread worker;
  // statistics (under mu)
  uint64_t submitted = 0, completed = 0, cancelled = 0, failed = 0;
  uint64_t steps = 0, particle_steps = 0;
  double step_s = 0, admit_s = 0, retire_s = 0;  // worker time per activity
  uint32_t status_flags = 0;  // device status flags of every step so far
  LatencyHistogram step_ms;  // each step weighted by the jobs it advanced
  bool started = false;
  Clock::time_point t_first{}, t_last{};
  std::string err;
  // pinned staging ring for admitted jobs' inputs (nullptr: not available)
  char* stage = nullptr;
  size_t stage_cap = 0;
  static constexpr size_t kStageBytes = 256ull << 20;
  static constexpr int kDeferred = 1;  // admission result: try next round
  static size_t StageAlign(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

  sph_server(uint64_t capacity, uint32_t max_scenes, int ss)
      : eng(capacity, max_scenes), substeps(ss) {}

  void Finish(const std::shared_ptr<Job>& j, int status, const std::string& why) {
    j->done = true;
    j->status = status;
    j->why = why;
    if (status == SPH_OK) {
      ++completed;
    } else {
      if (j->cancel) ++cancelled;
      else ++failed;
      if (!j->admitting) {  // else the worker still reads the inputs
        std::vector<float>().swap(j->pos);
        std::vector<float>().swap(j->vel);
      }
    }
    done_cv.notify_all();
  }

  // One round of the worker, entered and left with mu held (lk). The engine
  // is only touched by the worker and never under mu, so submitters,
  // cancellers and waiters are not held up by device calls:
  //   1. resident jobs cancelled since the last round leave the engine;
  //   2. the resident jobs advance one batched step (launched, not waited
  //      for), and meanwhile the waiting jobs are admitted in order while
  //      the budget has room (a later, smaller job may backfill): their
  //      inputs are staged and their uploads queued behind the step, so the
  //      host work of admission overlaps the step on the device;
  //   3. after the step completes, jobs at their last step are read back
  //      and retired.
  void Round(std::unique_lock<std::mutex>& lk) {
    for (auto it = resident.begin(); it != resident.end();) {
      if (it->second->cancel) {
        eng.RemoveScene(it->first);
        Finish(it->second, SPH_ERR_STATE, "cancelled");
        it = resident.erase(it);
      } else {
        ++it;
      }
    }
    std::vector<std::pair<uint32_t, std::shared_ptr<Job>>> stepped(resident.begin(),
                                                                   resident.end());
    uint64_t live = 0;
    for (auto& kv : stepped) live += kv.second->n;
    std::vector<std::shared_ptr<Job>> trying(waiting.begin(), waiting.end());
    for (auto& j : trying) j->admitting = true;
    lk.unlock();

    const Clock::time_point t0 = Clock::now();
    int rc = SPH_OK;
    if (!stepped.empty()) rc = eng.Step(substeps, stream);
    const Clock::time_point ta = Clock::now();
    std::vector<int> arc(trying.size(), SPH_ERR_NOMEM);
    std::vector<uint32_t> sids(trying.size(), 0);
    if (rc == SPH_OK) {
      // Inputs go through the pinned staging ring: the engine's import kernel
      // reads them from there on the stream, behind the step, while this
      // thread moves on. (A pageable upload would block this thread until the
      // stream reached it, i.e. until the step ends.) The ring is free again
      // after the round's synchronisation. A job too large for the ring is
      // uploaded from its own (pageable) arrays.
      size_t off = 0;
      for (size_t k = 0; k < trying.size(); ++k) {
        const Job& j = *trying[k];
        if (j.cancel) continue;  // cancelled before its turn
        const float* pp = j.pos.data();
        const float* vp = j.vel.empty() ? nullptr : j.vel.data();
        const size_t bytes = 12ull * j.n;
        const size_t need = StageAlign(bytes) * (vp ? 2 : 1);
        const size_t off0 = off;
        if (stage && need <= stage_cap) {
          if (off + need > stage_cap) {
            arc[k] = kDeferred;  // the ring is full this round
            continue;
          }
          std::memcpy(stage + off, pp, bytes);
          pp = reinterpret_cast<const float*>(stage + off);
          off += StageAlign(bytes);
          if (vp) {
            std::memcpy(stage + off, vp, bytes);
            vp = reinterpret_cast<const float*>(stage + off);
            off += StageAlign(bytes);
          }
        }
        arc[k] = eng.AddScene(j.prm, j.n, pp, vp, false, j.dt, &sids[k], stream);
        if (arc[k] != SPH_OK) off = off0;
      }
    }
    const Clock::time_point tb = Clock::now();
    std::string eerr;
    if (rc != SPH_OK) {
      eerr = eng.LastError();
    } else if (const cudaError_t e = cudaStreamSynchronize(stream); e != cudaSuccess) {
      rc = SPH_ERR_CUDA;
      eerr = std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e);
    }
    uint32_t flags = 0;
    if (rc == SPH_OK && !stepped.empty() && eng.Status(&flags, stream) != SPH_OK) {
      rc = SPH_ERR_CUDA;
      eerr = eng.LastError();
    }
    const Clock::time_point t1 = Clock::now();

    lk.lock();
    admit_s += Seconds(ta, tb);
    status_flags |= flags;
    bool admitted_any = false;
    for (size_t k = 0; k < trying.size(); ++k) {
      const std::shared_ptr<Job>& j = trying[k];
      j->admitting = false;
      if (j->done) {  // cancelled while being admitted
        if (arc[k] == SPH_OK) eng.RemoveScene(sids[k]);
        std::vector<float>().swap(j->pos);
        std::vector<float>().swap(j->vel);
        continue;
      }
      if (j->cancel) continue;  // finished by cancel() already
      if (arc[k] == SPH_ERR_NOMEM || arc[k] == kDeferred) continue;  // stays in the queue
      waiting.erase(std::remove(waiting.begin(), waiting.end(), j), waiting.end());
      if (arc[k] != SPH_OK) {
        Finish(j, arc[k], eng.LastError());
        continue;
      }
      admitted_any = true;
      j->scene = sids[k];
      j->resident = true;
      std::vector<float>().swap(j->pos);  // on the device now; results reuse them
      std::vector<float>().swap(j->vel);
      resident[sids[k]] = j;
      if (!started) {
        started = true;
        t_first = t0;
      }
    }
    if (rc != SPH_OK) {
      // the step or the round's synchronisation failed: every resident job,
      // the ones admitted behind it included, ends with the error
      err = eerr;
      for (auto& kv : resident) {
        eng.RemoveScene(kv.first);
        Finish(kv.second, rc, err);
      }
      resident.clear();
      return;
    }
    if (stepped.empty()) {
      if (!admitted_any && resident.empty() && !waiting.empty()) {
        // Nothing runs: a waiting job that did not fit an empty engine never
        // will. Jobs submitted after this round's snapshot are tried first.
        bool all_tried = true;
        for (auto& j : waiting) {
          const auto t = std::find(trying.begin(), trying.end(), j);
          all_tried = all_tried && t != trying.end() &&
                      arc[static_cast<size_t>(t - trying.begin())] == SPH_ERR_NOMEM;
        }
        if (all_tried) {
          for (auto& j : waiting) Finish(j, SPH_ERR_NOMEM, "job does not fit the server's budget");
          waiting.clear();
        }
      }
      return;
    }
    ++steps;
    particle_steps += live;
    step_s += Seconds(t0, t1);
    step_ms.Add(1000.0 * Seconds(t0, t1), static_cast<uint32_t>(stepped.size()));
    t_last = t1;
    std::vector<std::pair<uint32_t, std::shared_ptr<Job>>> retiring;
    for (auto& kv : stepped)
      if (--kv.second->steps_left == 0) retiring.push_back(kv);
    if (retiring.empty()) return;
    lk.unlock();
    const Clock::time_point r0 = Clock::now();
    std::vector<int> drc(retiring.size());
    for (size_t k = 0; k < retiring.size(); ++k) {
      Job& j = *retiring[k].second;
      j.pos.resize(3ull * j.n);
      j.vel.resize(3ull * j.n);
      j.dens.resize(2ull * j.n);
      drc[k] = eng.Download(retiring[k].first, j.pos.data(), j.vel.data(), j.dens.data(),
                            false, stream);
    }
    const Clock::time_point r1 = Clock::now();
    lk.lock();
    retire_s += Seconds(r0, r1);
    for (size_t k = 0; k < retiring.size(); ++k) {
      eng.RemoveScene(retiring[k].first);
      resident.erase(retiring[k].first);
      Finish(retiring[k].second, drc[k], drc[k] == SPH_OK ? "" : eng.LastError());
    }
  }

  void Run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      work_cv.wait(lk, [&] { return stop || !waiting.empty() || !resident.empty(); });
      if (stop) {
        for (auto& j : waiting) Finish(j, SPH_ERR_STATE, "server stopped");
        for (auto& kv : resident) Finish(kv.second, SPH_ERR_STATE, "server stopped");
        waiting.clear();
        resident.clear();
        break;
      }
      Round(lk);
    }
  }
};

extern "C" {

int sph_server_create(uint64_t budget_bytes, uint32_t max_scenes, int substeps,
                      sph_server** out) {
  if (!out || substeps < 1 || substeps > 64 || max_scenes == 0) return SPH_ERR_INVALID;
  *out = nullptr;
  const uint64_t cap = budget_bytes / sph::Engine::BytesPerParticle();
  if (cap == 0) return SPH_ERR_INVALID;
  std::unique_ptr<sph_server> s(new (std::nothrow) sph_server(cap, max_scenes, substeps));
  if (!s) return SPH_ERR_NOMEM;
  int rc = s->eng.Init();
  if (rc != SPH_OK) return rc;
  if (cudaGetDevice(&s->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  if (cudaHostAlloc(reinterpret_cast<void**>(&s->stage), sph_server::kStageBytes,
                    cudaHostAllocDefault) == cudaSuccess) {
    s->stage_cap = sph_server::kStageBytes;
  } else {
    cudaGetLastError();  // uploads then go from the jobs' own arrays
    s->stage = nullptr;
  }
  sph_server* raw = s.get();
  raw->worker = std::thread([raw] { raw->Run(); });
  *out = s.release();
  return SPH_OK;
}

int sph_server_destroy(sph_server* s) {
  if (!s) return SPH_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->work_cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->stream) cudaStreamDestroy(s->stream);
  if (s->stage) cudaFreeHost(s->stage);
  delete s;
  return SPH_OK;
}

int sph_server_submit(sph_server* s, const sph_params* params, uint32_t n, const float* pos3,
                      const float* vel3, float dt, uint32_t steps, uint64_t* job_id) {
  if (!s || !params || !pos3 || !job_id || n == 0 || n >= (1u << 24) || steps == 0)
    return SPH_ERR_INVALID;
  if (n > s->eng.Capacity()) return SPH_ERR_NOMEM;  // could never be admitted
  auto j = std::make_shared<Job>();
  j->prm = *params;
  j->n = n;
  j->dt = dt;
  j->steps_left = steps;
  j->pos.assign(pos3, pos3 + 3ull * n);
  if (vel3) j->vel.assign(vel3, vel3 + 3ull * n);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    j->id = s->next_id++;
    s->jobs[j->id] = j;
    s->waiting.push_back(j);
    ++s->submitted;
  }
  s->work_cv.notify_all();
  *job_id = j->id;
  return SPH_OK;
}

int sph_server_cancel(sph_server* s, uint64_t job_id) {
  if (!s) return SPH_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job_id);
  if (it == s->jobs.end()) return SPH_ERR_INVALID;
  const std::shared_ptr<Job>& j = it->second;
  if (j->done) return SPH_OK;
  j->cancel = true;
  if (!j->resident) {
    s->waiting.erase(std::remove(s->waiting.begin(), s->waiting.end(), j), s->waiting.end());
    s->Finish(j, SPH_ERR_STATE, "cancelled");
  }
  // a resident job leaves the batch at the worker's next step boundary
  return SPH_OK;
}

int sph_server_wait(sph_server* s, uint64_t job_id, float* pos3, float* vel3, float* dens2,
                    double timeout_s) {
  if (!s) return SPH_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job_id);
  if (it == s->jobs.end()) return SPH_ERR_INVALID;
  std::shared_ptr<Job> j = it->second;
  const auto limit = std::chrono::duration<double>(timeout_s < 0.0 ? 0.0 : timeout_s);
  if (!s->done_cv.wait_for(lk, limit, [&] { return j->done; })) {
    s->err = "job not finished within the timeout";
    return SPH_ERR_STATE;
  }
  s->jobs.erase(job_id);
  if (j->status != SPH_OK) {
    s->err = j->why;
    return j->status;
  }
  if (pos3) std::copy(j->pos.begin(), j->pos.end(), pos3);
  if (vel3) std::copy(j->vel.begin(), j->vel.end(), vel3);
  if (dens2) std::copy(j->dens.begin(), j->dens.end(), dens2);
  return SPH_OK;
}

int sph_server_get_stats(sph_server* s, sph_server_stats* out) {
  if (!s || !out) return SPH_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = sph_server_stats{};
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->cancelled = s->cancelled;
  out->failed = s->failed;
  out->queued = static_cast<uint32_t>(s->waiting.size());
  out->resident = static_cast<uint32_t>(s->resident.size());
  out->steps = s->steps;
  out->particle_steps = s->particle_steps;
  out->capacity_particles = s->eng.Capacity();
  if (s->started && s->steps) {
    out->wall_s = Seconds(s->t_first, s->t_last);
    out->particle_steps_per_s = out->wall_s > 0 ? s->particle_steps / out->wall_s : 0.0;
    // per-step latency as the jobs see it: every step weighted by the jobs
    // it advanced
    out->p50_step_ms = s->step_ms.Percentile(0.50);
    out->p99_step_ms = s->step_ms.Percentile(0.99);
  }
  out->step_s = s->step_s;
  out->admit_s = s->admit_s;
  out->retire_s = s->retire_s;
  out->status_flags = s->status_flags;
  return SPH_OK;
}

const char* sph_server_last_error(sph_server* s) {
  if (!s) return "null server";
  std::lock_guard<std::mutex> lk(s->mu);
  thread_local std::string copy;
  copy = s->err;
  return copy.c_str();
}

}  // extern "C"

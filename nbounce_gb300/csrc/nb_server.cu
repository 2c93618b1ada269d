// Render-job server: continuous batching of path-tracing jobs on one GPU.
//
// A scheduler thread owns a CUDA stream and one set of path buffers.  Each turn it
//   1. admits queued jobs in arrival order while their images fit the HBM budget (images are
//      allocated stream-ordered with cudaMallocAsync and zeroed, as the reference's fresh
//      texture is);
//   2. plans a wave: every admitted job with samples left gets one segment of consecutive
//      Sobol rows, sized by an equal share of the wave's path capacity (at least one sample);
//   3. launches the wave (raygen, trace + shade per bounce up to the largest bounce count of
//      the wave, accumulate) and records an event;
//   4. with two waves in flight, waits for the older one and completes the jobs whose last
//      samples it carried (copy-out to the caller's buffer if one was given, free, notify).
// Jobs that arrive while waves run join the next wave.  Every path depends only on its own
// job, pixel and sample, and a job's samples reach its image in sample order, so a job's
// image does not depend on what it was batched with.
//
// Per-job options (nb_job_desc.flags): NB_JOB_ENV_NEE jobs share the ordinary waves, which
// then run the next-event-estimation shade kernel gated per job (the other jobs' paths are
// unchanged).  NB_JOB_CACHE jobs run in waves of their own with the radiance cache of their
// scene (one per scene slot, created on first use, trained by every cache wave on it); a cache
// wave packs the pending cache jobs of one scene like an ordinary wave packs the others.  When
// both kinds are pending the scheduler alternates between a cache wave and an ordinary one.
// The caches' buffers are outside the HBM budget's accounting.
//
// Failure handling, all on the host side of the GPU work: a bounded queue sheds load beyond
// saturation (submit returns NB_ERR_BUSY), a job can be cancelled or given a deadline (it
// finishes with NB_ERR_CANCELLED / NB_ERR_EXPIRED; waves of it already on the GPU run to
// completion and its image is freed after them, stream-ordered), and a failed image
// allocation fails only its job (NB_ERR_OOM).  A job record stays alive while a wave on the
// GPU still refers to it, even if the caller releases it.

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "nb_mlp.cuh"
#include "nb_runtime.h"

namespace nb {
namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  uint64_t id = 0;
  nb_job_desc desc{};
  enum State { kQueued, kActive, kDone } state = kQueued;
  int status = NB_OK;
  uint32_t next_sample = 1;  // next Sobol row to plan
  uint32_t planned_waves = 0, finished_waves = 0;
  bool fully_planned = false;
  bool released = false;     // the caller released it; erased once no wave refers to it
  uint32_t inflight_refs = 0;  // waves on the GPU with a segment of this job
  float* d_img = nullptr;
  size_t bytes = 0;
  double t_submit = 0, t_admit = 0, t_finish = 0;
};

struct InFlight {
  cudaEvent_t start = nullptr, stop = nullptr;
  std::vector<Job*> jobs;  // jobs with a segment in this wave
};

}  // namespace
}  // namespace nb

using namespace nb;

struct nb_server {
  uint64_t budget = 0;
  uint32_t capacity = 0;
  int sms = 1;
  cudaStream_t stream = nullptr, copy_stream = nullptr;
  DeviceArena buffers;
  PathBatch pb{};
  uint32_t* d_counts = nullptr;
  unsigned long long* d_rays = nullptr;
  uint64_t fixed_bytes = 0;  // path buffers + tables
  ShadowQueue sq{};          // shadow rays of NB_JOB_ENV_NEE jobs
  std::map<uint32_t, nb_cache*> caches;  // scene slot -> radiance cache of NB_JOB_CACHE jobs
  nb_cache_config cache_cfg{};
  bool has_cache_cfg = false;            // else nb_cache_default_config
  bool last_wave_cache = false;

  std::vector<const nb_scene*> scenes;
  std::vector<const nb_env*> envs;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  std::vector<Job*> active;
  std::map<uint64_t, std::unique_ptr<Job>> jobs;
  uint64_t next_id = 1;
  bool stopping = false;
  std::thread scheduler;

  std::unique_ptr<WaveTables> wt{new WaveTables()};
  std::deque<InFlight> inflight;
  std::vector<cudaEvent_t> event_pool;
  Clock::time_point t0 = Clock::now();

  uint32_t queue_limit = 0;       // 0: unbounded
  uint32_t fail_alloc_in = 0;     // the fail_alloc_in-th image allocation from now fails (0: off)
  bool has_deadlines = false;

  // statistics (guarded by mu)
  uint64_t jobs_submitted = 0, jobs_done = 0, jobs_failed = 0, waves = 0;
  uint64_t jobs_rejected = 0, jobs_cancelled = 0, jobs_expired = 0;
  double gpu_busy_ms = 0.0;
  uint64_t bytes_in_use = 0, peak_bytes = 0;

  double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }

  cudaEvent_t take_event() {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }

  // fails every job that is not finished (after a CUDA error the context is unusable)
  void fail_all(int status) {
    for (auto& kv : jobs) {
      Job* j = kv.second.get();
      if (j->state != Job::kDone) {
        j->state = Job::kDone;
        j->status = status;
        j->t_finish = now_ms();
        ++jobs_failed;
      }
    }
    queue.clear();
    active.clear();
    cv_done.notify_all();
  }

  // Fails the unfinished queued or active jobs that `pick` accepts.  Waves of theirs still in
  // flight run to completion; the images are freed after them (stream order).
  template <class Pick>
  void fail_jobs_locked(Pick pick, int status) {
    auto doomed = [&](Job* j) { return j->state != Job::kDone && pick(j); };
    uint32_t n_failed = 0;
    auto count = [&] {
      ++n_failed;
      ++jobs_failed;
      if (status == NB_ERR_CANCELLED) ++jobs_cancelled;
      if (status == NB_ERR_EXPIRED) ++jobs_expired;
    };
    for (Job* j : queue)
      if (doomed(j)) j->state = Job::kDone, j->status = status, j->t_finish = now_ms(), count();
    queue.erase(std::remove_if(queue.begin(), queue.end(), [](Job* j) { return j->state == Job::kDone; }),
                queue.end());
    for (Job* j : active) {
      if (!doomed(j)) continue;
      if (j->d_img) {
        cudaFreeAsync(j->d_img, stream);
        j->d_img = nullptr;
        bytes_in_use -= j->bytes;
      }
      j->state = Job::kDone;
      j->status = status;
      j->t_finish = now_ms();
      count();
    }
    if (n_failed == 0) return;  // nothing changed: no erase, no wake-up (the deadline check runs every turn)
    active.erase(std::remove_if(active.begin(), active.end(), [](Job* j) { return j->state == Job::kDone; }),
                 active.end());
    cv_done.notify_all();
  }

  // fails the queued and active jobs whose deadline has passed
  void expire_locked() {
    if (!has_deadlines) return;
    const double now = now_ms();
    fail_jobs_locked([now](const Job* j) { return j->desc.deadline_ms && now > j->t_submit + j->desc.deadline_ms; },
                     NB_ERR_EXPIRED);
  }

  // drops a wave's reference to a job; a released job is erased with its last reference
  void unref_locked(Job* j) {
    if (j->inflight_refs) --j->inflight_refs;
    if (j->released && j->inflight_refs == 0) jobs.erase(j->id);
  }

  void admit_locked() {
    while (!queue.empty() && active.size() < kMaxWaveJobs) {
      Job* j = queue.front();
      if (bytes_in_use + j->bytes > budget) break;  // wait for images to be delivered
      queue.pop_front();
      void* p = nullptr;
      cudaError_t e;
      if (fail_alloc_in && --fail_alloc_in == 0) e = cudaErrorMemoryAllocation;  // nb_server_fail_alloc
      else e = cudaMallocAsync(&p, j->bytes, stream);
      if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, j->bytes, stream);
      if (e != cudaSuccess) {
        j->state = Job::kDone;
        j->status = cuda_fail(e, "job image");
        j->t_finish = now_ms();
        ++jobs_failed;
        cv_done.notify_all();
        continue;
      }
      j->d_img = (float*)p;
      j->state = Job::kActive;
      j->t_admit = now_ms();
      bytes_in_use += j->bytes;
      peak_bytes = std::max(peak_bytes, bytes_in_use);
      active.push_back(j);
    }
  }

  // plans one wave into *wt; returns false if no active job has samples left to plan
  // packs the unplanned active jobs that `pick` accepts into the next wave
  template <class Pick>
  bool plan_locked(std::vector<Job*>* wave_jobs, uint32_t* max_bounces, bool* single_scene, bool* any_nee,
                   Pick pick) {
    WaveTables& t = *wt;
    std::vector<Job*> cand;
    for (Job* j : active)
      if (!j->fully_planned && pick(j)) cand.push_back(j);
    if (cand.empty()) return false;
    const uint64_t share = std::max<uint64_t>(1, capacity / cand.size());
    uint64_t left = capacity;
    t.n_segs = t.n_jobs = t.n_scenes = 0;
    std::map<uint32_t, uint32_t> scene_slot;
    std::vector<uint32_t> want(cand.size(), 0);
    uint32_t n_segs = 0;
    // first pass: equal shares of the capacity; second pass: what is left, in arrival order
    for (int pass = 0; pass < 2; ++pass) {
      for (size_t i = 0; i < cand.size(); ++i) {
        Job* j = cand[i];
        const uint64_t npix = (uint64_t)j->desc.width * j->desc.height;
        const uint32_t remaining = j->desc.spp - (j->next_sample - 1) - want[i];
        if (remaining == 0 || npix > left) continue;
        if (want[i] == 0) {  // a new segment needs a segment slot and, maybe, a scene slot
          if (n_segs >= kMaxWaveSegments) continue;
          if (!scene_slot.count(j->desc.scene) && scene_slot.size() >= kMaxWaveScenes) continue;
        }
        const uint64_t paths = pass == 0 ? std::min<uint64_t>(left, std::max<uint64_t>(share, npix)) : left;
        const uint32_t s = (uint32_t)std::min<uint64_t>(remaining, paths / npix);
        if (s == 0) continue;
        if (want[i] == 0) ++n_segs;
        want[i] += s;
        left -= s * npix;
        scene_slot.emplace(j->desc.scene, (uint32_t)scene_slot.size());
      }
    }
    uint32_t path = 0, pix = 0;
    *max_bounces = 0;
    *any_nee = false;
    for (size_t i = 0; i < cand.size(); ++i) {
      if (want[i] == 0) continue;
      Job* j = cand[i];
      const uint32_t npix = j->desc.width * j->desc.height;
      const uint32_t jslot = t.n_jobs++;
      JobParams& jp = t.jobs[jslot];
      std::memcpy(jp.c2w, j->desc.camera.clip_to_world, sizeof(jp.c2w));
      jp.env = envs[j->desc.env]->dev;
      jp.out = (float4*)j->d_img;
      jp.scene = scene_slot.at(j->desc.scene);
      jp.width = j->desc.width;
      jp.height = j->desc.height;
      jp.npix = npix;
      jp.bounces = j->desc.bounces;
      jp.cf = j->desc.contribution_factor;
      jp.rr_start = 0;
      jp.flags = (j->desc.flags & NB_JOB_ENV_NEE) ? kJobEnvNee : 0u;
      *any_nee = *any_nee || jp.flags != 0u;
      t.segs[t.n_segs++] = Segment{jslot, j->next_sample, want[i], path, pix};
      path += want[i] * npix;
      pix += npix;
      j->next_sample += want[i];
      j->fully_planned = j->next_sample > j->desc.spp;
      j->planned_waves += 1;
      j->inflight_refs += 1;
      *max_bounces = std::max(*max_bounces, j->desc.bounces);
      wave_jobs->push_back(j);
    }
    for (auto& kv : scene_slot) t.scenes[kv.second] = scenes[kv.first]->dev;
    t.n_scenes = (uint32_t)scene_slot.size();
    t.n_paths = path;
    t.n_pix = pix;
    *single_scene = t.n_scenes == 1;
    return t.n_segs > 0;
  }

  // a cache wave: the cache jobs on the scene of the oldest cache job with samples left
  bool plan_cache_locked(std::vector<Job*>* wave_jobs, uint32_t* max_bounces, uint32_t* scene) {
    const Job* first = nullptr;
    for (const Job* a : active)
      if (!a->fully_planned && (a->desc.flags & NB_JOB_CACHE)) {
        first = a;
        break;
      }
    if (!first) return false;
    const uint32_t sc = first->desc.scene;
    bool single = true, nee = false;
    *scene = sc;
    return plan_locked(wave_jobs, max_bounces, &single, &nee,
                       [sc](const Job* j) { return (j->desc.flags & NB_JOB_CACHE) && j->desc.scene == sc; });
  }

  bool cache_job_pending_locked() const {
    for (Job* a : active)
      if (!a->fully_planned && (a->desc.flags & NB_JOB_CACHE)) return true;
    return false;
  }
  bool plain_job_pending_locked() const {
    for (Job* a : active)
      if (!a->fully_planned && !(a->desc.flags & NB_JOB_CACHE)) return true;
    return false;
  }

  cudaError_t launch_wave(uint32_t max_bounces, bool single_scene, bool nee) {
    PathBatch p = pb;
    cudaError_t e = cudaSuccess;
    wt->flags = nee ? kWaveZeroRadiance : 0u;  // NEE shading adds to radiance
    if (nee) e = cudaMemsetAsync(sq.counts, 0, 2 * kMaxBounceSlots * sizeof(uint32_t), stream);
    if (e == cudaSuccess) e = launch_raygen(p, *wt, sms, stream);
    for (uint32_t b = 0; b <= max_bounces && e == cudaSuccess; ++b) {
      e = launch_trace_wave(p, *wt, single_scene, b, d_rays, sms, stream);
      if (e == cudaSuccess) e = nee ? launch_shade_nee(p, *wt, sq, b, sms, stream) : launch_shade(p, *wt, b, sms, stream);
      if (e == cudaSuccess && nee) e = launch_trace_shadow(p, *wt, sq, b, sms, stream);
    }
    if (e == cudaSuccess) e = launch_accumulate(p, *wt, sms, stream);
    return e;
  }

  // the scene's cache (created on first use) and this wave's cache buffers; a failure here
  // has launched nothing
  int prepare_cache_wave(uint32_t scene_slot, nb_cache** out, CacheWave* cw) {
    nb_cache*& c = caches[scene_slot];
    int rc = NB_OK;
    if (!c && (rc = nb_cache_create(has_cache_cfg ? &cache_cfg : nullptr, &c))) {
      c = nullptr;
      return rc;
    }
    *out = c;
    return cache_wave_begin(c, scenes[scene_slot], wt->n_paths, cw, stream);
  }

  // a cache wave: the plain prefix kernels with cache-mode shading, lookups and training
  int launch_cache_wave(nb_cache* c, const CacheWave& cw, uint32_t max_bounces) {
    int rc = NB_OK;
    PathBatch p = pb;
    wt->flags = kWaveZeroRadiance;  // cache lookups add to radiance
    cudaError_t e = launch_raygen(p, *wt, sms, stream);
    for (uint32_t b = 0; b <= max_bounces && e == cudaSuccess; ++b) {
      e = launch_trace_wave(p, *wt, true, b, d_rays, sms, stream);
      if (e == cudaSuccess) e = launch_shade_cache(p, *wt, cw, b, sms, stream);
    }
    if (e != cudaSuccess) return cuda_fail(e, "cache wave launch");
    if ((rc = cache_wave_infer(c, p, sms, stream)) || (rc = cache_wave_train(c, wt->n_paths, sms, stream)))
      return rc;
    e = launch_accumulate(p, *wt, sms, stream);
    return e == cudaSuccess ? NB_OK : cuda_fail(e, "cache wave launch");
  }

  void complete_locked(Job* j) {
    if (j->desc.host_out) {
      cudaMemcpyAsync(j->desc.host_out, j->d_img, j->bytes, cudaMemcpyDeviceToHost, copy_stream);
      cudaStreamSynchronize(copy_stream);
      cudaFreeAsync(j->d_img, stream);
      j->d_img = nullptr;
      bytes_in_use -= j->bytes;
    }
    j->state = Job::kDone;
    j->t_finish = now_ms();
    ++jobs_done;
    active.erase(std::remove(active.begin(), active.end(), j), active.end());
    cv_done.notify_all();
  }

  void run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      expire_locked();
      admit_locked();
      bool launched = false;
      if (inflight.size() < 2) {
        std::vector<Job*> wave_jobs;
        uint32_t max_bounces = 0, cache_scene = 0;
        bool single = true, nee = false;
        const bool want_cache =
            cache_job_pending_locked() && (!plain_job_pending_locked() || !last_wave_cache);
        const bool planned = want_cache ? plan_cache_locked(&wave_jobs, &max_bounces, &cache_scene)
                                        : plan_locked(&wave_jobs, &max_bounces, &single, &nee,
                                                      [](const Job* j) { return !(j->desc.flags & NB_JOB_CACHE); });
        if (planned) {
          InFlight w;
          w.start = take_event();
          w.stop = take_event();
          w.jobs = std::move(wave_jobs);
          cudaEventRecord(w.start, stream);
          int rc = NB_OK;
          if (want_cache) {
            nb_cache* c = nullptr;
            CacheWave cw{};
            const int setup = prepare_cache_wave(cache_scene, &c, &cw);
            if (setup != NB_OK) {  // the scene's cache jobs fail; the other jobs go on
              for (Job* j : w.jobs) unref_locked(j);
              fail_jobs_locked([&](const Job* j) { return (j->desc.flags & NB_JOB_CACHE) && j->desc.scene == cache_scene; },
                               setup);
              event_pool.push_back(w.start);
              event_pool.push_back(w.stop);
              last_wave_cache = true;
              continue;
            }
            rc = launch_cache_wave(c, cw, max_bounces);
          } else {
            cudaError_t e = launch_wave(max_bounces, single, nee);
            if (e != cudaSuccess) rc = cuda_fail(e, "wave launch");
          }
          last_wave_cache = want_cache;
          cudaEventRecord(w.stop, stream);
          if (rc != NB_OK) {
            fail_all(rc);
            return;
          }
          ++waves;
          inflight.push_back(std::move(w));
          launched = true;
        }
      }
      if (launched) continue;
      if (!inflight.empty()) {
        InFlight w = std::move(inflight.front());
        inflight.pop_front();
        lk.unlock();
        cudaError_t e = cudaEventSynchronize(w.stop);
        float ms = 0.0f;
        if (e == cudaSuccess) cudaEventElapsedTime(&ms, w.start, w.stop);
        lk.lock();
        if (e != cudaSuccess) {
          cuda_fail(e, "wave");
          fail_all(NB_ERR_CUDA);
          return;
        }
        gpu_busy_ms += ms;
        for (Job* j : w.jobs) {
          if (j->state != Job::kDone) {  // else it failed while this wave ran
            j->finished_waves += 1;
            if (j->fully_planned && j->finished_waves == j->planned_waves) complete_locked(j);
          }
          unref_locked(j);
        }
        event_pool.push_back(w.start);
        event_pool.push_back(w.stop);
        continue;
      }
      if (stopping && queue.empty() && active.empty()) return;
      cv_work.wait_for(lk, std::chrono::milliseconds(2));
    }
  }

  int device = 0;
};

extern "C" {

int nb_server_create(uint64_t hbm_budget_bytes, uint32_t paths_per_wave, nb_server** out) {
  if (!out) return fail(NB_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (paths_per_wave == 0 || paths_per_wave > 0x7FFFFFFFu) return fail(NB_ERR_INVALID_ARG, "invalid paths_per_wave");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(NB_ERR_NO_DEVICE, "no CUDA device");
  std::unique_ptr<nb_server> s(new (std::nothrow) nb_server());
  if (!s) return fail(NB_ERR_OOM, "host allocation failed");
  s->budget = hbm_budget_bytes;
  s->capacity = paths_per_wave;
  s->sms = sm_count();
  cudaGetDevice(&s->device);
  NB_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  NB_CUDA(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
  // path buffers: 8 float4 queues/hits/radiance + instance ids, per path; 3 float4 of
  // shadow rays per path for NB_JOB_ENV_NEE jobs
  const size_t n_paths = paths_per_wave;
  const size_t path_bytes = n_paths * (11 * sizeof(float4) + sizeof(uint32_t)) + 2 * kMaxBounceSlots * sizeof(uint32_t);
  std::vector<float> table((size_t)kMaxSampleCount * kLdsStride * 4);
  sobol_burley_table(kMaxSampleCount, kLdsStride, 0, table.data());
  const size_t table_bytes = table.size() * sizeof(float);
  const size_t counter_bytes = 2 * kMaxBounceSlots * sizeof(uint32_t) + 16 + sizeof(unsigned long long);
  s->fixed_bytes = path_bytes + table_bytes + counter_bytes;
  if (s->fixed_bytes > hbm_budget_bytes)
    return fail(NB_ERR_OOM, "budget %llu B is below the path buffers (%zu B)", (unsigned long long)hbm_budget_bytes,
                s->fixed_bytes);
  void* p = nullptr;
  float4* f4[8];
  for (int k = 0; k < 8; ++k) {
    int st = s->buffers.alloc(n_paths * sizeof(float4), &p);
    if (st) { s->buffers.release(); return st; }
    f4[k] = (float4*)p;
  }
  int st = s->buffers.alloc(n_paths * sizeof(uint32_t), &p);
  if (st) { s->buffers.release(); return st; }
  float4* shadow[3];
  for (int k = 0; k < 3; ++k) {
    if ((st = s->buffers.alloc(n_paths * sizeof(float4), (void**)&shadow[k]))) { s->buffers.release(); return st; }
  }
  uint32_t* shadow_counts = nullptr;
  if ((st = s->buffers.alloc(2 * kMaxBounceSlots * sizeof(uint32_t), (void**)&shadow_counts))) {
    s->buffers.release();
    return st;
  }
  s->sq = ShadowQueue{shadow[0], shadow[1], shadow[2], shadow_counts, shadow_counts + kMaxBounceSlots};
  PathBatch& b = s->pb;
  b.q_o[0] = f4[0]; b.q_o[1] = f4[1];
  b.q_d[0] = f4[2]; b.q_d[1] = f4[3];
  b.q_t[0] = f4[4]; b.q_t[1] = f4[5];
  b.hits = f4[6];
  b.radiance = f4[7];
  b.hit_inst = (uint32_t*)p;
  if ((st = s->buffers.alloc(table_bytes, &p))) { s->buffers.release(); return st; }
  b.sobol = (const float4*)p;
  b.sobol_entries = kMaxSampleCount * kLdsStride;
  NB_CUDA(cudaMemcpy(p, table.data(), table_bytes, cudaMemcpyHostToDevice), "cudaMemcpy(sobol)");
  if ((st = s->buffers.alloc(counter_bytes, &p))) { s->buffers.release(); return st; }
  NB_CUDA(cudaMemset(p, 0, counter_bytes), "cudaMemset");
  b.counts = (uint32_t*)p;
  b.fetch = b.counts + kMaxBounceSlots;
  b.status = b.fetch + kMaxBounceSlots;
  s->d_rays = (unsigned long long*)((char*)p + 2 * kMaxBounceSlots * sizeof(uint32_t) + 16);
  s->bytes_in_use = s->fixed_bytes;
  s->peak_bytes = s->bytes_in_use;
  nb_server* raw = s.release();
  raw->scheduler = std::thread([raw] { raw->run(); });
  *out = raw;
  return NB_OK;
}

int nb_server_add_scene(nb_server* s, const nb_scene* scene, uint32_t* slot) {
  if (!s || !scene || !slot) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (!scene->uploaded) return fail(NB_ERR_INVALID_ARG, "scene was built with NB_SCENE_HOST_ONLY");
  std::lock_guard<std::mutex> lk(s->mu);
  *slot = (uint32_t)s->scenes.size();
  s->scenes.push_back(scene);
  return NB_OK;
}

int nb_server_add_env(nb_server* s, const nb_env* env, uint32_t* slot) {
  if (!s || !env || !slot) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  *slot = (uint32_t)s->envs.size();
  s->envs.push_back(env);
  return NB_OK;
}

int nb_server_set_cache_config(nb_server* s, const struct nb_cache_config* cfg) {
  if (!s) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  s->has_cache_cfg = cfg != nullptr;
  if (cfg) s->cache_cfg = *cfg;
  return NB_OK;
}

int nb_server_submit(nb_server* s, const nb_job_desc* desc, uint64_t* job_id) {
  if (!s || !desc || !job_id) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  const uint64_t npix = (uint64_t)desc->width * desc->height;
  if (npix == 0 || desc->spp == 0) return fail(NB_ERR_INVALID_ARG, "empty job");
  if (desc->spp > kMaxSampleCount) return fail(NB_ERR_INVALID_ARG, "spp above the Sobol table (%u rows)", kMaxSampleCount);
  if (desc->bounces + 2 > kMaxBounceSlots) return fail(NB_ERR_INVALID_ARG, "bounces must be <= %u", kMaxBounceSlots - 2);
  if (npix > s->capacity) return fail(NB_ERR_INVALID_ARG, "image larger than the paths of one wave");
  if (desc->flags & ~(uint32_t)(NB_JOB_ENV_NEE | NB_JOB_CACHE)) return fail(NB_ERR_INVALID_ARG, "unknown job flags 0x%x", desc->flags);
  if ((desc->flags & NB_JOB_ENV_NEE) && (desc->flags & NB_JOB_CACHE))
    return fail(NB_ERR_INVALID_ARG, "NB_JOB_ENV_NEE and NB_JOB_CACHE are exclusive");
  std::lock_guard<std::mutex> lk(s->mu);
  if (desc->scene >= s->scenes.size() || desc->env >= s->envs.size())
    return fail(NB_ERR_INVALID_ARG, "unknown scene or environment slot");
  if (s->stopping) return fail(NB_ERR_INVALID_ARG, "server is shutting down");
  if (s->queue_limit && s->queue.size() >= s->queue_limit) {
    ++s->jobs_rejected;
    return fail(NB_ERR_BUSY, "queue full (%u jobs waiting for admission)", s->queue_limit);
  }
  std::unique_ptr<Job> j(new (std::nothrow) Job());
  if (!j) return fail(NB_ERR_OOM, "host allocation failed");
  j->desc = *desc;
  j->bytes = npix * 4 * sizeof(float);
  if (s->fixed_bytes + j->bytes > s->budget) return fail(NB_ERR_OOM, "job image does not fit the budget");
  j->id = s->next_id++;
  j->t_submit = s->now_ms();
  if (desc->deadline_ms) s->has_deadlines = true;
  s->queue.push_back(j.get());
  *job_id = j->id;
  s->jobs.emplace(j->id, std::move(j));
  ++s->jobs_submitted;
  s->cv_work.notify_one();
  return NB_OK;
}

int nb_server_wait(nb_server* s, uint64_t job_id, int timeout_ms, nb_job_info* info) {
  if (!s) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job_id);
  if (it == s->jobs.end() || it->second->released)
    return fail(NB_ERR_INVALID_ARG, "unknown job %llu", (unsigned long long)job_id);
  Job* j = it->second.get();
  auto done = [&] { return j->state == Job::kDone; };
  if (timeout_ms < 0) s->cv_done.wait(lk, done);
  else s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done);
  if (info) {
    info->status = j->status;
    info->done = j->state == Job::kDone ? 1u : 0u;
    info->submit_ms = j->t_submit;
    info->admit_ms = j->t_admit;
    info->finish_ms = j->t_finish;
  }
  if (j->state != Job::kDone) return fail(NB_ERR_TIMEOUT, "job %llu not finished", (unsigned long long)job_id);
  return j->status == NB_OK ? NB_OK : fail(j->status, "job %llu failed", (unsigned long long)job_id);
}

int nb_server_fetch(nb_server* s, uint64_t job_id, float* host_rgba) {
  if (!s || !host_rgba) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job_id);
  if (it == s->jobs.end() || it->second->released) return fail(NB_ERR_INVALID_ARG, "unknown job");
  Job* j = it->second.get();
  if (j->state != Job::kDone) return fail(NB_ERR_TIMEOUT, "job not finished");
  if (j->status != NB_OK) return fail(j->status, "job failed");
  if (!j->d_img) return fail(NB_ERR_INVALID_ARG, "image already delivered");
  NB_CUDA(cudaMemcpyAsync(host_rgba, j->d_img, j->bytes, cudaMemcpyDeviceToHost, s->copy_stream), "cudaMemcpyAsync");
  NB_CUDA(cudaStreamSynchronize(s->copy_stream), "cudaStreamSynchronize");
  cudaFreeAsync(j->d_img, s->stream);
  j->d_img = nullptr;
  s->bytes_in_use -= j->bytes;
  s->cv_work.notify_one();
  return NB_OK;
}

int nb_server_release(nb_server* s, uint64_t job_id) {
  if (!s) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job_id);
  if (it == s->jobs.end() || it->second->released) return fail(NB_ERR_INVALID_ARG, "unknown job");
  Job* j = it->second.get();
  if (j->state != Job::kDone) return fail(NB_ERR_INVALID_ARG, "job not finished");
  if (j->d_img) {
    cudaFreeAsync(j->d_img, s->stream);
    j->d_img = nullptr;
    s->bytes_in_use -= j->bytes;
    s->cv_work.notify_one();
  }
  if (j->inflight_refs) j->released = true;  // a wave on the GPU still refers to it
  else s->jobs.erase(it);
  return NB_OK;
}

int nb_server_set_queue_limit(nb_server* s, uint32_t max_queued) {
  if (!s) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  s->queue_limit = max_queued;
  return NB_OK;
}

int nb_server_cancel(nb_server* s, uint64_t job_id) {
  if (!s) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job_id);
  if (it == s->jobs.end() || it->second->released)
    return fail(NB_ERR_INVALID_ARG, "unknown job %llu", (unsigned long long)job_id);
  Job* j = it->second.get();
  if (j->state == Job::kDone) return fail(NB_ERR_INVALID_ARG, "job %llu already finished", (unsigned long long)job_id);
  s->fail_jobs_locked([j](const Job* x) { return x == j; }, NB_ERR_CANCELLED);
  s->cv_work.notify_one();
  return NB_OK;
}

int nb_server_fail_alloc(nb_server* s, uint32_t nth) {
  if (!s) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  s->fail_alloc_in = nth;
  return NB_OK;
}

int nb_server_get_stats(nb_server* s, nb_server_stats* out) {
  if (!s || !out) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  unsigned long long rays = 0;
  NB_CUDA(cudaMemcpyAsync(&rays, s->d_rays, sizeof(rays), cudaMemcpyDeviceToHost, s->copy_stream), "cudaMemcpyAsync");
  NB_CUDA(cudaStreamSynchronize(s->copy_stream), "cudaStreamSynchronize");
  std::lock_guard<std::mutex> lk(s->mu);
  out->jobs_submitted = s->jobs_submitted;
  out->jobs_done = s->jobs_done;
  out->jobs_failed = s->jobs_failed;
  out->waves = s->waves;
  out->rays = rays;
  out->gpu_busy_ms = s->gpu_busy_ms;
  out->bytes_in_use = s->bytes_in_use;
  out->peak_bytes_in_use = s->peak_bytes;
  out->budget_bytes = s->budget;
  out->queued = (uint32_t)s->queue.size();
  out->active = (uint32_t)s->active.size();
  out->jobs_rejected = s->jobs_rejected;
  out->jobs_cancelled = s->jobs_cancelled;
  out->jobs_expired = s->jobs_expired;
  out->queue_limit = s->queue_limit;
  out->reserved = 0;
  return NB_OK;
}

void nb_server_destroy(nb_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
    s->cv_work.notify_all();
  }
  if (s->scheduler.joinable()) s->scheduler.join();
  cudaStreamSynchronize(s->stream);
  for (auto& kv : s->jobs)
    if (kv.second->d_img) cudaFree(kv.second->d_img);
  for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
  for (auto& kv : s->caches) nb_cache_destroy(kv.second);
  s->buffers.release();
  cudaStreamDestroy(s->stream);
  cudaStreamDestroy(s->copy_stream);
  delete s;
}

}  // extern "C"

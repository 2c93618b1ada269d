// Kernel parameter blocks and launcher declarations (nb_kernels.cu <-> nb_api.cu, nb_server.cu).
//
// A wave is one wavefront of paths: raygen, then trace + shade per bounce, then accumulate.
// Its paths come from segments; a segment is a run of consecutive samples of one job (one
// render request: scene, camera, environment, image).  The single-image Pathtracer runs
// waves of one segment; the server packs segments of many jobs into one wave.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "nb_device.cuh"

namespace nb {

constexpr uint32_t kMaxBounceSlots = 64;  // per-bounce queue counters (bounces <= 62)
constexpr uint32_t kMaxWaveJobs = 32;     // jobs per wave
constexpr uint32_t kMaxWaveSegments = 64; // segments per wave
constexpr uint32_t kMaxWaveScenes = 16;   // distinct scenes per wave

struct JobParams {
  float c2w[16];        // clip_to_world, column-major
  nbd::DevEnv env;
  float4* out;          // RGBA32F image, width * height
  uint32_t scene;       // index into WaveTables::scenes
  uint32_t width, height, npix;
  uint32_t bounces;
  float cf;             // contribution_factor
  uint32_t rr_start;    // Russian roulette from this bounce on (0: the reference schedule)
  uint32_t flags;       // kJobEnvNee: environment next-event estimation (k_shade_nee)
};
constexpr uint32_t kJobEnvNee = 1u << 0;

struct Segment {
  uint32_t job;           // index into WaveTables::jobs
  uint32_t first_sample;  // 1-based Sobol row of the segment's first sample
  uint32_t n_samples;
  uint32_t path_begin;    // first path id of the segment in the wave
  uint32_t pix_begin;     // first accumulate thread of the segment
};

// Passed by value to the wave kernels (well under the 32 KB parameter limit).
// flags: kWaveZeroRadiance - raygen zeroes every path's radiance, for waves whose shading adds
// to it (environment NEE, radiance cache); with the reference estimator every path's radiance
// is written once, where the path ends (k_shade), and raygen leaves it alone.
constexpr uint32_t kWaveZeroRadiance = 1u << 0;
// 64-bit counters per bounce slot of the instrumented traversal (nb_pathtracer_trace_counters):
// 0-4 node / triangle / instance / push counts, 5 rays, 6-10 warp-step statistics
constexpr uint32_t kTraceCounterSlots = 16;
struct WaveTables {
  uint32_t n_segs, n_jobs, n_scenes, n_paths, n_pix;
  uint32_t flags;
  uint32_t pad[2];
  Segment segs[kMaxWaveSegments];
  JobParams jobs[kMaxWaveJobs];
  nbd::DevScene scenes[kMaxWaveScenes];
};

// Device work buffers of a wave.  Path p is sample p / npix, pixel p % npix of its segment.
struct PathBatch {
  float4* q_o[2];       // ray origin, .w = path id (bits); double-buffered queues
  float4* q_d[2];       // ray direction, .w = scene index (bits)
  float4* q_t[2];       // throughput
  float4* hits;         // t, u, v, triangle (bits)
  uint32_t* hit_inst;   // TLAS-permuted instance of the hit
  float4* radiance;     // L per path id
  uint32_t* counts;     // rays entering bounce b (kMaxBounceSlots)
  uint32_t* fetch;      // work-fetch cursor per bounce (kMaxBounceSlots)
  uint32_t* status;     // device status word
  const float4* sobol;  // Sobol-Burley table, kLdsStride vec4 per sample row
  uint32_t sobol_entries;
};

// refill: lanes take new rays as theirs finish (for arrays whose neighbouring rays are unrelated)
cudaError_t launch_trace_rays(const nbd::DevScene& s, const float* rays, uint32_t n, bool any, bool refill,
                              float* hits, uint32_t* inst, uint32_t* fetch, uint32_t* status, int sms,
                              cudaStream_t st);

cudaError_t launch_raygen(const PathBatch& pb, const WaveTables& wt, int sms, cudaStream_t st);
// single_scene: all paths use wt.scenes[0] (passed by value); otherwise each ray's scene index.
// counters (optional): runs the instrumented traversal, which adds its work counters (TLAS
// node tests, BLAS node tests, triangle tests, instance entries, stack pushes) to
// counters[8 * bounce + 0..4].
cudaError_t launch_trace_wave(const PathBatch& pb, const WaveTables& wt, bool single_scene, uint32_t bounce,
                              unsigned long long* ray_total, int sms, cudaStream_t st,
                              unsigned long long* counters = nullptr);
cudaError_t launch_shade(const PathBatch& pb, const WaveTables& wt, uint32_t bounce, int sms, cudaStream_t st);
// Shadow rays of environment next-event estimation: one per path and bounce at most.
struct ShadowQueue {
  float4* o;          // origin, .w = path id (bits)
  float4* d;          // direction (unit)
  float4* c;          // radiance the path gains when the direction is unoccluded
  uint32_t* counts;   // rays appended per bounce (kMaxBounceSlots)
  uint32_t* fetch;    // work-fetch cursor per bounce (kMaxBounceSlots)
};

// environment next-event estimation (NB_SAMPLE_ENV_NEE): shade, then the bounce's shadow rays
cudaError_t launch_shade_nee(const PathBatch& pb, const WaveTables& wt, const ShadowQueue& sq, uint32_t bounce,
                             int sms, cudaStream_t st);
cudaError_t launch_trace_shadow(const PathBatch& pb, const WaveTables& wt, const ShadowQueue& sq, uint32_t bounce,
                                int sms, cudaStream_t st);
// directions and densities of env importance samples for uniform pairs u (device arrays)
cudaError_t launch_env_sample(const nbd::DevEnv& env, const float* u, uint32_t n, float4* out, int sms,
                              cudaStream_t st);

struct CacheWave;
// radiance-cache mode shade (nb_mlp.cuh describes the wave state)
cudaError_t launch_shade_cache(const PathBatch& pb, const WaveTables& wt, const CacheWave& cw, uint32_t bounce,
                               int sms, cudaStream_t st);
cudaError_t launch_accumulate(const PathBatch& pb, const WaveTables& wt, int sms, cudaStream_t st);

}  // namespace nb

// Kernel parameter blocks and launcher declarations (nb_kernels.cu <-> nb_api.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "nb_device.cuh"

namespace nb {

constexpr uint32_t kMaxBounceSlots = 64;  // per-bounce queue counters (bounces <= 62)

struct CameraParams {
  float c2w[16];  // clip_to_world, column-major
};

// Device work buffers of one batch of paths (n_paths = npix * samples of the batch).
// Paths are numbered p = k * npix + pixel for the batch's k-th sample.
struct PathBatch {
  float4* q_o[2];       // ray origin, .w = path id (bits); double-buffered queues
  float4* q_d[2];       // ray direction
  float4* q_t[2];       // throughput
  float4* hits;         // t, u, v, triangle (bits)
  uint32_t* hit_inst;   // TLAS-permuted instance of the hit
  float4* radiance;     // L per path id
  uint32_t* counts;     // rays entering bounce b (kMaxBounceSlots)
  uint32_t* fetch;      // work-fetch cursor per bounce (kMaxBounceSlots)
  uint32_t* status;     // device status word
  const float4* sobol;  // Sobol-Burley table, kLdsStride vec4 per sample row
  uint32_t sobol_entries;
  uint32_t n_paths;
  uint32_t npix, width, height;
  uint32_t first_sample;  // 1-based Sobol row of the batch's first sample
};

cudaError_t launch_trace_rays(const nbd::DevScene& s, const float* rays, uint32_t n, bool any, float* hits,
                              uint32_t* inst, uint32_t* fetch, uint32_t* status, int sms, cudaStream_t st);

// one batch = raygen, then trace + shade per bounce 0..bounces, then accumulate
cudaError_t launch_raygen(const PathBatch& pb, const CameraParams& cam, int sms, cudaStream_t st);
cudaError_t launch_trace_wave(const nbd::DevScene& s, const PathBatch& pb, uint32_t bounce,
                              unsigned long long* ray_total, int sms, cudaStream_t st);
cudaError_t launch_shade(const nbd::DevScene& s, const nbd::DevEnv& env, const PathBatch& pb, uint32_t bounce,
                         uint32_t bounces, float cf, int sms, cudaStream_t st);
cudaError_t launch_accumulate(const PathBatch& pb, uint32_t n_samples, float* out, int sms, cudaStream_t st);

}  // namespace nb

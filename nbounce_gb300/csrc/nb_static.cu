// nb_render_static: a render entry point that allocates nothing.
//
// Some callers cannot allocate device memory when they render: an engine that hands every
// byte of the GPU to its own allocator up front and forbids allocations afterwards, or a
// real-time loop whose memory footprint must not change once frames run.  For them this
// entry point renders into the caller's image with all wavefront scratch (path queues, hits,
// radiance, bounce counters, the Sobol table) in one file-scope device array of fixed size,
// reserved when the library is loaded on a device and held until the process exits.
//
// Limit: at most kStaticPaths = 262,144 paths per wave, so images of at most 262,144 pixels
// (512 x 512); samples run in waves of floor(262,144 / pixels) samples.  The array is 34.9 MB.
// Its device address is looked up once per device, with that device current, on the first
// call there (cudaGetSymbolAddress; the same call uploads the Sobol table and a marker word
// behind it).  Every later call looks
// the address up again and reads the marker back; if either changed (a device reset reloads
// the module, whose arrays then start zeroed) it repeats the set-up.  Every call shares the
// array and it keeps the last call's contents; the kernels reset what must start at zero.
// Calls whose work overlaps on the GPU (other streams, other host threads) race on the array:
// serialise them.

#include <cstring>
#include <mutex>

#include "nb_runtime.h"

namespace {

constexpr uint32_t kStaticPaths = 1u << 18;
constexpr size_t kQueueBytes = (size_t)kStaticPaths * 16;                 // one float4 per path
constexpr size_t kInstBytes = (size_t)kStaticPaths * 4;                   // hit instance ids
constexpr size_t kCounterBytes = 1024;                                    // counts, fetch, status, rays
constexpr size_t kSobolBytes = (size_t)nb::kMaxSampleCount * nb::kLdsStride * 16;
constexpr size_t kMarkerBytes = 256;                                      // set-up marker
constexpr size_t kSobolOffset = 8 * kQueueBytes + kInstBytes + kCounterBytes;
constexpr size_t kMarkerOffset = kSobolOffset + kSobolBytes;
constexpr size_t kScratchBytes = kMarkerOffset + kMarkerBytes;
constexpr unsigned long long kMarker = 0x6E625F7374617469ull;              // written after the table

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_base[kMaxDevices];    // device ordinal -> device address of g_scratch
nb::WaveTables g_tables;               // host staging of the kernel parameter tables
float g_table_host[(size_t)nb::kMaxSampleCount * nb::kLdsStride * 4];  // Sobol table staging

// Device address of the scratch array on the current device.  The first call per device
// looks it up and uploads the Sobol table and the marker; later calls check that the address
// and the marker are unchanged (one 8-byte read on the caller's stream) and redo the set-up
// otherwise.
int scratch_base(cudaStream_t st, unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return nb::cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return nb::fail(NB_ERR_INVALID_ARG, "device ordinal %d out of range", dev);
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) return nb::cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
  unsigned char* base = (unsigned char*)p;
  if (g_base[dev] == base) {
    unsigned long long mark = 0;
    e = cudaMemcpyAsync(&mark, base + kMarkerOffset, sizeof(mark), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return nb::cuda_fail(e, "static scratch marker read");
    if (mark == kMarker) {
      *out = base;
      return NB_OK;
    }
  }
  g_base[dev] = nullptr;
  nb::sobol_burley_table(nb::kMaxSampleCount, nb::kLdsStride, 0, g_table_host);
  e = cudaMemcpy(base + kSobolOffset, g_table_host, kSobolBytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return nb::cuda_fail(e, "cudaMemcpy(Sobol table)");
  const unsigned long long mark = kMarker;
  e = cudaMemcpy(base + kMarkerOffset, &mark, sizeof(mark), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return nb::cuda_fail(e, "cudaMemcpy(static scratch marker)");
  g_base[dev] = base;
  *out = base;
  return NB_OK;
}

}  // namespace

extern "C" int nb_render_static(const nb_scene* scene, const nb_env* env, const nb_camera* camera, uint32_t width,
                                uint32_t height, uint32_t first_sample, uint32_t n_samples, uint32_t bounces,
                                float contribution_factor, float* out_rgba, void* stream) {
  using namespace nb;
  if (!scene || !env || !camera || !out_rgba) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (!scene->uploaded) return fail(NB_ERR_INVALID_ARG, "scene was built with NB_SCENE_HOST_ONLY");
  const uint64_t npix = (uint64_t)width * height;
  if (npix == 0) return fail(NB_ERR_INVALID_ARG, "empty image");
  if (npix > kStaticPaths)
    return fail(NB_ERR_INVALID_ARG, "image of %llu pixels exceeds the static scratch (%u paths per wave)",
                (unsigned long long)npix, kStaticPaths);
  if (first_sample == 0 || (uint64_t)first_sample + n_samples - 1 > kMaxSampleCount)
    return fail(NB_ERR_INVALID_ARG, "samples must lie in Sobol rows 1..%u", kMaxSampleCount);
  if (bounces + 2 > kMaxBounceSlots) return fail(NB_ERR_INVALID_ARG, "bounces must be <= %u", kMaxBounceSlots - 2);
  if (n_samples == 0) return NB_OK;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* base = nullptr;
  int rc = scratch_base(st, &base);
  if (rc) return rc;

  PathBatch pb{};
  float4* q = (float4*)base;
  pb.q_o[0] = q; pb.q_o[1] = q + kStaticPaths;
  pb.q_d[0] = q + 2 * kStaticPaths; pb.q_d[1] = q + 3 * kStaticPaths;
  pb.q_t[0] = q + 4 * kStaticPaths; pb.q_t[1] = q + 5 * kStaticPaths;
  pb.hits = q + 6 * kStaticPaths;
  pb.radiance = q + 7 * kStaticPaths;
  pb.hit_inst = (uint32_t*)(base + 8 * kQueueBytes);
  uint32_t* counters = (uint32_t*)(base + 8 * kQueueBytes + kInstBytes);
  pb.counts = counters;
  pb.fetch = counters + kMaxBounceSlots;
  pb.status = counters + 2 * kMaxBounceSlots;
  unsigned long long* rays = (unsigned long long*)(counters + 2 * kMaxBounceSlots + 2);
  pb.sobol = (const float4*)(base + kSobolOffset);
  pb.sobol_entries = kMaxSampleCount * kLdsStride;
  cudaError_t e = cudaMemsetAsync(pb.status, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");

  WaveTables& wt = g_tables;
  wt.n_jobs = wt.n_scenes = wt.n_segs = 1;
  wt.flags = 0u;  // reference estimator: every path's radiance is written where it ends
  wt.scenes[0] = scene->dev;
  JobParams& jp = wt.jobs[0];
  std::memcpy(jp.c2w, camera->clip_to_world, sizeof(jp.c2w));
  jp.env = env->dev;
  jp.out = (float4*)out_rgba;
  jp.scene = 0;
  jp.width = width;
  jp.height = height;
  jp.npix = (uint32_t)npix;
  jp.bounces = bounces;
  jp.cf = contribution_factor;
  const int sms = sm_count();
  const uint32_t per_wave = kStaticPaths / (uint32_t)npix;
  for (uint32_t done = 0; done < n_samples && e == cudaSuccess;) {
    const uint32_t S = std::min(per_wave, n_samples - done);
    wt.segs[0] = Segment{0u, first_sample + done, S, 0u, 0u};
    wt.n_paths = (uint32_t)npix * S;
    wt.n_pix = (uint32_t)npix;
    e = launch_raygen(pb, wt, sms, st);
    for (uint32_t b = 0; b <= bounces && e == cudaSuccess; ++b) {
      e = launch_trace_wave(pb, wt, true, b, rays, sms, st);
      if (e == cudaSuccess) e = launch_shade(pb, wt, b, sms, st);
    }
    if (e == cudaSuccess) e = launch_accumulate(pb, wt, sms, st);
    done += S;
  }
  if (e != cudaSuccess) return cuda_fail(e, "static render launch");
  uint32_t status = 0;
  e = cudaMemcpyAsync(&status, pb.status, sizeof(status), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "static render");
  if (status & nbd::kStatusStackOverflow) return fail(NB_ERR_STACK_OVERFLOW, "traversal stack overflow");
  if (status & nbd::kStatusIterationCap) return fail(NB_ERR_TIMEOUT, "traversal iteration cap reached");
  return NB_OK;
}

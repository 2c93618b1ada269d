// Host runtime pieces shared by the C ABI (nb_api.cu) and the job server (nb_server.cu):
// CUDA error mapping, the device allocation arena and the scene / environment handles.
#pragma once

#include <cstdio>
#include <vector>

#include <cuda_runtime.h>

#include "nb_internal.h"
#include "nb_launch.h"

namespace nb {

inline int cuda_fail(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation) return fail(NB_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return fail(NB_ERR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
  return fail(NB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define NB_CUDA(call, what)                       \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

inline int sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  return sms > 0 ? sms : 1;
}

// A list of device allocations released together.
struct DeviceArena {
  std::vector<void*> ptrs;
  size_t bytes = 0;
  template <class T>
  int upload(const std::vector<T>& v, const T** out) {
    if (v.empty()) { *out = nullptr; return NB_OK; }
    void* p = nullptr;
    NB_CUDA(cudaMalloc(&p, v.size() * sizeof(T)), "cudaMalloc(scene)");
    ptrs.push_back(p);
    bytes += v.size() * sizeof(T);
    NB_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy(scene)");
    *out = (const T*)p;
    return NB_OK;
  }
  int alloc(size_t n, void** out) {
    void* p = nullptr;
    NB_CUDA(cudaMalloc(&p, n), "cudaMalloc");
    ptrs.push_back(p);
    bytes += n;
    *out = p;
    return NB_OK;
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
    bytes = 0;
  }
};

// nb_bc6h.cu: BC6H blocks (layers x ceil(height / 4) x ceil(width / 4) 16-byte blocks, device)
// decoded into layers x height x width RGBA32F texels (device), alpha 1.
int decode_bc6h_device(const void* d_blocks, uint32_t width, uint32_t height, uint32_t layers, bool is_signed,
                       float4* d_out, cudaStream_t stream);

// nb_bc6h.cu: a DDS cube map's format, face size and the mip-0 data of its six faces.
enum DdsFormat : uint32_t { kDdsBc6hUf16, kDdsBc6hSf16, kDdsRgba16f, kDdsRgba32f };
struct DdsCube {
  uint32_t format = 0;
  uint32_t size = 0;
  const uint8_t* face[6] = {};
  size_t face_bytes = 0;
};
int parse_dds_cube(const uint8_t* bytes, size_t n, DdsCube* out);

}  // namespace nb

struct nb_scene {
  nb::HostScene host;
  nbd::DevScene dev{};
  nb::DeviceArena arena;
  uint32_t* d_fetch = nullptr;
  uint32_t* d_status = nullptr;
  int sms = 1;
  bool uploaded = false;
};

struct nb_env {
  nbd::DevEnv dev{};
  nb::DeviceArena arena;
};

// radiance-cache mode of a wave (nb_cache.cu)
namespace nb {
struct CacheWave;
// before raygen: buffers, counters and the wave state read by launch_shade_cache
int cache_wave_begin(nb_cache* c, const nb_scene* scene, uint32_t n_paths, CacheWave* cw, cudaStream_t st);
// after the last bounce: cache lookups (image queries and training-path tails)
int cache_wave_infer(nb_cache* c, const PathBatch& pb, int sms, cudaStream_t st);
// then: training records and optimiser steps
int cache_wave_train(nb_cache* c, uint32_t n_paths, int sms, cudaStream_t st);
}  // namespace nb

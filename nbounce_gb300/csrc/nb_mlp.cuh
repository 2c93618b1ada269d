// Radiance cache: record layouts, the cache-mode wave descriptor and the input encoding.
//
// The cache is a fully fused MLP (Mueller, Rousselle, Novak, Keller 2021, "Real-time Neural
// Radiance Caching for Path Tracing"): 64 encoded inputs -> 5 hidden layers of 64 (ReLU) ->
// 3 outputs (RGB), no biases (input 62 is a constant 1).  Weights are one flat FP32 array
//   layer l < 5 : W_l[out][in], 64 x 64, at l * 4096
//   layer 5     : W_5[out][in], 16 x 64, at 20480 (rows 3..15 stay zero)
// i.e. 336 rows of 64 inputs; the tensor-core kernels read a BF16 copy of the same layout.
//
// The network predicts outgoing radiance divided by (diffuse + specular reflectance) of the
// vertex ("reflectance factorisation" of the paper); callers multiply by it again.
#pragma once

#include <cstdint>

#include "nb_device.cuh"

namespace nb {

constexpr int kMlpWidth = 64;
constexpr int kMlpHidden = 5;
constexpr int kMlpOutPad = 16;
constexpr int kMlpOutputs = 3;
constexpr int kMlpRows = kMlpHidden * kMlpWidth + kMlpOutPad;  // 336 weight rows
constexpr int kMlpParams = kMlpRows * kMlpWidth;                // 21,504
constexpr int kMlpLiveParams = kMlpHidden * kMlpWidth * kMlpWidth + kMlpOutputs * kMlpWidth;  // 20,672

constexpr uint32_t kCacheMaxVertices = 8;     // recorded vertices per training path
constexpr uint32_t kCacheTailBit = 0x80000000u;  // query target: training slot instead of path id
constexpr uint32_t kCacheMaxStride = 1u << 20;

// Inputs of one cache lookup (64 B).  tag: path id of a query, unused in training vertices.
struct CacheFeatures {
  float pos[3];
  float roughness;
  float wo[3];
  float metallic;
  float n[3];
  uint32_t tag;
  float color[3];
  float pad;
};
static_assert(sizeof(CacheFeatures) == 64, "CacheFeatures");

// A path's prefix ends here: its pixel gets T * cache(x).  (80 B)
struct CacheQuery {
  CacheFeatures f;
  float4 T;
};
// One vertex of a training path; w = throughput factor to the next vertex (BSDF weight over
// the Russian-roulette probability), 0 where the path was terminated.  (80 B)
struct TrainVertex {
  CacheFeatures f;
  float4 w;
};
static_assert(sizeof(CacheQuery) == 80 && sizeof(TrainVertex) == 80, "cache records");

struct CacheBounds {
  float lo[3];
  float inv_extent[3];
};

// Device state of one cache-mode wave (passed by value).
struct CacheWave {
  float4* q_x[2];          // per queued ray (double-buffered like the ray queues): x = spread
                           // budget left, y = density of the ray's direction, z = training slot
                           // (bits, ~0u if none), w = flags (bits)
  CacheQuery* queries;     // lookups of this wave (image queries and training-path tails)
  uint32_t* n_queries;
  uint32_t max_queries;
  TrainVertex* verts;      // [slot][kCacheMaxVertices]
  uint32_t* vert_count;    // per slot
  float4* tail;            // per slot: radiance arriving after the last recorded vertex
  const uint32_t* stride;  // training-path group size (one training path per group of paths)
  uint32_t max_slots;
  uint32_t frame;          // varies the training path chosen in each group
  float spread_c;          // terminate when the path spread exceeds c * a0; < 0: at the primary hit
  uint32_t extra;          // training vertices recorded past the query vertex
};

// q_x.w flags
constexpr uint32_t kPathImageDone = 1u << 0;  // the pixel sample was resolved by a query
constexpr uint32_t kPathTraining = 1u << 1;
constexpr uint32_t kPathSinceShift = 8;       // vertices recorded since the query, bits 8..15

}  // namespace nb

namespace nbd {

// Triangular one-blob: 4 bins over [0,1], bin i peaks at (i + 0.5) / 4 and falls to 0 one bin
// away (Mueller et al. 2019 one-blob with a triangular instead of a Gaussian kernel).
__device__ __forceinline__ void one_blob4(float s, float* f) {
#pragma unroll
  for (int i = 0; i < 4; ++i) f[i] = fmaxf(0.0f, 1.0f - fabsf(s * 4.0f - ((float)i + 0.5f)));
}

// Triangle wave of period 1 with values in [-1, 1]: 1 at integers, -1 at half-integers.
__device__ __forceinline__ float tri_wave(float x) { return fabsf(4.0f * fract(x) - 2.0f) - 1.0f; }

// The 64 network inputs of a vertex:
//   0..35   position normalised to the scene box, triangle waves of 12 octaves per axis
//           (axis-major: feature 12 a + k = tri(p_a 2^k))
//   36..43  one-blob of the outgoing direction in spherical coordinates (theta/pi, phi/2pi+1/2)
//   44..51  one-blob of the shading normal, same mapping
//   52..55  one-blob of the roughness
//   56..58  diffuse reflectance (1 - metallic) * color
//   59..61  specular reflectance F0 = 0.04 (1 - metallic) + color * metallic
//   62      1, 63 0
__device__ __forceinline__ void cache_encode(const nb::CacheFeatures& v, const nb::CacheBounds& b, float* f) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float p = (v.pos[a] - b.lo[a]) * b.inv_extent[a];
    p = fminf(fmaxf(p, 0.0f), 1.0f);
    float s = 1.0f;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      f[12 * a + k] = tri_wave(p * s);
      s *= 2.0f;
    }
  }
  const float inv_pi = 0.318309886f, inv_2pi = 0.159154943f;
  one_blob4(nb_acos(fminf(fmaxf(v.wo[2], -1.0f), 1.0f)) * inv_pi, f + 36);
  one_blob4(nb_atan2(v.wo[1], v.wo[0]) * inv_2pi + 0.5f, f + 40);
  one_blob4(nb_acos(fminf(fmaxf(v.n[2], -1.0f), 1.0f)) * inv_pi, f + 44);
  one_blob4(nb_atan2(v.n[1], v.n[0]) * inv_2pi + 0.5f, f + 48);
  one_blob4(v.roughness, f + 52);
  const float m = v.metallic;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    f[56 + c] = (1.0f - m) * v.color[c];
    f[59 + c] = 0.04f * (1.0f - m) + v.color[c] * m;
  }
  f[62] = 1.0f;
  f[63] = 0.0f;
}

// Reflectance factor the network output is scaled by: diffuse + specular reflectance,
// floored so that black materials keep a finite training target.
__device__ __forceinline__ V3 cache_factor(const nb::CacheFeatures& v) {
  const float m = v.metallic;
  V3 r;
  r.x = fmaxf((1.0f - m) * v.color[0] + (0.04f * (1.0f - m) + v.color[0] * m), 1e-3f);
  r.y = fmaxf((1.0f - m) * v.color[1] + (0.04f * (1.0f - m) + v.color[1] * m), 1e-3f);
  r.z = fmaxf((1.0f - m) * v.color[2] + (0.04f * (1.0f - m) + v.color[2] * m), 1e-3f);
  return r;
}

}  // namespace nbd

// Device-side math and scene view for the nBounce pass kernels.
//
// Arithmetic contract (the same one the CPU oracle states; both follow the WGSL source):
// every expression is evaluated left to right in IEEE binary32, round to nearest, with no
// contraction - this translation unit is compiled with -fmad=false, -prec-div=true,
// -prec-sqrt=true, -ftz=false - and the WGSL builtins are pinned as
//   dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, cross the usual three differences,
//   normalize(v) = v / sqrt(dot(v,v)), M*v = ((M0*v.x + M1*v.y) + M2*v.z) (+ M3*v.w),
//   mix(a,b,t) = a*(1-t) + b*t, min/max = fminf/fmaxf, pow(x,n) = repeated products,
//   sin/cos = Cody-Waite reduction by pi/2 + Taylor polynomials (nb_sincos below).
// With identical inputs the kernels therefore produce the oracle's bits; the remaining
// differences come from traversal near-ties (documented in the tests).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace nbd {

constexpr float kNoHit = 3.40282346638528859812e+38f;  // raytracing_sw.wgsl:1-2
constexpr float kEps = 0.00000001f;                     // raytracing_sw.wgsl:3
constexpr float kBias = 0.1f;                           // raytracing_sw.wgsl:4
constexpr float kPi = 3.14159265359f;                   // common.wgsl:1
constexpr float kTwoPi = 2.0f * kPi;
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kLdsStride = 17u;
constexpr uint32_t kLdsPerBounce = 2u;

// status word bits written by kernels (read back by the host)
constexpr uint32_t kStatusStackOverflow = 1u << 0;
constexpr uint32_t kStatusIterationCap = 1u << 1;

// Correctly rounded 1 / b for b in [kRcpNewtonMin, kRcpNewtonMax) without a division: the
// hardware's approximate reciprocal refined by one Newton-Raphson step in fused multiply-adds,
// e = 1 - b y, y + y e (Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990).  Compared bit for bit with the
// correctly rounded division for every float of that range by tests/test_gpu_reciprocal.py
// (1,280,586,633 values, no difference); outside it the caller divides.  Below 2^126 the
// reciprocal stays a normal number, which the flush-to-zero approximation needs.
constexpr float kRcpNewtonMin = 1e-8f;  // kEps: the smallest determinant a triangle test divides by
constexpr float kRcpNewtonMax = 0x1p126f;
__device__ __forceinline__ float rcp_newton(float b) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(b));
  return fmaf(fmaf(-b, y, 1.0f), y, y);
}

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3 normalize(V3 v) {
  float l = sqrtf(dot(v, v));
  return V3{v.x / l, v.y / l, v.z / l};
}
__device__ __forceinline__ V3 rcp3(V3 v) { return V3{1.0f / v.x, 1.0f / v.y, 1.0f / v.z}; }
__device__ __forceinline__ float luminance(V3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
__device__ __forceinline__ float pow2(float x) { return x * x; }
__device__ __forceinline__ float pow5(float x) {
  float x2 = x * x;
  return x2 * x2 * x;
}
__device__ __forceinline__ float pow8(float x) {
  float x2 = x * x;
  float x4 = x2 * x2;
  return x4 * x4;
}
__device__ __forceinline__ V3 xyz(float4 q) { return V3{q.x, q.y, q.z}; }

// sin and cos of x for |x| < 64: Cody-Waite reduction by pi/2 with a three-part split of
// pi/2 (leading parts with 8 and 12 significant bits, so k*A and k*B are exact), then the
// Taylor polynomials of sin (degree 9) and cos (degree 10) on [-pi/4, pi/4] in Horner form.
__device__ __forceinline__ void nb_sincos(float x, float* s, float* c) {
  const float kA = 1.5703125f, kB = 0x1.fb6p-12f, kC = -0x1.777a5cp-25f;
  float kf = floorf(x * 0.636619772367581343f + 0.5f);
  int k = (int)kf;
  float r = ((x - kf * kA) - kf * kB) - kf * kC;
  float r2 = r * r;
  float ps = r + r * r2 * (-1.0f / 6.0f + r2 * (1.0f / 120.0f + r2 * (-1.0f / 5040.0f + r2 * (1.0f / 362880.0f))));
  float pc = 1.0f + r2 * (-0.5f + r2 * (1.0f / 24.0f + r2 * (-1.0f / 720.0f + r2 * (1.0f / 40320.0f + r2 * (-1.0f / 3628800.0f)))));
  switch (k & 3) {
    case 0: *s = ps; *c = pc; break;
    case 1: *s = pc; *c = -ps; break;
    case 2: *s = -ps; *c = -pc; break;
    default: *s = -pc; *c = ps; break;
  }
}

// PCG4D (common.wgsl:27-33) and map4f (common.wgsl:7-9)
__device__ __forceinline__ float4 hash4f(uint32_t x, uint32_t y) {
  uint32_t v0 = x * 1664525u + 1013904223u, v1 = y * 1664525u + 1013904223u;
  uint32_t v2 = v0, v3 = v1;
  v0 += v1 * v3; v1 += v2 * v0; v2 += v0 * v1; v3 += v1 * v2;
  v0 ^= v0 >> 16; v1 ^= v1 >> 16; v2 ^= v2 >> 16; v3 ^= v3 >> 16;
  v0 += v1 * v3; v1 += v2 * v0; v2 += v0 * v1; v3 += v1 * v2;
  return make_float4(__uint_as_float((v0 >> 9) | 0x3F800000u) - 1.0f, __uint_as_float((v1 >> 9) | 0x3F800000u) - 1.0f,
                     __uint_as_float((v2 >> 9) | 0x3F800000u) - 1.0f, __uint_as_float((v3 >> 9) | 0x3F800000u) - 1.0f);
}

__device__ __forceinline__ float fract(float x) { return x - floorf(x); }

// atan2 / acos in binary32 by octant reduction and a degree-7 polynomial in x^2 for atan on
// [0,1] (least-squares fit, max error 1.7e-7), Horner without fusion: the oracle
// evaluates the identical sequence, so both sides agree bit for bit.
__device__ __forceinline__ float nb_atan2(float y, float x) {
  const float P[8] = {0x1.fffffcp-1f, -0x1.5551dp-2f, 0x1.98faep-3f, -0x1.1f1e82p-3f,
                      0x1.96172p-4f,  -0x1.e75096p-5f, 0x1.8d5abp-6f, -0x1.3394dap-8f};
  float ax = fabsf(x), ay = fabsf(y);
  float mx = ax > ay ? ax : ay, mn = ax > ay ? ay : ax;
  float a = mx > 0.0f ? mn / mx : 0.0f;
  float a2 = a * a;
  float p = P[7];
#pragma unroll
  for (int k = 6; k >= 0; --k) p = p * a2 + P[k];
  float r = a * p;
  if (ay > ax) r = 1.57079637f - r;
  if (x < 0.0f) r = 3.14159274f - r;
  if (y < 0.0f) r = -r;
  return r;
}
__device__ __forceinline__ float nb_acos(float y) { return nb_atan2(sqrtf((1.0f - y) * (1.0f + y)), y); }

// Device view of a scene (pointers into library-owned device memory).
struct DevScene {
  const float4* tlas_wide;    // 5 float4 per 8-wide TLAS node; the root is node 0
  const float4* blas_wide;    // 5 float4 per 8-wide BLAS node
  const float4* inst_trace;   // 4 float4 per instance, in wide-TLAS leaf order
  const float4* inst_shade;   // 6 float4 per instance, reference (TLAS-permuted) order
  const float4* tris;         // 3 float4 per triangle, in wide-BLAS leaf order
  const uint32_t* tri_idx;    // 3 vertex ids per reference triangle
  const float4* vattr;        // 2 float4 per vertex
  uint32_t has_tlas;
  uint32_t n_tris, n_inst, n_vertices;
};

enum EnvKind : uint32_t { kEnvConstant = 0, kEnvEquirect = 1, kEnvCube = 2 };
struct DevEnv {
  uint32_t kind;
  float r, g, b;
  const float4* texels;
  uint32_t width, height;  // cube: width = face size, height = 6 x face size (faces stacked)
  // importance-sampling distribution of an equirect or cube map over its texel rows and
  // columns (piecewise constant over texels, weight = luminance x the texel's solid angle):
  // marginal CDF over rows (height + 1), conditional CDFs per row (height x (width + 1)),
  // density over (u, v) of the whole texel table per texel (width x height)
  const float* cdf_rows;
  const float* cdf_cols;
  const float* pdf_uv;
};

}  // namespace nbd

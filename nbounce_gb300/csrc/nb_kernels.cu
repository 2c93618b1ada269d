// CUDA kernels of the nBounce path-tracing pass for sm_103a.
//
// The reference runs one WGSL invocation per pixel that loops over bounces with the whole
// traversal inline (pathtracing.wgsl:161-260).  Here the pass is a wavefront:
//   raygen      one path per (pixel, sample) of a batch: Cranley-Patterson-rotated Sobol
//               jitter and generate_ray (pathtracing.wgsl:27-41, 245-255)
//   trace       persistent warps pull 32-ray chunks with one atomic each and run the
//               two-level stack traversal (raytracing_sw.wgsl:176-319) on the device layout
//   shade       hit attributes (raytracing_sw.wgsl:138-173), env/emission termination, lobe
//               choice, VNDF / cosine sampling, Russian roulette (pathtracing.wgsl:161-241);
//               survivors are appended to the next bounce's queue with warp-aggregated atomics
//   accumulate  running mean over the batch's samples in sample order (pathtracing.wgsl:258)
// so traversal runs in a lean kernel at full occupancy and the path state lives in HBM.
//
// Traversal differs from the reference in two work-saving ways that leave results unchanged
// except for near-ties: the current closest hit prunes BLAS nodes (the reference restarts
// each BLAS from NO_HIT, raytracing_sw.wgsl:255) and one stack serves both levels.

#include <algorithm>
#include <cstdint>

#include "nb_device.cuh"
#include "nb_launch.h"

namespace nbd {

using nb::CameraParams;
using nb::kMaxBounceSlots;
using nb::PathBatch;

constexpr int kStackSize = 64;
constexpr uint32_t kIterationCap = 1u << 22;

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }

// slab test (raytracing_sw.wgsl:81-89)
__device__ __forceinline__ float slab(V3 ro, V3 rinv, float mnx, float mxx, float mny, float mxy, float mnz,
                                      float mxz) {
  float tminx = (mnx - ro.x) * rinv.x, tmaxx = (mxx - ro.x) * rinv.x;
  float tminy = (mny - ro.y) * rinv.y, tmaxy = (mxy - ro.y) * rinv.y;
  float tminz = (mnz - ro.z) * rinv.z, tmaxz = (mxz - ro.z) * rinv.z;
  float t1x = fminf(tminx, tmaxx), t1y = fminf(tminy, tmaxy), t1z = fminf(tminz, tmaxz);
  float t2x = fmaxf(tminx, tmaxx), t2y = fmaxf(tminy, tmaxy), t2z = fmaxf(tminz, tmaxz);
  float tn = fmaxf(t1x, fmaxf(t1y, t1z));
  float tf = fminf(t2x, fminf(t2y, t2z));
  return (tn <= tf && tf >= 0.0f) ? tn : kNoHit;
}

struct Hit {
  float t, u, v;
  uint32_t tri, inst;
};

// Traversal state of one lane (one ray) in the persistent kernels.  The stack lives in
// local memory; everything else stays in registers.
struct Lane {
  V3 wo, wd, winv;  // world ray
  V3 ro, rd, rinv;  // ray of the current level (world, or instance-local inside a BLAS)
  Hit h;
  int sp, blas_base;
  uint32_t inst_cur, inst_end, cur_inst;
  uint32_t ray, iter;
  bool in_blas;
};

__device__ __forceinline__ void push(Lane& L, uint2* stack, uint32_t ref, float d, uint32_t& status) {
  if (L.sp < kStackSize) {
    stack[L.sp] = make_uint2(ref, __float_as_uint(d));
    ++L.sp;
  } else {
    status |= kStatusStackOverflow;
  }
}

// Enter the BLAS of instance j: transform the world ray (raytracing_sw.wgsl:202-206), test
// the BLAS root box and push the root (raytracing_sw.wgsl:259-265).
__device__ __forceinline__ void enter_instance(const DevScene& s, Lane& L, uint2* stack, uint32_t j,
                                               uint32_t& status) {
  const float4* it = s.inst_trace + 4 * (size_t)j;
  const float4 r0 = ld4(it), r1 = ld4(it + 1), r2 = ld4(it + 2);
  const uint32_t root = __float_as_uint(ld4(it + 3).x);
  const V3 wo = L.wo, wd = L.wd;
  L.ro = V3{r0.x * wo.x + r0.y * wo.y + r0.z * wo.z + r0.w * 1.0f, r1.x * wo.x + r1.y * wo.y + r1.z * wo.z + r1.w * 1.0f,
            r2.x * wo.x + r2.y * wo.y + r2.z * wo.z + r2.w * 1.0f};
  L.rd = V3{r0.x * wd.x + r0.y * wd.y + r0.z * wd.z, r1.x * wd.x + r1.y * wd.y + r1.z * wd.z,
            r2.x * wd.x + r2.y * wd.y + r2.z * wd.z};
  L.rinv = rcp3(L.rd);
  L.cur_inst = j;
  const float4 lo = ld4(s.blas_roots + 2 * (size_t)root), hi = ld4(s.blas_roots + 2 * (size_t)root + 1);
  const float d = slab(L.ro, L.rinv, lo.x, hi.x, lo.y, hi.y, lo.z, hi.z);
  if (d < L.h.t) push(L, stack, __float_as_uint(lo.w), d, status);
}

// Start a new ray: test the TLAS root and push it (raytracing_sw.wgsl:182-191).
__device__ __forceinline__ void lane_start(const DevScene& s, Lane& L, uint2* stack, V3 o, V3 d, uint32_t& status) {
  L.wo = o; L.wd = d; L.winv = rcp3(d);
  L.ro = o; L.rd = d; L.rinv = L.winv;
  L.h.t = kNoHit; L.h.u = 0.0f; L.h.v = 0.0f; L.h.tri = 0xFFFFFFFFu; L.h.inst = 0xFFFFFFFFu;
  L.sp = 0; L.blas_base = 0; L.in_blas = false; L.iter = 0;
  L.inst_cur = L.inst_end = L.cur_inst = 0;
  if (!s.has_tlas) return;
  const float4 lo = s.tlas_root_lo, hi = s.tlas_root_hi;
  const float dr = slab(o, L.winv, lo.x, hi.x, lo.y, hi.y, lo.z, hi.z);
  if (dr < L.h.t) push(L, stack, __float_as_uint(lo.w), dr, status);
}

// One stack pop of the two-level traversal.  Returns true when the ray is finished.
template <bool kAny>
__device__ __forceinline__ bool lane_step(const DevScene& s, Lane& L, uint2* stack, uint32_t& status) {
  if (++L.iter > kIterationCap) {
    status |= kStatusIterationCap;
    return true;
  }
  if (L.in_blas && L.sp == L.blas_base) {
    if (L.inst_cur < L.inst_end) {  // next instance of the TLAS leaf (raytracing_sw.wgsl:201)
      enter_instance(s, L, stack, L.inst_cur++, status);
      return false;
    }
    L.in_blas = false;
    L.ro = L.wo; L.rd = L.wd; L.rinv = L.winv;
  }
  if (L.sp == 0) return true;
  --L.sp;
  const uint2 e = stack[L.sp];
  if (__uint_as_float(e.y) >= L.h.t) return false;  // raytracing_sw.wgsl:197,271
  const uint32_t ref = e.x;
  if (ref & kLeafBit) {
    const uint32_t first = ref & ~kLeafBit;
    if (!L.in_blas) {
      // TLAS leaf: its instances one after the other (raytracing_sw.wgsl:200-217)
      const uint32_t n = __float_as_uint(ld4(s.inst_trace + 4 * (size_t)first + 3).y);
      L.inst_cur = first + 1;
      L.inst_end = first + n;
      L.in_blas = true;
      L.blas_base = L.sp;
      enter_instance(s, L, stack, first, status);
      return false;
    }
    // BLAS leaf: Moller-Trumbore over the leaf's triangles (raytracing_sw.wgsl:51-78, 274-286)
    const float4* tp = s.tris + 3 * (size_t)first;
    float4 a = ld4(tp);
    const uint32_t n = __float_as_uint(a.w);
    for (uint32_t k = 0; k < n; ++k) {
      if (k) a = ld4(tp + 3 * k);
      const float4 b = ld4(tp + 3 * k + 1), c = ld4(tp + 3 * k + 2);
      const V3 e1 = xyz(b), e2 = xyz(c);
      const V3 hv = cross(L.rd, e2);
      const float det = dot(e1, hv);
      if (det < kEps) continue;
      const float inv_det = 1.0f / det;
      const V3 sv = L.ro - xyz(a);
      const float u = inv_det * dot(sv, hv);
      if (u < 0.0f || u > 1.0f) continue;
      const V3 q = cross(sv, e1);
      const float v = inv_det * dot(L.rd, q);
      if (v < 0.0f || u + v > 1.0f) continue;
      const float t = inv_det * dot(e2, q);
      if (t < kBias) continue;
      if (t < L.h.t) {
        L.h.t = t; L.h.u = u; L.h.v = v;
        L.h.tri = first + k;
        L.h.inst = L.cur_inst;
        if (kAny) return true;
      }
    }
    return false;
  }
  // inner node: test both children, push far then near (raytracing_sw.wgsl:218-247)
  const float4* np = (L.in_blas ? s.blas_nodes : s.tlas_nodes) + 4 * (size_t)ref;
  const float4 q0 = ld4(np), q1 = ld4(np + 1), q2 = ld4(np + 2), q3 = ld4(np + 3);
  const float dl = slab(L.ro, L.rinv, q0.x, q0.y, q0.z, q0.w, q2.x, q2.y);
  const float dr = slab(L.ro, L.rinv, q1.x, q1.y, q1.z, q1.w, q2.z, q2.w);
  const uint32_t lref = __float_as_uint(q3.x), rref = __float_as_uint(q3.y);
  uint32_t fref = lref, nref = rref;
  float fd = dl, nd = dr;
  if (dl < dr) { fref = rref; fd = dr; nref = lref; nd = dl; }
  if (fd < L.h.t) push(L, stack, fref, fd, status);
  if (nd < L.h.t) push(L, stack, nref, nd, status);
  return false;
}

// Persistent traversal over rays [0, n): every lane whose ray finished takes the next ray
// (one warp-aggregated atomic per refill), so warps stay full until the work runs out
// instead of waiting for their slowest ray.
constexpr uint32_t kFullMask = 0xFFFFFFFFu;
template <bool kAny, class Io>
__device__ __forceinline__ void trace_persistent(const DevScene& s, const Io& io, uint32_t n, uint32_t* fetch,
                                                 uint32_t* status_out) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint2 stack[kStackSize];
  Lane L;
  bool active = false, retired = false;
  uint32_t status = 0;
  while (true) {
    const bool want = !active && !retired;
    const uint32_t wmask = __ballot_sync(kFullMask, want);
    if (wmask) {
      const int leader = __ffs(wmask) - 1;
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(wmask));
      base = __shfl_sync(kFullMask, base, leader);
      if (want) {
        const uint32_t idx = base + (uint32_t)__popc(wmask & lt_mask);
        if (idx < n) {
          V3 o, d;
          io.load(idx, o, d);
          L.ray = idx;
          lane_start(s, L, stack, o, d, status);
          active = true;
        } else {
          retired = true;
        }
      }
    }
    if (!__any_sync(kFullMask, active)) break;
    if (active && lane_step<kAny>(s, L, stack, status)) {
      io.store(L.ray, L.h);
      active = false;
    }
  }
  if (status) atomicOr(status_out, status);
}

struct QueryIo {  // caller rays of 8 floats (origin, pad, direction, pad)
  const float4* rays;
  float4* hits;
  uint32_t* inst;
  __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d) const {
    o = xyz(__ldg(rays + 2 * (size_t)i));
    d = xyz(__ldg(rays + 2 * (size_t)i + 1));
  }
  __device__ __forceinline__ void store(uint32_t i, const Hit& h) const {
    hits[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.tri));
    if (inst) inst[i] = h.inst;
  }
};

// ------------------------------------------------------------------------------------------
// traversal-only query (nb_trace_rays)
// ------------------------------------------------------------------------------------------
template <bool kAny>
__global__ void __launch_bounds__(128, 8) k_trace_rays(DevScene s, const float4* __restrict__ rays, uint32_t n,
                                                     float4* __restrict__ hits, uint32_t* __restrict__ inst,
                                                     uint32_t* __restrict__ fetch, uint32_t* __restrict__ status) {
  trace_persistent<kAny>(s, QueryIo{rays, hits, inst}, n, fetch, status);
}

// ------------------------------------------------------------------------------------------
// wavefront path tracer
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float4 sobol_read(const float4* table, uint32_t n_entries, uint32_t idx) {
  return idx < n_entries ? __ldg(table + idx) : make_float4(0.f, 0.f, 0.f, 0.f);  // robust buffer access
}

// generate_ray (pathtracing.wgsl:27-41)
__device__ __forceinline__ void generate_ray(uint32_t x, uint32_t y, uint32_t W, uint32_t H, float rx, float ry,
                                             const CameraParams& cam, V3* o, V3* d) {
  float uvx = 2.0f * ((float)x + rx) / (float)W - 1.0f;
  float uvy = 2.0f * ((float)y + ry) / (float)H - 1.0f;
  const float* m = cam.c2w;
  V3 pos = V3{m[12], m[13], m[14]} / m[15];
  float cx = -uvx, cy = -uvy, cz = -1.0f, cw = 1.0f;
  float wd[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) wd[r] = m[r] * cx + m[4 + r] * cy + m[8 + r] * cz + m[12 + r] * cw;
  *o = pos;
  *d = pos - V3{wd[0], wd[1], wd[2]} / wd[3];
}

__global__ void __launch_bounds__(256) k_raygen(PathBatch pb, CameraParams cam) {
  const uint32_t n = pb.n_paths;
  if (blockIdx.x == 0 && threadIdx.x < kMaxBounceSlots) {
    pb.counts[threadIdx.x] = threadIdx.x == 0 ? n : 0u;
    pb.fetch[threadIdx.x] = 0u;
  }
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    uint32_t pix = p % pb.npix;
    uint32_t sample = pb.first_sample + p / pb.npix;
    uint32_t x = pix % pb.width, y = pix / pb.width;
    float4 shift = hash4f(x, y);
    float4 sb = sobol_read(pb.sobol, pb.sobol_entries, sample * kLdsStride);
    float jx = fract(sb.x + shift.x), jy = fract(sb.y + shift.y);
    V3 o, d;
    generate_ray(x, y, pb.width, pb.height, jx, jy, cam, &o, &d);
    pb.q_o[0][p] = make_float4(o.x, o.y, o.z, __uint_as_float(p));
    pb.q_d[0][p] = make_float4(d.x, d.y, d.z, 0.0f);
    pb.q_t[0][p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    pb.radiance[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}

struct WaveIo {  // the bounce's ray queue and hit buffers
  const float4* qo;
  const float4* qd;
  float4* hits;
  uint32_t* inst;
  __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d) const {
    o = xyz(qo[i]);
    d = xyz(qd[i]);
  }
  __device__ __forceinline__ void store(uint32_t i, const Hit& h) const {
    hits[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.tri));
    inst[i] = h.inst;
  }
};

__global__ void __launch_bounds__(128, 8) k_trace_wave(DevScene s, PathBatch pb, uint32_t bounce,
                                                    unsigned long long* __restrict__ ray_total) {
  const uint32_t n = pb.counts[bounce];
  const WaveIo io{(bounce & 1) ? pb.q_o[1] : pb.q_o[0], (bounce & 1) ? pb.q_d[1] : pb.q_d[0], pb.hits, pb.hit_inst};
  trace_persistent<false>(s, io, n, pb.fetch + bounce, pb.status);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(ray_total, (unsigned long long)n);
}

// atan2 / acos in binary32 by octant reduction and a degree-7 polynomial in x^2 for atan on
// [0,1] (fitted for this build, max error 1.7e-7), Horner without fusion: the oracle
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

// equirect lookup (the oracle's definition): u = atan2(d.x, -d.z)/(2 pi) + 0.5, v = acos(d.y)/pi
// of the normalised direction, bilinear with wrap in u and clamp in v; NaN directions see black
__device__ V3 env_lookup(const DevEnv& env, V3 dir) {
  if (env.kind == kEnvConstant) return V3{env.r, env.g, env.b};
  V3 d = normalize(dir);
  float u = nb_atan2(d.x, -d.z) * 0.159154943f + 0.5f;
  float v = nb_acos(fminf(fmaxf(d.y, -1.0f), 1.0f)) * 0.318309886f;
  float fx = u * (float)env.width - 0.5f, fy = v * (float)env.height - 0.5f;
  if (fx != fx || fy != fy) return V3{0.0f, 0.0f, 0.0f};
  float x0 = floorf(fx), y0 = floorf(fy);
  float tx = fx - x0, ty = fy - y0;
  int W = (int)env.width, H = (int)env.height;
  int xi = (int)x0, yi = (int)y0;
  int xa = ((xi % W) + W) % W, xb = (((xi + 1) % W) + W) % W;
  int ya = yi < 0 ? 0 : (yi > H - 1 ? H - 1 : yi), yb = yi + 1 < 0 ? 0 : (yi + 1 > H - 1 ? H - 1 : yi + 1);
  float4 t00 = __ldg(env.texels + (size_t)ya * W + xa), t10 = __ldg(env.texels + (size_t)ya * W + xb);
  float4 t01 = __ldg(env.texels + (size_t)yb * W + xa), t11 = __ldg(env.texels + (size_t)yb * W + xb);
  return V3{(t00.x * (1.0f - tx) + t10.x * tx) * (1.0f - ty) + (t01.x * (1.0f - tx) + t11.x * tx) * ty,
            (t00.y * (1.0f - tx) + t10.y * tx) * (1.0f - ty) + (t01.y * (1.0f - tx) + t11.y * tx) * ty,
            (t00.z * (1.0f - tx) + t10.z * tx) * (1.0f - ty) + (t01.z * (1.0f - tx) + t11.z * tx) * ty};
}

// sample_vndf_iso (pathtracing.wgsl:68-98)
__device__ __forceinline__ V3 sample_vndf_iso(float r0, float r1, V3 wi, float alpha, V3 n) {
  if (alpha == 0.0f) return n;
  V3 wi_z = n * dot(wi, n);
  V3 wi_xy = wi - wi_z;
  V3 wiStd = normalize(wi_z - alpha * wi_xy);
  float wiStd_z = dot(wiStd, n);
  float phi = (2.0f * r0 - 1.0f) * kPi;
  float z = (1.0f - r1) * (1.0f + wiStd_z) - wiStd_z;
  float sinTheta = sqrtf(fminf(fmaxf(1.0f - z * z, 0.0f), 1.0f));
  float sp, cp;
  nb_sincos(phi, &sp, &cp);
  V3 cStd{sinTheta * cp, sinTheta * sp, z};
  V3 wr = n + V3{0.0f, 0.0f, 1.0f};
  float safe_wrz = fmaxf(wr.z, 1e-6f);
  V3 c = dot(wr, cStd) * wr / safe_wrz - cStd;
  V3 wmStd = c + wiStd;
  V3 wmStd_z = n * dot(n, wmStd);
  V3 wmStd_xy = wmStd_z - wmStd;
  return normalize(wmStd_z + alpha * wmStd_xy);
}

__device__ __forceinline__ V3 F_schlick(float hdotv, V3 r0) {  // pathtracing.wgsl:113-115
  float p = pow5(1.0f - hdotv);
  return r0 + (V3{1.0f, 1.0f, 1.0f} - r0) * p;
}
__device__ __forceinline__ float lambda_tr(float ndotv, float alpha2) {  // pathtracing.wgsl:119-125
  float cos2 = ndotv * ndotv;
  float sin2 = 1.0f - cos2;
  float tan2 = sin2 / cos2;
  return (-1.0f + sqrtf(1.0f + alpha2 * tan2)) / 2.0f;
}

__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool active) {
  const uint32_t mask = __ballot_sync(0xFFFFFFFFu, active);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
  base = __shfl_sync(0xFFFFFFFFu, base, leader < 0 ? 0 : leader);
  return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(256) k_shade(DevScene s, DevEnv env, PathBatch pb, uint32_t bounce,
                                               uint32_t bounces, float cf) {
  const uint32_t n = pb.counts[bounce];
  const bool odd = (bounce & 1) != 0;
  const float4* __restrict__ in_o = odd ? pb.q_o[1] : pb.q_o[0];
  const float4* __restrict__ in_d = odd ? pb.q_d[1] : pb.q_d[0];
  const float4* __restrict__ in_t = odd ? pb.q_t[1] : pb.q_t[0];
  float4* __restrict__ out_o = odd ? pb.q_o[0] : pb.q_o[1];
  float4* __restrict__ out_d = odd ? pb.q_d[0] : pb.q_d[1];
  float4* __restrict__ out_t = odd ? pb.q_t[0] : pb.q_t[1];
  const uint32_t stride = gridDim.x * blockDim.x;
  // whole warps iterate together so warp_append sees converged warps
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    bool cont = false;
    float4 next_o = make_float4(0.f, 0.f, 0.f, 0.f), next_d = next_o, next_t = next_o;
    if (i < n) {
      float4 O = in_o[i], D = in_d[i], Tq = in_t[i], H = pb.hits[i];
      const uint32_t id = __float_as_uint(O.w);
      V3 T = xyz(Tq);
      V3 rdir = xyz(D);
      if (H.x == kNoHit) {
        V3 L = T * env_lookup(env, rdir);
        pb.radiance[id] = make_float4(L.x, L.y, L.z, 0.0f);
      } else {
        const uint32_t inst = pb.hit_inst[i];
        const float4* sh = s.inst_shade + 6 * (size_t)inst;
        float4 c0 = ld4(sh), c1 = ld4(sh + 1), c2 = ld4(sh + 2);
        float4 l0 = ld4(sh + 3), l1 = ld4(sh + 4), l2 = ld4(sh + 5);
        V3 color{c0.w, c1.w, c2.w};
        if (l2.w > 0.0f) {  // EMISSIVE (raytracing_sw.wgsl:168-170, pathtracing.wgsl:172-174)
          V3 L = T * color;
          pb.radiance[id] = make_float4(L.x, L.y, L.z, 0.0f);
        } else {
          // hit attributes (raytracing_sw.wgsl:146-158)
          const uint32_t tri = __float_as_uint(H.w);
          const uint32_t i0 = __ldg(s.tri_idx + 3 * (size_t)tri), i1 = __ldg(s.tri_idx + 3 * (size_t)tri + 1),
                         i2 = __ldg(s.tri_idx + 3 * (size_t)tri + 2);
          float4 a0 = ld4(s.vattr + 2 * (size_t)i0), a1 = ld4(s.vattr + 2 * (size_t)i1), a2 = ld4(s.vattr + 2 * (size_t)i2);
          float4 b0 = ld4(s.vattr + 2 * (size_t)i0 + 1), b1 = ld4(s.vattr + 2 * (size_t)i1 + 1),
                 b2 = ld4(s.vattr + 2 * (size_t)i2 + 1);
          const float u = H.y, v = H.z;
          const float w0 = 1.0f - u - v;
          V3 ln = xyz(a0) * w0 + xyz(a1) * u + xyz(a2) * v;
          V3 lt = xyz(b0) * w0 + xyz(b1) * u + xyz(b2) * v;
          V3 nrm{dot(xyz(c0), ln), dot(xyz(c1), ln), dot(xyz(c2), ln)};
          V3 tng{dot(xyz(l0), lt), dot(xyz(l1), lt), dot(xyz(l2), lt)};
          V3 pos = xyz(O) + H.x * rdir;

          const uint32_t pix = id % pb.npix;
          const uint32_t sample = pb.first_sample + id / pb.npix;
          const float4 shift = hash4f(pix % pb.width, pix / pb.width);
          const float roughness = l0.w, metallic = l1.w;
          const float alpha = roughness * roughness;
          const float alpha2 = alpha * alpha;
          V3 nn = normalize(nrm);
          const uint32_t sb = sample * kLdsStride + 1u + bounce * kLdsPerBounce;
          float4 s0 = sobol_read(pb.sobol, pb.sobol_entries, sb);
          float4 s1 = sobol_read(pb.sobol, pb.sobol_entries, sb + 1u);
          s0 = make_float4(fract(s0.x + shift.x), fract(s0.y + shift.y), fract(s0.z + shift.z), 0.0f);
          s1 = make_float4(0.0f, fract(s1.y + shift.y), fract(s1.z + shift.z), 0.0f);
          V3 wo = normalize(-rdir);
          float cosThetaO = dot(wo, nn);
          V3 wi;
          V3 F0 = V3{0.04f, 0.04f, 0.04f} * (1.0f - metallic) + color * metallic;
          float specular_weight = luminance(F_schlick(dot(wo, nn), F0));
          float diffuse_weight = (1.0f - metallic) * luminance(color);
          float p_specular = specular_weight / (specular_weight + diffuse_weight);
          float p_diffuse = 1.0f - p_specular;
          if (s0.x < p_specular) {
            V3 wm = sample_vndf_iso(s0.y, s0.z, wo, alpha, nn);
            V3 ni = -wo;
            wi = ni - (2.0f * dot(wm, ni)) * wm;  // reflect(-wo, wm)
            float cosThetaD = dot(wo, wm);
            float cosThetaI = dot(wi, nn);
            V3 F = F_schlick(cosThetaD, F0);
            float LambdaL = lambda_tr(cosThetaI, alpha2);
            float LambdaV = lambda_tr(cosThetaO, alpha2);
            V3 spec = F * (1.0f + LambdaV) / (1.0f + LambdaL + LambdaV);
            T = T * (spec / p_specular);
          } else {
            V3 nt = normalize(tng - dot(tng, nn) * nn);  // build_tbn (common.wgsl:55-59)
            V3 bt = cross(nn, nt);
            float phi = kTwoPi * s1.y;
            float sinT = sqrtf(1.0f - s1.z);
            float cosT = sqrtf(s1.z);
            float sp, cp;
            nb_sincos(phi, &sp, &cp);
            V3 ls{cp * sinT, sp * sinT, cosT};
            wi = nt * ls.x + bt * ls.y + nn * ls.z;
            V3 wm = normalize(wi + wo);
            float cosThetaD = dot(wi, wm);
            float cosThetaI = dot(wi, nn);
            float FD90 = 0.5f + 2.0f * alpha * pow2(cosThetaD);
            float response = (1.0f + (FD90 - 1.0f) * pow5(1.0f - cosThetaI)) * (1.0f + (FD90 - 1.0f) * pow5(1.0f - cosThetaO));
            V3 diffuse = (1.0f - metallic) * color * response;
            T = T * (diffuse / p_diffuse);
          }
          // Russian roulette (pathtracing.wgsl:225-236)
          float p_continue = fminf(1.0f - pow8((float)bounce / (float)bounces), 1.0f);
          p_continue = p_continue * fminf(luminance(T) * cf, 1.0f);
          if (s0.z < p_continue && bounce < bounces) {
            T = T / p_continue;
            cont = true;
            next_o = make_float4(pos.x, pos.y, pos.z, O.w);
            next_d = make_float4(wi.x, wi.y, wi.z, 0.0f);
            next_t = make_float4(T.x, T.y, T.z, 0.0f);
          }
        }
      }
    }
    const uint32_t slot = warp_append(pb.counts + bounce + 1, cont);
    if (cont) {
      out_o[slot] = next_o;
      out_d[slot] = next_d;
      out_t[slot] = next_t;
    }
  }
}

// running mean in sample order: out = mix(out, L_k, 1/k) (pathtracing.wgsl:246-260)
__global__ void __launch_bounds__(256) k_accumulate(PathBatch pb, float4* __restrict__ out, uint32_t n_samples) {
  for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < pb.npix; pix += gridDim.x * blockDim.x) {
    float4 c = out[pix];
    for (uint32_t k = 0; k < n_samples; ++k) {
      const float w = 1.0f / (float)(pb.first_sample + k);
      const float4 L = pb.radiance[(size_t)k * pb.npix + pix];
      c.x = c.x * (1.0f - w) + L.x * w;
      c.y = c.y * (1.0f - w) + L.y * w;
      c.z = c.z * (1.0f - w) + L.z * w;
    }
    out[pix] = make_float4(c.x, c.y, c.z, 1.0f);
  }
}

}  // namespace nbd

// ------------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------------
namespace nb {

static int blocks_for(const void* kernel, int threads, int sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  return per_sm * sms;
}

cudaError_t launch_trace_rays(const nbd::DevScene& s, const float* rays, uint32_t n, bool any, float* hits,
                              uint32_t* inst, uint32_t* fetch, uint32_t* status, int sms, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(fetch, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
  if (any) {
    int g = blocks_for((const void*)nbd::k_trace_rays<true>, 128, sms);
    nbd::k_trace_rays<true><<<g, 128, 0, st>>>(s, (const float4*)rays, n, (float4*)hits, inst, fetch, status);
  } else {
    int g = blocks_for((const void*)nbd::k_trace_rays<false>, 128, sms);
    nbd::k_trace_rays<false><<<g, 128, 0, st>>>(s, (const float4*)rays, n, (float4*)hits, inst, fetch, status);
  }
  return cudaGetLastError();
}

cudaError_t launch_raygen(const PathBatch& pb, const CameraParams& cam, int sms, cudaStream_t st) {
  int g = (int)std::min<uint64_t>((pb.n_paths + 255) / 256, (uint64_t)sms * 16);
  nbd::k_raygen<<<g < 1 ? 1 : g, 256, 0, st>>>(pb, cam);
  return cudaGetLastError();
}

cudaError_t launch_trace_wave(const nbd::DevScene& s, const PathBatch& pb, uint32_t bounce,
                              unsigned long long* ray_total, int sms, cudaStream_t st) {
  static const int grid = blocks_for((const void*)nbd::k_trace_wave, 128, sms);
  nbd::k_trace_wave<<<grid, 128, 0, st>>>(s, pb, bounce, ray_total);
  return cudaGetLastError();
}

cudaError_t launch_shade(const nbd::DevScene& s, const nbd::DevEnv& env, const PathBatch& pb, uint32_t bounce,
                         uint32_t bounces, float cf, int sms, cudaStream_t st) {
  static const int grid = blocks_for((const void*)nbd::k_shade, 256, sms);
  nbd::k_shade<<<grid, 256, 0, st>>>(s, env, pb, bounce, bounces, cf);
  return cudaGetLastError();
}

cudaError_t launch_accumulate(const PathBatch& pb, uint32_t n_samples, float* out, int sms, cudaStream_t st) {
  int g = (int)std::min<uint64_t>((pb.npix + 255) / 256, (uint64_t)sms * 16);
  nbd::k_accumulate<<<g < 1 ? 1 : g, 256, 0, st>>>(pb, (float4*)out, n_samples);
  return cudaGetLastError();
}

}  // namespace nb

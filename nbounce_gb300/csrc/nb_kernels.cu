// CUDA kernels of the nBounce path-tracing pass for sm_103a.
//
// The reference runs one WGSL invocation per pixel that loops over bounces with the whole
// traversal inline (pathtracing.wgsl:161-260).  Here the pass is a wavefront:
//   raygen      one path per (pixel, sample) of a batch: Cranley-Patterson-rotated Sobol
//               jitter and generate_ray (pathtracing.wgsl:27-41, 245-255), queued in 8x8
//               pixel tiles
//   trace       persistent warps take 32 rays at a time with one atomic and walk 8-wide
//               quantised trees (raytracing_sw.wgsl:176-319): BLASes collapsed from the
//               reference's, a TLAS over tight world boxes of the instances (large instances
//               split at their BLAS root).  One 80-byte node load tests eight child boxes; hit
//               children are pushed in distance order so the nearest is visited next, then the
//               node's hit leaf triangles are tested
//   shade       hit attributes (raytracing_sw.wgsl:138-173), env/emission termination, lobe
//               choice, VNDF / cosine sampling, Russian roulette (pathtracing.wgsl:161-241);
//               each block appends its survivors to the next bounce's queue grouped by
//               direction bin (one atomic per block)
//   accumulate  running mean over the batch's samples in sample order (pathtracing.wgsl:258)
// so traversal runs in a lean kernel and the path state lives in HBM.  A wave can hold paths
// of several jobs (render requests): tables of segments, jobs and scenes ride in the kernel
// parameters and each path finds its job through its path id.
//
// The traversal finds the reference's closest hit: quantised BLAS boxes contain the reference
// boxes, TLAS boxes contain each instance's geometry, triangles are tested with the
// reference's Moller-Trumbore arithmetic, and a hit replaces the current one only when
// strictly closer.  Visiting order differs from the
// reference (8-wide nodes, BLAS nodes pruned by the running closest hit where the reference
// restarts each BLAS from NO_HIT, raytracing_sw.wgsl:255), so among triangles at exactly the
// same distance another one may win: the documented near-tie class.

#include <algorithm>
#include <cstdint>

#include "nb_device.cuh"
#include "nb_launch.h"
#include "nb_mlp.cuh"

namespace nbd {

using nb::JobParams;
using nb::kMaxBounceSlots;
using nb::PathBatch;
using nb::Segment;
using nb::ShadowQueue;
using nb::WaveTables;

constexpr int kStackSize = 64;
constexpr uint32_t kIterationCap = 1u << 22;
constexpr uint32_t kInstanceBit = 0x80000000u;

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }
__device__ __forceinline__ uint32_t f2u(float x) { return __float_as_uint(x); }

// Direction reciprocal for box tests only: components below 1e-20 in magnitude are nudged to
// +-1e-20 so that every plane distance stays finite (triangle tests use the true direction).
// The hardware's approximate reciprocal (relative error <= 2^-23, no slow path) instead of a
// correctly rounded division: the box test's per-axis margins cover the extra rounding (see
// trace_step), and the correctly rounded division cost 2.2 ms of the benchmark frame's traversal.
__device__ __forceinline__ float safe_rcp(float d) {
  const float m = 1e-20f;
  const float x = fabsf(d) < m ? copysignf(m, d) : d;
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

struct Hit {
  float t, u, v;
  uint32_t tri, inst;
};

// Traversal state of one ray: the world ray, the current ray (world, or instance-local inside
// a BLAS), the distance of the closest hit so far and the depth of the stack both levels share.
// The stack itself is a separate per-thread array, so that these scalars stay in registers;
// the rest of the hit record (u, v, triangle, instance), written only when a closer hit is
// found, lives in two extra slots at the end of that array (kHitSlot), and the world ray's
// reciprocal direction is recomputed when a BLAS is left - both to keep the state within the
// register budget of 8 resident blocks of 128 threads.
constexpr int kHitSlot = kStackSize;  // stack[kHitSlot] = (u, v), stack[kHitSlot + 1] = (tri, inst)
struct TraceState {
  V3 wo, wd;
  V3 ro, rd, rinv;
  float t_hit;
  int sp, blas_base;
  uint32_t cur_inst, node, iter, status;
  bool in_blas, have_node;
};

__device__ __forceinline__ void trace_begin(TraceState& t, uint2* stack, const DevScene& s, const V3 wo,
                                            const V3 wd) {
  t.t_hit = kNoHit;
  stack[kHitSlot] = make_uint2(0u, 0u);
  stack[kHitSlot + 1] = make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu);
  t.status = 0;
  t.wo = wo;
  t.wd = wd;
  t.ro = wo;
  t.rd = wd;
  t.rinv = V3{safe_rcp(wd.x), safe_rcp(wd.y), safe_rcp(wd.z)};
  t.sp = 0;
  t.blas_base = 0;
  t.in_blas = false;
  t.cur_inst = 0;
  t.node = 0;  // the TLAS root
  // no TLAS, or a ray with a NaN or infinite component: nothing to hit (every slab and
  // triangle comparison of the reference fails on NaN; the box test below relies on it)
  const float fin = fabsf(wo.x) + fabsf(wo.y) + fabsf(wo.z) + fabsf(wd.x) + fabsf(wd.y) + fabsf(wd.z);
  t.have_node = s.has_tlas != 0u && fin <= 3.4028235e38f;
  t.iter = 0;
}

// Where trace_step reads the world ray and its box-test reciprocal when it enters or leaves an
// instance.  A per-warp array in shared memory, component-major so that the 32 lanes' loads hit
// distinct banks, kWorldFloats floats: origin, direction, reciprocal direction x 32 lanes.
//   WorldShared  all three in shared memory: keeps six registers free in the lane-refill
//                kernels, whose register budget is tightest;
//   WorldMixed   origin and direction in registers, the reciprocal in shared memory (the
//                camera-ray kernel, which enters and leaves instances at most steps);
//   WorldRegs    origin and direction in registers, the reciprocal recomputed (caller rays
//                without refill).
// Keeping the reciprocal instead of recomputing it when a BLAS is left measured 2.3 ms faster
// traversal on the benchmark frame.
constexpr int kWorldFloats = 9 * 32;
constexpr int kTraceWarps = 4;  // every traversal kernel runs blocks of 128 threads
constexpr int kTraceThreads = 32 * kTraceWarps;
struct WorldRegs {
  const TraceState& t;
  __device__ __forceinline__ V3 o() const { return t.wo; }
  __device__ __forceinline__ V3 d() const { return t.wd; }
  __device__ __forceinline__ V3 inv() const { return V3{safe_rcp(t.wd.x), safe_rcp(t.wd.y), safe_rcp(t.wd.z)}; }
};
// a warp's reciprocal directions: kInvFloats floats, component-major
constexpr int kInvFloats = 3 * 32;
__device__ __forceinline__ V3 world_inv(const float* w) {
  const uint32_t l = threadIdx.x & 31u;
  return V3{w[l], w[32 + l], w[64 + l]};
}
__device__ __forceinline__ void set_world_inv(float* w, V3 r) {
  const uint32_t l = threadIdx.x & 31u;
  w[l] = r.x; w[32 + l] = r.y; w[64 + l] = r.z;
}
struct WorldMixed {
  const TraceState& t;
  const float* w;  // kInvFloats
  __device__ __forceinline__ V3 o() const { return t.wo; }
  __device__ __forceinline__ V3 d() const { return t.wd; }
  __device__ __forceinline__ V3 inv() const { return world_inv(w); }
};
struct WorldShared {
  float* w;
  __device__ __forceinline__ V3 o() const {
    const uint32_t l = threadIdx.x & 31u;
    return V3{w[l], w[32 + l], w[64 + l]};
  }
  __device__ __forceinline__ V3 d() const {
    const uint32_t l = threadIdx.x & 31u;
    return V3{w[96 + l], w[128 + l], w[160 + l]};
  }
  __device__ __forceinline__ V3 inv() const { return world_inv(w + 192); }
  __device__ __forceinline__ void set(V3 o, V3 d) const {
    const uint32_t l = threadIdx.x & 31u;
    w[l] = o.x; w[32 + l] = o.y; w[64 + l] = o.z;
    w[96 + l] = d.x; w[128 + l] = d.y; w[160 + l] = d.z;
  }
  __device__ __forceinline__ void set_inv(V3 r) const { set_world_inv(w + 192, r); }
};

// Work counters of the instrumented traversal (kCount instantiations only): what the device
// layout fetches per ray - 80-byte wide nodes of the TLAS and the BLASes, 48-byte triangle
// records, 64-byte instance records - and the 8-byte stack entries pushed (each later popped);
// and how the lanes of a warp share the node steps: warp steps (lanes that test a node
// together count one step, recorded by the lowest of them) with their lanes, and of those the
// steps in which some lane tests leaf triangles, with the lanes that do and the largest
// triangle count among them (the warp's iterations of the leaf loop).
struct TraceCount {
  uint32_t tlas_nodes = 0, blas_nodes = 0, tris = 0, insts = 0, pushes = 0;
  uint32_t warp_steps = 0, lane_steps = 0, leaf_steps = 0, leaf_lanes = 0, leaf_trips = 0;
};
__device__ __forceinline__ bool lowest_active(uint32_t mask) {
  return (threadIdx.x & 31u) == (uint32_t)(__ffs(mask) - 1);
}

// One traversal step: pop the next entry when no node is pending, then test one 8-wide node
// and its leaf triangles.  Returns false once the ray is finished (stack empty, an any-hit
// found, or the iteration cap reached).  wr gives the world ray (WorldRegs, WorldMixed or
// WorldShared).
template <bool kAny, bool kCount, class World>
__device__ __forceinline__ bool trace_step(TraceState& t, uint2* stack, const DevScene& s, TraceCount* cnt,
                                           const World& wr) {
  if (t.iter > kIterationCap) {
    t.status |= kStatusIterationCap;
    return false;
  }
  ++t.iter;
  V3 &ro = t.ro, &rd = t.rd, &rinv = t.rinv;
  float& h_t = t.t_hit;
  int &sp = t.sp, &blas_base = t.blas_base;
  bool &in_blas = t.in_blas, &have_node = t.have_node;
  uint32_t &cur_inst = t.cur_inst, &node = t.node, &status = t.status;
  if (!have_node) {
    bool done = false;
    for (;;) {
      if (in_blas && sp == blas_base) {  // BLAS finished: back to the world ray
        in_blas = false;
        const V3 wd = wr.d();
        ro = wr.o(); rd = wd;
        rinv = wr.inv();
      }
      if (sp == 0) {
        done = true;
        break;
      }
      --sp;
      const uint2 e = stack[sp];
      if (__uint_as_float(e.y) >= h_t) continue;  // raytracing_sw.wgsl:197,271
      if (!in_blas && (e.x & kInstanceBit)) {
        // enter an instance: transform the world ray (raytracing_sw.wgsl:202-206)
        if (kCount) ++cnt->insts;
        const float4* it = s.inst_trace + 4 * (size_t)(e.x & ~kInstanceBit);
        const float4 r0 = ld4(it), r1 = ld4(it + 1), r2 = ld4(it + 2), r3 = ld4(it + 3);
        const V3 wo = wr.o(), wd = wr.d();
        ro = V3{r0.x * wo.x + r0.y * wo.y + r0.z * wo.z + r0.w * 1.0f,
                r1.x * wo.x + r1.y * wo.y + r1.z * wo.z + r1.w * 1.0f,
                r2.x * wo.x + r2.y * wo.y + r2.z * wo.z + r2.w * 1.0f};
        rd = V3{r0.x * wd.x + r0.y * wd.y + r0.z * wd.z, r1.x * wd.x + r1.y * wd.y + r1.z * wd.z,
                r2.x * wd.x + r2.y * wd.y + r2.z * wd.z};
        rinv = V3{safe_rcp(rd.x), safe_rcp(rd.y), safe_rcp(rd.z)};
        node = f2u(r3.x);
        cur_inst = f2u(r3.y);
        in_blas = true;
        blas_base = sp;
      } else {
        node = e.x;
      }
      break;
    }
    if (done) return false;
  }
  have_node = false;

  // ---- one 8-wide node: quantised slab tests of all children ----
  if (kCount) {
    ++(in_blas ? cnt->blas_nodes : cnt->tlas_nodes);
    const uint32_t together = __activemask();
    if (lowest_active(together)) {
      ++cnt->warp_steps;
      cnt->lane_steps += (uint32_t)__popc(together);
    }
  }
  const float4* np = (in_blas ? s.blas_wide : s.tlas_wide) + 5 * (size_t)node;
  const float4 q0 = ld4(np), q1 = ld4(np + 1), q2 = ld4(np + 2), q3 = ld4(np + 3), q4 = ld4(np + 4);
  const uint32_t eb = f2u(q0.w);
  const float ax = __uint_as_float((eb & 0xFFu) << 23) * rinv.x;
  const float ay = __uint_as_float(((eb >> 8) & 0xFFu) << 23) * rinv.y;
  const float az = __uint_as_float(((eb >> 16) & 0xFFu) << 23) * rinv.z;
  const float bx = (q0.x - ro.x) * rinv.x, by = (q0.y - ro.y) * rinv.y, bz = (q0.z - ro.z) * rinv.z;
  // A plane byte q is read as the float F = 2^15 + q (one byte permute: bytes 0, q, 0, 0x47)
  // and its distance taken as fma(F, a, b - 2^15 a), one rounding more than fma(q, a, b): the
  // folded constant differs from b - 2^15 a by at most 2^-24 (|b| + 2^15 |a|), so each plane's
  // distance lies within e = 2^-24 (3 |b| + (2^15 + 510) |a|) of fma(q, a, b).  Near-plane
  // constants are lowered and far-plane constants raised by d = |a| / 128 + |b| / 2^19 per
  // axis.  For every plane t = b + q a of the node (|t| <= |b| + 255 |a|) the margin covers
  // the fold (e <= 1.8e-7 |b| + 0.002 |a|), the approximate reciprocal (<= 2^-22 |t|) and the
  // rounding of the plane evaluation against the exact reference box (4e-7 |t|): together
  // at most 8.2e-7 |b| + 0.0022 |a| <= d, so a box never rejects a ray the reference box
  // accepts.
  const float dx = fmaf(fabsf(ax), 0.0078125f, fabsf(bx) * 1.9073486328125e-6f);
  const float dy = fmaf(fabsf(ay), 0.0078125f, fabsf(by) * 1.9073486328125e-6f);
  const float dz = fmaf(fabsf(az), 0.0078125f, fabsf(bz) * 1.9073486328125e-6f);
  const float cx = fmaf(-32768.0f, ax, bx), cy = fmaf(-32768.0f, ay, by), cz = fmaf(-32768.0f, az, bz);
  const float cnx = cx - dx, cfx = cx + dx, cny = cy - dy, cfy = cy + dy, cnz = cz - dz, cfz = cz + dz;
  const uint32_t child_base = f2u(q1.x), prim_base = f2u(q1.y);
  const uint32_t m0 = f2u(q1.z), m1 = f2u(q1.w);
  // near/far planes per axis by the sign of the direction: the near plane of a child is its
  // low plane where rinv >= 0 (t grows with the quantised coordinate), else its high plane
  const bool pxs = rinv.x >= 0.0f, pys = rinv.y >= 0.0f, pzs = rinv.z >= 0.0f;
  const uint32_t nx0 = pxs ? f2u(q2.x) : f2u(q3.z), nx1 = pxs ? f2u(q2.y) : f2u(q3.w);
  const uint32_t fx0 = pxs ? f2u(q3.z) : f2u(q2.x), fx1 = pxs ? f2u(q3.w) : f2u(q2.y);
  const uint32_t ny0 = pys ? f2u(q2.z) : f2u(q4.x), ny1 = pys ? f2u(q2.w) : f2u(q4.y);
  const uint32_t fy0 = pys ? f2u(q4.x) : f2u(q2.z), fy1 = pys ? f2u(q4.y) : f2u(q2.w);
  const uint32_t nz0 = pzs ? f2u(q3.x) : f2u(q4.z), nz1 = pzs ? f2u(q3.y) : f2u(q4.w);
  const uint32_t fz0 = pzs ? f2u(q4.z) : f2u(q3.x), fz1 = pzs ? f2u(q4.w) : f2u(q3.y);
  // a child is hit when max(tn, 0) <= min(tf, the largest float below the closest hit)
  const float t_below = __uint_as_float(f2u(h_t) - 1u);  // h_t > 0
  uint32_t key[8];
  uint32_t leaf_mask = 0, n_push = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    // byte k of the plane words as the float 2^15 + q: bits 0x4700qq00
    const uint32_t sel = 0x7404u + ((uint32_t)(k & 3) << 4);
    const uint32_t meta = __byte_perm(k < 4 ? m0 : m1, 0u, 0x4440u + (uint32_t)(k & 3));
    const float nx = __uint_as_float(__byte_perm(k < 4 ? nx0 : nx1, 0x47000000u, sel));
    const float fx = __uint_as_float(__byte_perm(k < 4 ? fx0 : fx1, 0x47000000u, sel));
    const float ny = __uint_as_float(__byte_perm(k < 4 ? ny0 : ny1, 0x47000000u, sel));
    const float fy = __uint_as_float(__byte_perm(k < 4 ? fy0 : fy1, 0x47000000u, sel));
    const float nz = __uint_as_float(__byte_perm(k < 4 ? nz0 : nz1, 0x47000000u, sel));
    const float fz = __uint_as_float(__byte_perm(k < 4 ? fz0 : fz1, 0x47000000u, sel));
    const float tn = fmaxf(fmaxf(fmaf(nx, ax, cnx), fmaf(ny, ay, cny)), fmaf(nz, az, cnz));
    const float tf = fminf(fminf(fmaf(fx, ax, cfx), fmaf(fy, ay, cfy)), fmaf(fz, az, cfz));
    const float lo = fmaxf(tn, 0.0f);
    const bool hit = meta != 0u && lo <= fminf(tf, t_below);
    key[k] = 0xFFFFFFFFu;
    if (hit) {
      if (in_blas && !(meta & 0x80u)) {
        leaf_mask |= 1u << k;
      } else {
        key[k] = (f2u(lo) & ~7u) | (uint32_t)k;
        ++n_push;
      }
    }
  }

  // The hit children are ordered and pushed before the node's leaf triangles are tested:
  // the keys' registers are free again during the triangle loads (measured 1.6% faster than
  // testing leaves first).  A leaf hit closer than the child visited next drops that child.
  float next_d = 0.0f;
  // ---- order hit children near to far (19-comparator network) ----
#define NB_CX(i, j)                                  \
{                                                  \
  const uint32_t lo_ = min(key[i], key[j]);        \
  key[j] = max(key[i], key[j]);                    \
  key[i] = lo_;                                    \
}
  // push far to near; the nearest inner child is visited next without a push
  auto take = [&](uint32_t kk, bool nearest) {
    const float d = __uint_as_float(kk & ~7u);
    const uint32_t slot = kk & 7u;
    const uint32_t meta = ((slot < 4 ? m0 : m1) >> (8 * (slot & 3))) & 0xFFu;
    const uint32_t ref = (meta & 0x80u) ? child_base + (meta & 7u) : (kInstanceBit | (prim_base + (meta & 31u)));
    if (nearest && (meta & 0x80u)) {
      node = ref;
      have_node = true;
      next_d = d;
    } else if (sp < kStackSize) {
      stack[sp] = make_uint2(ref, kk & ~7u);
      ++sp;
      if (kCount) ++cnt->pushes;
    } else {
      status |= kStatusStackOverflow;
    }
  };
  if (n_push == 1) {  // the single hit child: no sort, no loop over the empty keys
    uint32_t m = key[0];
#pragma unroll
    for (int k = 1; k < 8; ++k) m = min(m, key[k]);
    take(m, true);
  } else if (n_push > 1) {
    NB_CX(0, 2) NB_CX(1, 3) NB_CX(4, 6) NB_CX(5, 7)
    NB_CX(0, 4) NB_CX(1, 5) NB_CX(2, 6) NB_CX(3, 7)
    NB_CX(0, 1) NB_CX(2, 3) NB_CX(4, 5) NB_CX(6, 7)
    NB_CX(2, 4) NB_CX(3, 5)
    NB_CX(1, 4) NB_CX(3, 6)
    NB_CX(1, 2) NB_CX(3, 4) NB_CX(5, 6)
#pragma unroll
    for (int k = 7; k >= 0; --k) {
      if (key[k] != 0xFFFFFFFFu) take(key[k], k == 0);
    }
  }
#undef NB_CX
  if (kCount) {
    const uint32_t together = __activemask();
    uint32_t n_tris = 0;
    for (uint32_t lm = leaf_mask; lm; lm &= lm - 1) {
      const int k = __ffs(lm) - 1;
      n_tris += (((k < 4 ? m0 : m1) >> (8 * (k & 3))) & 0xFFu) >> 5;
    }
    const uint32_t with_leaves = __ballot_sync(together, leaf_mask != 0u);
    const uint32_t most = __reduce_max_sync(together, n_tris);
    if (with_leaves && lowest_active(together)) {
      ++cnt->leaf_steps;
      cnt->leaf_lanes += (uint32_t)__popc(with_leaves);
      cnt->leaf_trips += most;
    }
  }
  // ---- BLAS leaves: Moller-Trumbore (raytracing_sw.wgsl:51-78, 274-286) ----
  while (leaf_mask) {
    const int k = __ffs(leaf_mask) - 1;
    leaf_mask &= leaf_mask - 1;
    const uint32_t meta = ((k < 4 ? m0 : m1) >> (8 * (k & 3))) & 0xFFu;
    const uint32_t first = prim_base + (meta & 31u), n = meta >> 5;
    for (uint32_t j = 0; j < n; ++j) {
      if (kCount) ++cnt->tris;
      const float4* tp = s.tris + 3 * (size_t)(first + j);
      const float4 a = ld4(tp), b = ld4(tp + 1), c = ld4(tp + 2);
      const V3 e1 = xyz(b), e2 = xyz(c);
      const V3 hv = cross(rd, e2);
      const float det = dot(e1, hv);
      if (det < kEps) continue;
      // det >= kEps here; 1 / det correctly rounded, as the reference arithmetic divides
      const float inv_det = det < kRcpNewtonMax ? rcp_newton(det) : 1.0f / det;
      const V3 sv = ro - xyz(a);
      const float u = inv_det * dot(sv, hv);
      if (u < 0.0f || u > 1.0f) continue;
      const V3 q = cross(sv, e1);
      const float v = inv_det * dot(rd, q);
      if (v < 0.0f || u + v > 1.0f) continue;
      const float t = inv_det * dot(e2, q);
      if (t < kBias) continue;
      if (t < h_t) {
        h_t = t;
        stack[kHitSlot] = make_uint2(f2u(u), f2u(v));
        stack[kHitSlot + 1] = make_uint2(f2u(b.w), cur_inst);
        if (kAny) return false;
      }
    }
  }

  if (have_node && next_d >= h_t) have_node = false;  // a leaf above is closer than the next node
  return true;
}

// Closest (or any) hit of one world-space ray.  Returns the status bits it raised.
template <bool kAny, bool kCount = false>
__device__ __forceinline__ uint32_t trace_ray(const DevScene& s, const V3 wo, const V3 wd, Hit& h,
                                              TraceCount* cnt = nullptr) {
  TraceState t;
  uint2 stack[kStackSize + 2];
  trace_begin(t, stack, s, wo, wd);
  while (trace_step<kAny, kCount>(t, stack, s, cnt, WorldRegs{t})) {
  }
  const uint2 uv = stack[kHitSlot], ti = stack[kHitSlot + 1];
  h.t = t.t_hit;
  h.u = __uint_as_float(uv.x);
  h.v = __uint_as_float(uv.y);
  h.tri = ti.x;
  h.inst = ti.y;
  return t.status;
}

// Traces rays 0 .. n-1 of a queue with one warp, refilling lanes: a lane whose ray finished
// takes a new one once kRefillIdle lanes of the warp are idle (a whole idle warp always takes
// 32), all of them with one atomic on *fetch.  load(r, o, d, sidx) reads ray r and its scene
// index; scene(sidx) gives that scene; finish(r, t_hit, uv, tri_inst) consumes ray r's hit
// record (t = kNoHit on a miss).  world is this warp's kWorldFloats floats of shared memory,
// where the lanes' world rays are kept (WorldShared).  Every lane of the warp must call it.
// Returns the status bits its rays raised.  Used where the rays of a warp are incoherent
// (secondary and shadow rays, caller rays): their traversal lengths differ widely, and without
// refill most lanes would idle while the longest ray of each 32 finishes.  Refill changes only
// which lane traces a ray, not its result.
constexpr uint32_t kRefillIdle = 6;
template <bool kAny, bool kCount, class Load, class SceneOf, class Finish>
__device__ __forceinline__ uint32_t trace_refill(uint32_t* fetch, uint32_t n, Load load, SceneOf scene, Finish finish,
                                                 TraceCount* cnt, float* world) {
  const WorldShared wr{world};
  const uint32_t lane = threadIdx.x & 31u;
  TraceState t;
  uint2 stack[kStackSize + 2];
  constexpr uint32_t kNone = 0xFFFFFFFFu;
  uint32_t my = kNone, sidx = 0, st = 0;  // this lane's ray (queue index) and its scene
  bool exhausted = false;                 // warp-uniform: the queue has no rays left to take
  uint32_t idle = 0xFFFFFFFFu;            // lanes without a ray
  while (true) {
    if (!exhausted && (uint32_t)__popc(idle) >= (idle == 0xFFFFFFFFu ? 1u : kRefillIdle)) {
      const uint32_t want = (uint32_t)__popc(idle);
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(fetch, want);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base + want >= n) exhausted = true;
      if (my == kNone) {
        const uint32_t r = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
        if (r < n) {
          my = r;
          V3 o, d;
          load(r, o, d, sidx);
          trace_begin(t, stack, scene(sidx), o, d);
          wr.set(o, d);
          wr.set_inv(t.rinv);
        }
      }
    }
    if (my != kNone && !trace_step<kAny, kCount>(t, stack, scene(sidx), cnt, wr)) {
      finish(my, t.t_hit, stack[kHitSlot], stack[kHitSlot + 1]);
      st |= t.status;
      my = kNone;
    }
    idle = __ballot_sync(0xFFFFFFFFu, my == kNone);
    if (exhausted && idle == 0xFFFFFFFFu) break;
  }
  return st;
}

// ------------------------------------------------------------------------------------------
// traversal-only query (nb_trace_rays)
// ------------------------------------------------------------------------------------------
// kRefill: lanes refill as they finish (trace_refill), for rays whose neighbours in the array
// are unrelated; else each warp traces 32 consecutive rays to the end.  Blocks per SM: 9 with
// refill (56 registers; 1M-triangle soup, incoherent rays: 28.0 -> 26.8 ms against 8 blocks),
// 8 for any hit without refill (64 registers), 7 for closest hit without refill (72).
template <bool kAny, bool kRefill>
__global__ void __launch_bounds__(kTraceThreads, kRefill ? 9 : kAny ? 8 : 7)
    k_trace_rays(DevScene s, const float4* __restrict__ rays, uint32_t n, float4* __restrict__ hits,
                 uint32_t* __restrict__ inst, uint32_t* __restrict__ fetch, uint32_t* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  uint32_t st = 0;
  if (kRefill) {
    __shared__ float world[kTraceWarps][kWorldFloats];
    st = trace_refill<kAny, false>(
        fetch, n,
        [&](uint32_t r, V3& o, V3& d, uint32_t& sidx) {
          o = xyz(__ldg(rays + 2 * (size_t)r));
          d = xyz(__ldg(rays + 2 * (size_t)r + 1));
          sidx = 0;
        },
        [&](uint32_t) -> const DevScene& { return s; },
        [&](uint32_t r, float t_hit, uint2 uv, uint2 ti) {
          hits[r] = make_float4(t_hit, __uint_as_float(uv.x), __uint_as_float(uv.y), __uint_as_float(ti.x));
          if (inst) inst[r] = ti.y;
        },
        nullptr, world[threadIdx.x >> 5]);
  } else {
    while (true) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(fetch, 32u);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base >= n) break;
      const uint32_t i = base + lane;
      if (i < n) {
        const float4 o = __ldg(rays + 2 * (size_t)i), d = __ldg(rays + 2 * (size_t)i + 1);
        Hit h;
        st |= trace_ray<kAny>(s, xyz(o), xyz(d), h);
        hits[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.tri));
        if (inst) inst[i] = h.inst;
      }
    }
  }
  if (st) atomicOr(status, st);
}


// ------------------------------------------------------------------------------------------
// wavefront path tracer
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float4 sobol_read(const float4* table, uint32_t n_entries, uint32_t idx) {
  return idx < n_entries ? __ldg(table + idx) : make_float4(0.f, 0.f, 0.f, 0.f);  // robust buffer access
}

// generate_ray (pathtracing.wgsl:27-41); m is clip_to_world, column-major
__device__ __forceinline__ void generate_ray(uint32_t x, uint32_t y, uint32_t W, uint32_t H, float rx, float ry,
                                             const float* m, V3* o, V3* d) {
  float uvx = 2.0f * ((float)x + rx) / (float)W - 1.0f;
  float uvy = 2.0f * ((float)y + ry) / (float)H - 1.0f;
  V3 pos = V3{m[12], m[13], m[14]} / m[15];
  float cx = -uvx, cy = -uvy, cz = -1.0f, cw = 1.0f;
  float wd[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) wd[r] = m[r] * cx + m[4 + r] * cy + m[8 + r] * cz + m[12 + r] * cw;
  *o = pos;
  *d = pos - V3{wd[0], wd[1], wd[2]} / wd[3];
}

// index of the last segment whose begin (path or accumulate index) is <= p
template <bool kByPixel>
__device__ __forceinline__ uint32_t find_segment(const Segment* segs, uint32_t n, uint32_t p) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    const uint32_t b = kByPixel ? segs[mid].pix_begin : segs[mid].path_begin;
    if (b <= p) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void stage_segments(Segment* dst, const WaveTables& wt) {
  for (uint32_t i = threadIdx.x; i < wt.n_segs; i += blockDim.x) dst[i] = wt.segs[i];
  __syncthreads();
}

// Pixel of the i-th queue entry of one sample plane (a bijection of [0, W*H)): the image's
// 8x8 tiles in row order, Z-order inside a tile; the columns right of the last whole tile,
// then the rows below it, in row order.  Compact warps of primary rays measured 14% faster
// traversal than rows of 32 pixels.
__device__ __forceinline__ void tile_pixel(uint32_t i, uint32_t W, uint32_t H, uint32_t* x, uint32_t* y) {
  const uint32_t Wt = W & ~7u, Ht = H & ~7u;
  if (i < Wt * Ht) {
    const uint32_t tile = i >> 6, z = i & 63u, tiles_x = Wt >> 3;
    *x = ((tile % tiles_x) << 3) | (z & 1u) | ((z >> 1) & 2u) | ((z >> 2) & 4u);
    *y = ((tile / tiles_x) << 3) | ((z >> 1) & 1u) | ((z >> 2) & 2u) | ((z >> 3) & 4u);
    return;
  }
  i -= Wt * Ht;
  const uint32_t rw = W - Wt;
  if (i < rw * Ht) {
    *x = Wt + i % rw;
    *y = i / rw;
  } else {
    i -= rw * Ht;
    *x = i % W;
    *y = Ht + i / W;
  }
}

// Samples of one pixel queued together: a warp of camera rays is 32 samples of one pixel,
// nearly the same ray 32 times over, instead of one sample of an 8x4 pixel patch (the whole
// frame is one wave, so all samples are present): 12-14% faster traversal.
constexpr uint32_t kSampleGroup = 64;

// Camera ray of queue entry q (pathtracing.wgsl:245-255): origin with the path id in .w,
// direction with the scene index in .w.  Path ids stay row-major per sample (pixel = id %
// (W*H)); the queue lists them by sample group and tile order (tile_pixel), which every later
// kernel follows through the path id each ray carries.  segs: the wave's segments.
__device__ __forceinline__ void camera_ray(const Segment* segs, const WaveTables& wt, const PathBatch& pb, uint32_t q,
                                           float4& o4, float4& d4) {
  const Segment sg = segs[find_segment<false>(segs, wt.n_segs, q)];
  const JobParams& jp = wt.jobs[sg.job];
  const uint32_t local = q - sg.path_begin;
  // the segment's samples in groups of kSampleGroup: the queue runs over one group's samples
  // of a pixel, then the next pixel in tile order (a last, smaller group the same way)
  const uint32_t span = kSampleGroup * jp.npix, full = sg.n_samples / kSampleGroup;
  uint32_t plane, order;
  if (local < full * span) {
    const uint32_t grp = local / span, j = local - grp * span;
    plane = grp * kSampleGroup + j % kSampleGroup;
    order = j / kSampleGroup;
  } else {
    const uint32_t g = sg.n_samples - full * kSampleGroup, j = local - full * span;
    plane = full * kSampleGroup + j % g;
    order = j / g;
  }
  uint32_t x, y;
  tile_pixel(order, jp.width, jp.height, &x, &y);
  const uint32_t p = sg.path_begin + plane * jp.npix + y * jp.width + x;
  const uint32_t sample = sg.first_sample + plane;
  const float4 shift = hash4f(x, y);
  const float4 sb = sobol_read(pb.sobol, pb.sobol_entries, sample * kLdsStride);
  const float jx = fract(sb.x + shift.x), jy = fract(sb.y + shift.y);
  V3 o, d;
  generate_ray(x, y, jp.width, jp.height, jx, jy, jp.c2w, &o, &d);
  o4 = make_float4(o.x, o.y, o.z, __uint_as_float(p));
  d4 = make_float4(d.x, d.y, d.z, __uint_as_float(jp.scene));
}

// Start of a wave: the bounce counters and work cursors, and (kWaveZeroRadiance: waves whose
// shading adds to radiance) every path's radiance zeroed.  The camera rays themselves are made
// by the bounce-0 traversal, which writes them to the queue for shading (camera_ray).  A
// segment's queue positions and path ids cover the same range, so zeroing by queue position
// clears every path's radiance with coalesced stores.
__global__ void __launch_bounds__(256) k_raygen(PathBatch pb, const WaveTables wt) {
  const uint32_t n = wt.n_paths;
  if (blockIdx.x == 0 && threadIdx.x < kMaxBounceSlots) {
    pb.counts[threadIdx.x] = threadIdx.x == 0 ? n : 0u;
    pb.fetch[threadIdx.x] = 0u;
  }
  if (wt.flags & nb::kWaveZeroRadiance) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
      pb.radiance[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}

// kSingle: every ray of the wave uses wt.scenes[0]; else the scene index carried in q_d.w.
// Bounce 0 (camera rays): persistent warps take 32 consecutive queue entries per atomic - 32
// samples of one pixel - make each lane's camera ray (camera_ray), write it to the queue for
// shading and trace the 32 together, so the lanes walk largely the same nodes (shared cache
// lines, agreeing branches).  The world ray stays in registers, its box-test reciprocal in
// shared memory (WorldMixed).
// kCount: the instrumented variant, which also adds the TraceCount totals of the launch to
// counters[kTraceCounterSlots * bounce + ...] (run only when a caller asks for the counters).
//
// kRefill (bounces >= 1): a lane whose ray finished does not wait for the rest of its warp's
// 32 rays; once kRefillIdle lanes of the warp are idle, the warp takes that many new rays with
// one atomic and those lanes start on them (trace_refill, world rays in shared memory).
// Secondary rays of a warp come from different pixels and surfaces and their traversal lengths
// differ widely, so without refill most lanes idle while the longest ray finishes (11 of 32
// lanes active per instruction on bounce 1).  Camera rays keep whole-warp chunks: a warp's 32
// samples of one pixel finish together, and refilling them measured 9% slower traversal.
// Refill changes only which lane traces a ray, not its result.  The refill instantiation runs
// 9 blocks of 128 per SM at 56 registers (8 bytes spilled); per benchmark frame 8 blocks at 64
// registers took 1.2 ms longer and 10 at 48 (100 bytes spilled) 4.7 ms longer: secondary rays
// wait on dependent loads, and more warps hide them.
template <bool kSingle, bool kCount, bool kRefill>
__global__ void __launch_bounds__(kTraceThreads, kRefill ? 9 : 7) k_trace_wave(PathBatch pb, const WaveTables wt,
                                                                     uint32_t bounce,
                                                       unsigned long long* __restrict__ ray_total,
                                                       unsigned long long* __restrict__ counters) {
  __shared__ DevScene scenes[kSingle ? 1 : nb::kMaxWaveScenes];
  if (!kSingle) {
    for (uint32_t i = threadIdx.x; i < wt.n_scenes; i += blockDim.x) scenes[i] = wt.scenes[i];
    __syncthreads();
  }
  const uint32_t n = pb.counts[bounce];
  const float4* __restrict__ qo = (bounce & 1) ? pb.q_o[1] : pb.q_o[0];
  const float4* __restrict__ qd = (bounce & 1) ? pb.q_d[1] : pb.q_d[0];
  const int lane = threadIdx.x & 31;
  uint32_t st = 0;
  TraceCount cnt;
  if (!kRefill) {  // bounce 0: camera rays, made here and written to the queue for shading
    __shared__ Segment segs[nb::kMaxWaveSegments];
    __shared__ float inv_c[kTraceWarps][kInvFloats];
    stage_segments(segs, wt);
    while (true) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(pb.fetch + bounce, 32u);
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base >= n) break;
      const uint32_t i = base + lane;
      if (i < n) {
        float4 o, d;
        camera_ray(segs, wt, pb, i, o, d);
        pb.q_o[0][i] = o;
        pb.q_d[0][i] = d;
        const DevScene& sc0 = kSingle ? wt.scenes[0] : scenes[__float_as_uint(d.w)];
        TraceState t;
        uint2 stack[kStackSize + 2];
        trace_begin(t, stack, sc0, xyz(o), xyz(d));
        set_world_inv(inv_c[threadIdx.x >> 5], t.rinv);
        const WorldMixed wm{t, inv_c[threadIdx.x >> 5]};
        while (trace_step<false, kCount>(t, stack, sc0, &cnt, wm)) {
        }
        st |= t.status;
        const uint2 uv = stack[kHitSlot], ti = stack[kHitSlot + 1];
        pb.hits[i] = make_float4(t.t_hit, __uint_as_float(uv.x), __uint_as_float(uv.y), __uint_as_float(ti.x));
        pb.hit_inst[i] = ti.y;
      }
    }
  } else {
    __shared__ float world[kTraceWarps][kWorldFloats];
    const DevScene* sc = kSingle ? wt.scenes : scenes;
    st = trace_refill<false, kCount>(
        pb.fetch + bounce, n,
        [&](uint32_t r, V3& o, V3& d, uint32_t& sidx) {
          const float4 o4 = qo[r], d4 = qd[r];
          o = xyz(o4);
          d = xyz(d4);
          sidx = kSingle ? 0u : __float_as_uint(d4.w);
        },
        [&](uint32_t sidx) -> const DevScene& { return sc[sidx]; },
        [&](uint32_t r, float t_hit, uint2 uv, uint2 ti) {
          pb.hits[r] = make_float4(t_hit, __uint_as_float(uv.x), __uint_as_float(uv.y), __uint_as_float(ti.x));
          pb.hit_inst[r] = ti.y;
        },
        &cnt, world[threadIdx.x >> 5]);
  }
  if (st) atomicOr(pb.status, st);
  if (kCount) {  // counters[kTraceCounterSlots * bounce + 0..10]: see nb_pathtracer_trace_counters
    const uint32_t c[10] = {cnt.tlas_nodes, cnt.blas_nodes, cnt.tris, cnt.insts, cnt.pushes,
                            cnt.warp_steps, cnt.lane_steps, cnt.leaf_steps, cnt.leaf_lanes, cnt.leaf_trips};
    unsigned long long* slot = counters + nb::kTraceCounterSlots * bounce;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      unsigned long long v = c[k];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
      if (lane == 0 && v) atomicAdd(slot + (k < 5 ? k : k + 1), v);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(slot + 5, (unsigned long long)n);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(ray_total, (unsigned long long)n);
}

// Cube-map face of a direction and its coordinates s, t in [-1, 1] on that face: the standard
// cube-map table (Vulkan / D3D, which wgpu's cube textures follow) with faces 0..5 = +X, -X,
// +Y, -Y, +Z, -Z; the largest magnitude picks the face, ties going to X, then Y.
__device__ __forceinline__ uint32_t cube_face(V3 d, float* s, float* t) {
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  float sc, tc, ma;
  uint32_t f;
  if (ax >= ay && ax >= az) {
    f = d.x >= 0.0f ? 0u : 1u;
    ma = ax;
    sc = d.x >= 0.0f ? -d.z : d.z;
    tc = -d.y;
  } else if (ay >= az) {
    f = d.y >= 0.0f ? 2u : 3u;
    ma = ay;
    sc = d.x;
    tc = d.y >= 0.0f ? d.z : -d.z;
  } else {
    f = d.z >= 0.0f ? 4u : 5u;
    ma = az;
    sc = d.z >= 0.0f ? d.x : -d.x;
    tc = -d.y;
  }
  *s = sc / ma;
  *t = tc / ma;
  return f;
}

// Environment radiance seen along dir (pathtracing.wgsl:168).
//  equirect (the oracle's definition): u = atan2(d.x, -d.z)/(2 pi) + 0.5, v = acos(d.y)/pi of the
//    normalised direction, bilinear with wrap in u and clamp in v;
//  cube (the reference's texture_cube at mip 0 with a linear clamp-to-edge sampler,
//    texture.rs:89-144): face and (s, t) by cube_face, texel coordinates ((s + 1) / 2) N - 1/2,
//    bilinear inside the face with clamp at its edges (GPUs blend across face seams within half
//    a texel of an edge; this definition does not);
// NaN (and zero) directions see black.
__device__ V3 env_lookup(const DevEnv& env, V3 dir) {
  if (env.kind == kEnvConstant) return V3{env.r, env.g, env.b};
  if (env.kind == kEnvCube) {
    float s, t;
    const uint32_t f = cube_face(dir, &s, &t);
    const int N = (int)env.width;
    const float fx = (s + 1.0f) * 0.5f * (float)N - 0.5f, fy = (t + 1.0f) * 0.5f * (float)N - 0.5f;
    if (fx != fx || fy != fy) return V3{0.0f, 0.0f, 0.0f};
    const float x0 = floorf(fx), y0 = floorf(fy);
    const float tx = fx - x0, ty = fy - y0;
    const int xi = (int)x0, yi = (int)y0;
    const int xa = min(max(xi, 0), N - 1), xb = min(max(xi + 1, 0), N - 1);
    const int ya = (int)f * N + min(max(yi, 0), N - 1), yb = (int)f * N + min(max(yi + 1, 0), N - 1);
    const float4 t00 = __ldg(env.texels + (size_t)ya * N + xa), t10 = __ldg(env.texels + (size_t)ya * N + xb);
    const float4 t01 = __ldg(env.texels + (size_t)yb * N + xa), t11 = __ldg(env.texels + (size_t)yb * N + xb);
    return V3{(t00.x * (1.0f - tx) + t10.x * tx) * (1.0f - ty) + (t01.x * (1.0f - tx) + t11.x * tx) * ty,
              (t00.y * (1.0f - tx) + t10.y * tx) * (1.0f - ty) + (t01.y * (1.0f - tx) + t11.y * tx) * ty,
              (t00.z * (1.0f - tx) + t10.z * tx) * (1.0f - ty) + (t01.z * (1.0f - tx) + t11.z * tx) * ty};
  }
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

// ---- environment importance sampling (NB_SAMPLE_ENV_NEE; no counterpart in the reference,
// whose README lists it as planned work) ----------------------------------------------------

// largest i in [0, n - 2] with c[i] <= u, for a CDF c[0] = 0 ... c[n - 1] = 1 and u in [0, 1)
__device__ __forceinline__ uint32_t cdf_index(const float* c, uint32_t n, float u) {
  uint32_t lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(c + mid) <= u) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Direction of an environment sample for uniform (u1, u2).  Constant environment: uniform on
// the sphere.  Equirect and cube: texel row by the marginal CDF, column by the row's CDF,
// uniform inside the texel cell, mapped like env_lookup.  Equirect: theta = pi v,
// phi = 2 pi (u - 1/2), d = (sin theta sin phi, cos theta, -sin theta cos phi).  Cube: row
// f N + r of face f, s = 2 (x + du) / N - 1, t = 2 (r + dv) / N - 1, d = the point (s, t) of
// face f (the inverse of cube_face), normalised.
__device__ V3 env_sample_dir(const DevEnv& env, float u1, float u2) {
  if (env.kind == kEnvConstant) {
    const float z = 1.0f - 2.0f * u1;
    const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float sp, cp;
    nb_sincos(kTwoPi * u2 - kPi, &sp, &cp);
    return V3{r * cp, r * sp, z};
  }
  const uint32_t W = env.width, H = env.height;
  const uint32_t y = cdf_index(env.cdf_rows, H + 1, u1);
  const float r0 = __ldg(env.cdf_rows + y), r1 = __ldg(env.cdf_rows + y + 1);
  const float dv = r1 > r0 ? fminf((u1 - r0) / (r1 - r0), 0.99999994f) : 0.5f;
  const float* row = env.cdf_cols + (size_t)y * (W + 1);
  const uint32_t x = cdf_index(row, W + 1, u2);
  const float c0 = __ldg(row + x), c1 = __ldg(row + x + 1);
  const float du = c1 > c0 ? fminf((u2 - c0) / (c1 - c0), 0.99999994f) : 0.5f;
  if (env.kind == kEnvCube) {
    const uint32_t f = y / W, r = y - f * W;
    const float s = 2.0f * (((float)x + du) / (float)W) - 1.0f, t = 2.0f * (((float)r + dv) / (float)W) - 1.0f;
    V3 d;
    switch (f) {
      case 0: d = V3{1.0f, -t, -s}; break;
      case 1: d = V3{-1.0f, -t, s}; break;
      case 2: d = V3{s, 1.0f, t}; break;
      case 3: d = V3{s, -1.0f, -t}; break;
      case 4: d = V3{s, -t, 1.0f}; break;
      default: d = V3{-s, -t, -1.0f}; break;
    }
    return normalize(d);
  }
  const float u = ((float)x + du) / (float)W, v = ((float)y + dv) / (float)H;
  float st, ct, sp, cp;
  nb_sincos(kPi * v, &st, &ct);
  nb_sincos(kTwoPi * (u - 0.5f), &sp, &cp);
  return V3{st * sp, ct, -st * cp};
}

// Solid-angle density with which env_sample_dir produces the unit direction d: 1/(4 pi) for a
// constant environment; pdf_uv of d's texel / (2 pi^2 sin theta) for an equirect map; for a
// cube map pdf_uv of d's texel x (1 + s^2 + t^2)^(3/2) / 24 (the table's v spans 6 faces,
// (s, t) spans [-1, 1]^2 per face, and d omega = ds dt / (1 + s^2 + t^2)^(3/2)).
__device__ float env_pdf(const DevEnv& env, V3 d) {
  if (env.kind == kEnvConstant) return 0.0795774715f;
  if (env.kind == kEnvCube) {
    float s, t;
    const uint32_t f = cube_face(d, &s, &t);
    if (s != s || t != t) return 0.0f;
    const int N = (int)env.width;
    const int x = min(max((int)((s + 1.0f) * 0.5f * (float)N), 0), N - 1);
    const int y = (int)f * N + min(max((int)((t + 1.0f) * 0.5f * (float)N), 0), N - 1);
    const float j = 1.0f + s * s + t * t;
    return __ldg(env.pdf_uv + (size_t)y * N + x) * (j * sqrtf(j)) * (1.0f / 24.0f);
  }
  const float u = nb_atan2(d.x, -d.z) * 0.159154943f + 0.5f;
  const float cy = fminf(fmaxf(d.y, -1.0f), 1.0f);
  const float v = nb_acos(cy) * 0.318309886f;
  if (u != u || v != v) return 0.0f;
  const int W = (int)env.width, H = (int)env.height;
  const int x = min(max((int)(u * (float)W), 0), W - 1), y = min(max((int)(v * (float)H), 0), H - 1);
  const float sin_t = sqrtf(fmaxf(0.0f, (1.0f - cy) * (1.0f + cy)));
  if (!(sin_t > 0.0f)) return 0.0f;
  return __ldg(env.pdf_uv + (size_t)y * W + x) / (19.7392088f * sin_t);  // 2 pi^2
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

// Appends the surviving rays of one block to the next bounce's queue grouped by direction (a
// counting sort over the block: one global atomic per block).  The block's input rays are
// neighbours in the image (tiled queue order), so each run of same-bin rays that a trace warp
// takes together starts from one small patch of the image and points nearly the same way.
// Bins: the cube face of the direction's major axis (6) x a 4 x 4 grid of the other two
// components over that face (96).  Against grouping by octant (itself 12% faster secondary
// traversal than the input order): 6.5% faster on uniform-hemisphere probe rays, +0.6% on the
// benchmark frame, whose cosine and GGX bounces the octant already groups well.
// The queue order changes no result: rays carry their path id.  Call from every thread of
// the block (block-uniform control flow); sh holds 2 kDirBins words, the first kDirBins
// zero before the first call (append_init) - each call leaves them zero again.
constexpr uint32_t kDirBins = 96;
__device__ __forceinline__ uint32_t dir_bin(float4 d) {
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  float a, u, v;
  uint32_t face;
  if (ax >= ay && ax >= az) {
    a = ax; face = d.x < 0.0f ? 1u : 0u; u = d.y; v = d.z;
  } else if (ay >= az) {
    a = ay; face = d.y < 0.0f ? 3u : 2u; u = d.z; v = d.x;
  } else {  // also NaN directions: face 4, cell 0
    a = az; face = d.z < 0.0f ? 5u : 4u; u = d.x; v = d.y;
  }
  const float h = 0.5f * a;
  const uint32_t qu = (uint32_t)(u > -h) + (uint32_t)(u > 0.0f) + (uint32_t)(u > h);
  const uint32_t qv = (uint32_t)(v > -h) + (uint32_t)(v > 0.0f) + (uint32_t)(v > h);
  return face * 16u + qu * 4u + qv;
}
__device__ __forceinline__ void append_init(uint32_t* sh) {
  for (uint32_t i = threadIdx.x; i < kDirBins; i += blockDim.x) sh[i] = 0u;
  __syncthreads();
}
// k_shade: blocks of 256 threads at 64 registers, 4 per SM.  Each block bins its survivors
// by direction, and the binning's two block-wide barriers stall only that block.  With one
// 1024-thread block per SM (twice the survivors per bin of 512 threads, which once paid) every
// barrier stalled the whole SM; since lanes refill during traversal, the larger bins save
// little: benchmark frame 101.1 ms with 1024 threads, 100.4 with 512, 100.1 with 256 (shading
// 9.6 -> 8.2 ms, traversal +0.3 ms); a warp-level append without binning: 100.4 (shading 7.4,
// traversal +1.4).  The NEE and cache shade kernels (78 registers) run 256 threads without the
// register cap, which would spill
constexpr int kShadeThreads = 256;
constexpr int kShadeBlocksPerSM = 4;
constexpr int kShadeExtThreads = 256;
__device__ __forceinline__ uint32_t block_append_binned(uint32_t* counter, bool active, float4 dir, uint32_t* sh) {
  uint32_t* cnt = sh;
  uint32_t* off = sh + kDirBins;
  const uint32_t key = active ? dir_bin(dir) : kDirBins;  // kDirBins: no bin
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t grp = __match_any_sync(0xFFFFFFFFu, key);
  const int leader = __ffs(grp) - 1;
  uint32_t woff = 0;
  if (active && lane == leader) woff = atomicAdd(&cnt[key], (uint32_t)__popc(grp));
  woff = __shfl_sync(0xFFFFFFFFu, woff, leader);
  const uint32_t rank = (uint32_t)__popc(grp & ((1u << lane) - 1u));
  __syncthreads();
  if (warp == 0) {  // exclusive bin offsets, one global atomic; counts cleared for the next call
    static_assert(kDirBins == 96, "three bins per lane of the scanning warp");
    const uint32_t c0 = cnt[3 * lane], c1 = cnt[3 * lane + 1], c2 = cnt[3 * lane + 2];
    const uint32_t own = c0 + c1 + c2;
    uint32_t incl = own;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
      if (lane >= d) incl += t;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    uint32_t base = 0;
    if (lane == 0 && total) base = atomicAdd(counter, total);
    base = __shfl_sync(0xFFFFFFFFu, base, 0) + incl - own;
    off[3 * lane] = base;
    off[3 * lane + 1] = base + c0;
    off[3 * lane + 2] = base + c0 + c1;
    cnt[3 * lane] = cnt[3 * lane + 1] = cnt[3 * lane + 2] = 0u;
  }
  __syncthreads();
  return active ? off[key] + woff + rank : 0u;
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


// Material and geometry of a hit (raytracing_sw.wgsl:138-173).  pos / nrm / tng are only
// filled for non-emissive hits: an emissive hit ends the path (pathtracing.wgsl:172-174).
struct HitSurface {
  V3 color;
  float roughness, metallic;
  bool emissive;
  V3 pos, nrm, tng;
};

__device__ __forceinline__ void load_hit_surface(const DevScene& s, uint32_t inst, float4 O, float4 H, V3 rdir,
                                                 HitSurface& hs) {
  // the triangle's vertex indices are loaded before the instance record is looked at, so the
  // two loads overlap (they are valid for every hit, emissive or not)
  const uint32_t tri = __float_as_uint(H.w);
  const uint32_t i0 = __ldg(s.tri_idx + 3 * (size_t)tri), i1 = __ldg(s.tri_idx + 3 * (size_t)tri + 1),
                 i2 = __ldg(s.tri_idx + 3 * (size_t)tri + 2);
  const float4* sh = s.inst_shade + 6 * (size_t)inst;
  const float4 c0 = ld4(sh), c1 = ld4(sh + 1), c2 = ld4(sh + 2);
  const float4 l0 = ld4(sh + 3), l1 = ld4(sh + 4), l2 = ld4(sh + 5);
  hs.color = V3{c0.w, c1.w, c2.w};
  hs.roughness = l0.w;
  hs.metallic = l1.w;
  hs.emissive = l2.w > 0.0f;  // EMISSIVE (raytracing_sw.wgsl:168-170)
  if (hs.emissive) return;
  // hit attributes (raytracing_sw.wgsl:146-158)
  const float4 a0 = ld4(s.vattr + 2 * (size_t)i0), a1 = ld4(s.vattr + 2 * (size_t)i1),
               a2 = ld4(s.vattr + 2 * (size_t)i2);
  const float4 b0 = ld4(s.vattr + 2 * (size_t)i0 + 1), b1 = ld4(s.vattr + 2 * (size_t)i1 + 1),
               b2 = ld4(s.vattr + 2 * (size_t)i2 + 1);
  const float u = H.y, v = H.z;
  const float w0 = 1.0f - u - v;
  const V3 ln = xyz(a0) * w0 + xyz(a1) * u + xyz(a2) * v;
  const V3 lt = xyz(b0) * w0 + xyz(b1) * u + xyz(b2) * v;
  hs.nrm = V3{dot(xyz(c0), ln), dot(xyz(c1), ln), dot(xyz(c2), ln)};
  hs.tng = V3{dot(xyz(l0), lt), dot(xyz(l1), lt), dot(xyz(l2), lt)};
  hs.pos = xyz(O) + H.x * rdir;
}

// Rotated Sobol samples of a bounce (pathtracing.wgsl:151-159, 176-178)
__device__ __forceinline__ void bounce_samples(const PathBatch& pb, uint32_t sample, uint32_t bounce, float4 shift,
                                               float4& s0, float4& s1) {
  const uint32_t sb = sample * kLdsStride + 1u + bounce * kLdsPerBounce;
  s0 = sobol_read(pb.sobol, pb.sobol_entries, sb);
  s1 = sobol_read(pb.sobol, pb.sobol_entries, sb + 1u);
  s0 = make_float4(fract(s0.x + shift.x), fract(s0.y + shift.y), fract(s0.z + shift.z), 0.0f);
  s1 = make_float4(0.0f, fract(s1.y + shift.y), fract(s1.z + shift.z), 0.0f);
}

// Lobe choice and direction sampling at a non-emissive hit (pathtracing.wgsl:179-224).
// weight is the factor the throughput is multiplied by.  With kPdf, pdf is the solid-angle
// density of wi under the chosen lobe times its selection probability (used only by the
// radiance cache's path-spread heuristic; +inf for a perfect mirror).
struct BsdfSample {
  V3 wi, weight, wo, n;
  float cos_o, pdf;
};

template <bool kPdf>
__device__ __forceinline__ BsdfSample sample_bsdf(const HitSurface& hs, V3 rdir, float4 s0, float4 s1) {
  BsdfSample out;
  const V3 color = hs.color;
  const float roughness = hs.roughness, metallic = hs.metallic;
  const float alpha = roughness * roughness;
  const float alpha2 = alpha * alpha;
  const V3 nn = normalize(hs.nrm);
  const V3 wo = normalize(-rdir);
  const float cosThetaO = dot(wo, nn);
  V3 wi;
  const V3 F0 = V3{0.04f, 0.04f, 0.04f} * (1.0f - metallic) + color * metallic;
  const float specular_weight = luminance(F_schlick(dot(wo, nn), F0));
  const float diffuse_weight = (1.0f - metallic) * luminance(color);
  const float p_specular = specular_weight / (specular_weight + diffuse_weight);
  const float p_diffuse = 1.0f - p_specular;
  out.pdf = 0.0f;
  if (s0.x < p_specular) {
    const V3 wm = sample_vndf_iso(s0.y, s0.z, wo, alpha, nn);
    const V3 ni = -wo;
    wi = ni - (2.0f * dot(wm, ni)) * wm;  // reflect(-wo, wm)
    const float cosThetaD = dot(wo, wm);
    const float cosThetaI = dot(wi, nn);
    const V3 F = F_schlick(cosThetaD, F0);
    const float LambdaL = lambda_tr(cosThetaI, alpha2);
    const float LambdaV = lambda_tr(cosThetaO, alpha2);
    const V3 spec = F * (1.0f + LambdaV) / (1.0f + LambdaL + LambdaV);
    out.weight = spec / p_specular;
    if (kPdf) {
      // VNDF reflection density: G1(wo) D(wm) / (4 cos_o), D the Trowbridge-Reitz NDF
      const float nm = dot(nn, wm);
      const float den = nm * nm * (alpha2 - 1.0f) + 1.0f;
      const float D = alpha2 / (kPi * den * den);
      out.pdf = alpha2 > 0.0f ? p_specular * D / (4.0f * (1.0f + LambdaV) * fabsf(cosThetaO))
                              : __int_as_float(0x7f800000);
    }
  } else {
    const V3 nt = normalize(hs.tng - dot(hs.tng, nn) * nn);  // build_tbn (common.wgsl:55-59)
    const V3 bt = cross(nn, nt);
    const float phi = kTwoPi * s1.y;
    const float sinT = sqrtf(1.0f - s1.z);
    const float cosT = sqrtf(s1.z);
    float sp, cp;
    nb_sincos(phi, &sp, &cp);
    const V3 ls{cp * sinT, sp * sinT, cosT};
    wi = nt * ls.x + bt * ls.y + nn * ls.z;
    const V3 wm = normalize(wi + wo);
    const float cosThetaD = dot(wi, wm);
    const float cosThetaI = dot(wi, nn);
    const float FD90 = 0.5f + 2.0f * alpha * pow2(cosThetaD);
    const float response =
        (1.0f + (FD90 - 1.0f) * pow5(1.0f - cosThetaI)) * (1.0f + (FD90 - 1.0f) * pow5(1.0f - cosThetaO));
    const V3 diffuse = (1.0f - metallic) * color * response;
    out.weight = diffuse / p_diffuse;
    if (kPdf) out.pdf = p_diffuse * cosT * (1.0f / kPi);
  }
  out.wi = wi;
  out.wo = wo;
  out.n = nn;
  out.cos_o = cosThetaO;
  return out;
}

// Russian roulette probability (pathtracing.wgsl:225-236).  rr_start > 0 is the start-bounce
// variant (BASELINE's "RR from bounce 3"): survival 1 before that bounce, the reference's
// schedule from it on; 0 is the reference.
__device__ __forceinline__ float rr_continue(uint32_t bounce, const JobParams& jp, V3 T) {
  float p_continue = fminf(1.0f - pow8((float)bounce / (float)jp.bounces), 1.0f);
  p_continue = p_continue * fminf(luminance(T) * jp.cf, 1.0f);
  return bounce < jp.rr_start ? 1.0f : p_continue;
}

__global__ void __launch_bounds__(kShadeThreads, kShadeBlocksPerSM) k_shade(PathBatch pb, const WaveTables wt, uint32_t bounce) {
  __shared__ Segment segs[nb::kMaxWaveSegments];
  __shared__ uint32_t append_sh[2 * kDirBins];
  stage_segments(segs, wt);
  append_init(append_sh);
  const uint32_t n = pb.counts[bounce];
  const bool odd = (bounce & 1) != 0;
  const float4* __restrict__ in_o = odd ? pb.q_o[1] : pb.q_o[0];
  const float4* __restrict__ in_d = odd ? pb.q_d[1] : pb.q_d[0];
  const float4* __restrict__ in_t = odd ? pb.q_t[1] : pb.q_t[0];
  float4* __restrict__ out_o = odd ? pb.q_o[0] : pb.q_o[1];
  float4* __restrict__ out_d = odd ? pb.q_d[0] : pb.q_d[1];
  float4* __restrict__ out_t = odd ? pb.q_t[0] : pb.q_t[1];
  const uint32_t stride = gridDim.x * blockDim.x;
  // whole blocks iterate together: block_append_binned synchronises the block
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    bool cont = false;
    float4 next_o = make_float4(0.f, 0.f, 0.f, 0.f), next_d = next_o, next_t = next_o;
    if (i < n) {
      const float4 O = in_o[i], D = in_d[i], H = pb.hits[i];
      const float4 Tq = bounce == 0 ? make_float4(1.0f, 1.0f, 1.0f, 0.0f) : in_t[i];
      const uint32_t id = __float_as_uint(O.w);
      const Segment sg = segs[find_segment<false>(segs, wt.n_segs, id)];
      const JobParams& jp = wt.jobs[sg.job];
      const DevScene& s = wt.scenes[jp.scene];
      V3 T = xyz(Tq);
      const V3 rdir = xyz(D);
      if (H.x == kNoHit) {
        const V3 L = T * env_lookup(jp.env, rdir);
        pb.radiance[id] = make_float4(L.x, L.y, L.z, 0.0f);
      } else {
        HitSurface hs;
        load_hit_surface(s, pb.hit_inst[i], O, H, rdir, hs);
        if (hs.emissive) {  // pathtracing.wgsl:172-174
          const V3 L = T * hs.color;
          pb.radiance[id] = make_float4(L.x, L.y, L.z, 0.0f);
        } else {
          const uint32_t local = id - sg.path_begin;
          const uint32_t pix = local % jp.npix;
          const uint32_t sample = sg.first_sample + local / jp.npix;
          float4 s0, s1;
          bounce_samples(pb, sample, bounce, hash4f(pix % jp.width, pix / jp.width), s0, s1);
          const BsdfSample bs = sample_bsdf<false>(hs, rdir, s0, s1);
          T = T * bs.weight;
          const float p_continue = rr_continue(bounce, jp, T);
          if (s0.z < p_continue && bounce < jp.bounces) {
            T = T / p_continue;
            cont = true;
            next_o = make_float4(hs.pos.x, hs.pos.y, hs.pos.z, O.w);
            next_d = make_float4(bs.wi.x, bs.wi.y, bs.wi.z, D.w);
            next_t = make_float4(T.x, T.y, T.z, 0.0f);
          } else {
            pb.radiance[id] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // ends without radiance
          }
        }
      }
    }
    const uint32_t slot = block_append_binned(pb.counts + bounce + 1, cont, next_d, append_sh);
    if (cont) {
      out_o[slot] = next_o;
      out_d[slot] = next_d;
      out_t[slot] = next_t;
    }
  }
}

// 32-bit integer finaliser (Wellons' lowbias32)
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ nb::CacheFeatures cache_features(const HitSurface& hs, const BsdfSample& bs, uint32_t tag) {
  nb::CacheFeatures f;
  f.pos[0] = hs.pos.x; f.pos[1] = hs.pos.y; f.pos[2] = hs.pos.z;
  f.roughness = hs.roughness;
  f.wo[0] = bs.wo.x; f.wo[1] = bs.wo.y; f.wo[2] = bs.wo.z;
  f.metallic = hs.metallic;
  f.n[0] = bs.n.x; f.n[1] = bs.n.y; f.n[2] = bs.n.z;
  f.tag = tag;
  f.color[0] = hs.color.x; f.color[1] = hs.color.y; f.color[2] = hs.color.z;
  f.pad = 0.0f;
  return f;
}

// Shade for the radiance-cache mode.  The prefix of every path is the plain tracer's (same
// samples, lobes and Russian roulette); what changes is where it ends:
//  - path spread (Mueller et al. 2021, sec. 3.3): a0 = |x0 - x1|^2 / (4 pi cos1) at the
//    primary hit, and sqrt a(x1..xn) = sum_{i>=2} |x_{i-1} - x_i| / sqrt(p_{i-1} cos_i), with
//    p the density of the sampled direction.  At the first vertex where sqrt a > sqrt(c a0)
//    (or at the last bounce) the path becomes an image query: its sample is T * cache(x).
//  - one path per group of `stride` path ids (position in the group hashed from the group
//    and the frame) is a training path: it records each vertex (features and the factor its
//    throughput is multiplied by), continues past its query vertex for `extra` vertices and
//    ends in a tail query that closes its radiance chain with the cache (self-training),
//    unless a miss, an emitter or Russian roulette ends it first.
__global__ void __launch_bounds__(kShadeExtThreads) k_shade_cache(PathBatch pb, const WaveTables wt, const nb::CacheWave cw,
                                                     uint32_t bounce) {
  using nb::CacheQuery;
  __shared__ Segment segs[nb::kMaxWaveSegments];
  __shared__ uint32_t append_sh[2 * kDirBins];
  stage_segments(segs, wt);
  append_init(append_sh);
  const uint32_t n = pb.counts[bounce];
  const bool odd = (bounce & 1) != 0;
  const float4* __restrict__ in_o = odd ? pb.q_o[1] : pb.q_o[0];
  const float4* __restrict__ in_d = odd ? pb.q_d[1] : pb.q_d[0];
  const float4* __restrict__ in_t = odd ? pb.q_t[1] : pb.q_t[0];
  const float4* __restrict__ in_x = odd ? cw.q_x[1] : cw.q_x[0];
  float4* __restrict__ out_o = odd ? pb.q_o[0] : pb.q_o[1];
  float4* __restrict__ out_d = odd ? pb.q_d[0] : pb.q_d[1];
  float4* __restrict__ out_t = odd ? pb.q_t[0] : pb.q_t[1];
  float4* __restrict__ out_x = odd ? cw.q_x[0] : cw.q_x[1];
  const uint32_t G = *cw.stride;
  const uint32_t frame_key = mix32(cw.frame ^ 0x5bd1e995u);
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    bool cont = false, image_q = false, tail_q = false;
    float4 next_o = make_float4(0.f, 0.f, 0.f, 0.f), next_d = next_o, next_t = next_o, next_x = next_o;
    nb::CacheFeatures f{};
    V3 Tq3{0.0f, 0.0f, 0.0f};
    uint32_t slot = ~0u;
    if (i < n) {
      const float4 O = in_o[i], D = in_d[i], H = pb.hits[i];
      const float4 Tq = bounce == 0 ? make_float4(1.0f, 1.0f, 1.0f, 0.0f) : in_t[i];
      const uint32_t id = __float_as_uint(O.w);
      const Segment sg = segs[find_segment<false>(segs, wt.n_segs, id)];
      const JobParams& jp = wt.jobs[sg.job];
      const DevScene& s = wt.scenes[jp.scene];
      V3 T = xyz(Tq);
      const V3 rdir = xyz(D);
      float budget = 0.0f, pdf_prev = 0.0f;
      uint32_t flags = 0;
      if (bounce == 0) {
        const uint32_t group = id / G;
        const bool train = group < cw.max_slots && id % G == mix32(group ^ frame_key) % G;
        slot = train ? group : ~0u;
        flags = train ? nb::kPathTraining : 0u;
      } else {
        const float4 X = in_x[i];
        budget = X.x;
        pdf_prev = X.y;
        slot = __float_as_uint(X.z);
        flags = __float_as_uint(X.w);
      }
      const bool training = (flags & nb::kPathTraining) != 0;
      const bool image_done = (flags & nb::kPathImageDone) != 0;
      if (H.x == kNoHit) {
        const V3 E = env_lookup(jp.env, rdir);
        if (!image_done) {
          const V3 L = T * E;
          pb.radiance[id] = make_float4(L.x, L.y, L.z, 0.0f);
        }
        if (training) cw.tail[slot] = make_float4(E.x, E.y, E.z, 0.0f);
      } else {
        HitSurface hs;
        load_hit_surface(s, pb.hit_inst[i], O, H, rdir, hs);
        if (hs.emissive) {
          if (!image_done) {
            const V3 L = T * hs.color;
            pb.radiance[id] = make_float4(L.x, L.y, L.z, 0.0f);
          }
          if (training) cw.tail[slot] = make_float4(hs.color.x, hs.color.y, hs.color.z, 0.0f);
        } else {
          const uint32_t local = id - sg.path_begin;
          const uint32_t pix = local % jp.npix;
          const uint32_t sample = sg.first_sample + local / jp.npix;
          float4 s0, s1;
          bounce_samples(pb, sample, bounce, hash4f(pix % jp.width, pix / jp.width), s0, s1);
          const BsdfSample bs = sample_bsdf<true>(hs, rdir, s0, s1);
          const float dist2 = H.x * H.x * dot(rdir, rdir);
          const float cos_v = fabsf(bs.cos_o);
          if (bounce == 0)
            budget = cw.spread_c < 0.0f ? -1.0f : sqrtf(cw.spread_c * dist2 / (4.0f * kPi * cos_v));
          else
            budget = budget - sqrtf(dist2 / (pdf_prev * cos_v));
          f = cache_features(hs, bs, id);
          Tq3 = T;
          const V3 Tn = T * bs.weight;
          const float p_continue = rr_continue(bounce, jp, Tn);
          const bool rr_ok = s0.z < p_continue && bounce < jp.bounces;
          // an infinite c turns the spread rule off; otherwise NaN budgets (degenerate
          // geometry) end the prefix as well
          const bool spread_end = !isinf(cw.spread_c) && !(budget >= 0.0f);
          image_q = !image_done && (spread_end || bounce >= jp.bounces);
          bool go = false;
          if (!training) {
            go = !image_q && rr_ok;
          } else {
            uint32_t since = (flags >> nb::kPathSinceShift) & 0xFFu;
            // a training path that reaches the vertex cap ends here, its pixel sample included
            if (bounce >= nb::kCacheMaxVertices) image_q = !image_done;
            if (image_q) {
              flags |= nb::kPathImageDone;
              since = 0;
            }
            if (((flags & nb::kPathImageDone) && since >= cw.extra) || bounce >= nb::kCacheMaxVertices) {
              tail_q = true;
            } else {
              const V3 w = rr_ok ? bs.weight / p_continue : V3{0.0f, 0.0f, 0.0f};
              nb::TrainVertex tv;
              tv.f = f;
              tv.w = make_float4(w.x, w.y, w.z, 0.0f);
              cw.verts[(size_t)slot * nb::kCacheMaxVertices + bounce] = tv;
              cw.vert_count[slot] = bounce + 1;
              go = rr_ok;
              if (!go) cw.tail[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
              if (go && (flags & nb::kPathImageDone)) since += 1;
            }
            flags = (flags & 0xFFu) | (since << nb::kPathSinceShift);
          }
          if (go) {
            const V3 Tc = Tn / p_continue;
            cont = true;
            next_o = make_float4(hs.pos.x, hs.pos.y, hs.pos.z, O.w);
            next_d = make_float4(bs.wi.x, bs.wi.y, bs.wi.z, D.w);
            next_t = make_float4(Tc.x, Tc.y, Tc.z, 0.0f);
            next_x = make_float4(budget, bs.pdf, __uint_as_float(slot), __uint_as_float(flags));
          }
        }
      }
    }
    const uint32_t at = block_append_binned(pb.counts + bounce + 1, cont, next_d, append_sh);
    if (cont) {
      out_o[at] = next_o;
      out_d[at] = next_d;
      out_t[at] = next_t;
      out_x[at] = next_x;
    }
    const uint32_t qi = warp_append(cw.n_queries, image_q);
    if (image_q && qi < cw.max_queries) {
      CacheQuery q;
      q.f = f;
      q.T = make_float4(Tq3.x, Tq3.y, Tq3.z, 0.0f);
      cw.queries[qi] = q;
    }
    const uint32_t ti = warp_append(cw.n_queries, tail_q);
    if (tail_q && ti < cw.max_queries) {
      CacheQuery q;
      q.f = f;
      q.f.tag = nb::kCacheTailBit | slot;
      q.T = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
      cw.queries[ti] = q;
    }
  }
}

// f cos(theta_i) of each lobe of the reference BRDF for an arbitrary direction wi, and each
// lobe's sampling density for wi times its selection probability (the densities the lobe
// sampling of sample_bsdf realises).  Specular: F D G2 / (4 cos_o) with the Trowbridge-Reitz
// D and the reference's Lambda (so that f cos / pdf_vndf is the reference's F (1 + L_V) /
// (1 + L_L + L_V)); diffuse: (1 - metallic) color response cos_i / pi.  A perfect mirror
// (alpha = 0) has no specular part here: only lobe sampling can find it.
struct BsdfEval {
  V3 spec, diff;
  float q_spec, q_diff;
};

__device__ __forceinline__ BsdfEval eval_bsdf(const HitSurface& hs, const BsdfSample& bs, V3 wi) {
  BsdfEval ev;
  const V3 color = hs.color;
  const float metallic = hs.metallic;
  const float alpha = hs.roughness * hs.roughness;
  const float alpha2 = alpha * alpha;
  const V3 nn = bs.n, wo = bs.wo;
  const float cos_o = bs.cos_o, cos_i = dot(wi, nn);
  const V3 F0 = V3{0.04f, 0.04f, 0.04f} * (1.0f - metallic) + color * metallic;
  const float specular_weight = luminance(F_schlick(dot(wo, nn), F0));
  const float diffuse_weight = (1.0f - metallic) * luminance(color);
  const float p_specular = specular_weight / (specular_weight + diffuse_weight);
  const float p_diffuse = 1.0f - p_specular;
  const V3 wm = normalize(wi + wo);
  if (alpha2 > 0.0f) {
    const float nm = dot(nn, wm);
    const float den = nm * nm * (alpha2 - 1.0f) + 1.0f;
    const float D = alpha2 / (kPi * den * den);
    const float LambdaV = lambda_tr(cos_o, alpha2), LambdaL = lambda_tr(cos_i, alpha2);
    const V3 F = F_schlick(dot(wo, wm), F0);
    ev.spec = F * (D / ((1.0f + LambdaV + LambdaL) * 4.0f * cos_o));
    ev.q_spec = p_specular * D / (4.0f * (1.0f + LambdaV) * cos_o);
  } else {
    ev.spec = V3{0.0f, 0.0f, 0.0f};
    ev.q_spec = __int_as_float(0x7f800000);
  }
  const float cosThetaD = dot(wi, wm);
  const float FD90 = 0.5f + 2.0f * alpha * pow2(cosThetaD);
  const float response = (1.0f + (FD90 - 1.0f) * pow5(1.0f - cos_i)) * (1.0f + (FD90 - 1.0f) * pow5(1.0f - cos_o));
  ev.diff = (1.0f - metallic) * color * (response * cos_i * (1.0f / kPi));
  ev.q_diff = p_diffuse * cos_i * (1.0f / kPi);
  return ev;
}

__device__ __forceinline__ bool finite3(V3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }

// Shade with environment next-event estimation (NB_SAMPLE_ENV_NEE).  The path is the
// reference's (same samples, lobe choice, VNDF / cosine sampling, Russian roulette); in
// addition every non-emissive vertex samples one environment direction (importance sampling
// of the environment's radiance, Sobol dimensions the reference leaves unused: sobol_0.w and
// sobol_1.x of the bounce) and queues a shadow ray carrying that sample's contribution.  The
// two techniques are combined per BRDF lobe with the power heuristic: an environment sample
// weighs lobe k by p_env^2 / (q_k^2 + p_env^2), a lobe-sampled ray that escapes to the
// environment by q^2 / (q^2 + p_env^2), q = the lobe's density (carried in q_t.w).  Where
// next-event estimation cannot reach a direction (below the shading normal, cos_o <= 0, a
// mirror lobe) the carried density is +inf and the lobe sample keeps full weight, so the
// estimator stays unbiased.  Radiance accumulates per path (+=) instead of being written once.
__global__ void __launch_bounds__(kShadeExtThreads) k_shade_nee(PathBatch pb, const WaveTables wt, const ShadowQueue sq,
                                                   uint32_t bounce) {
  __shared__ Segment segs[nb::kMaxWaveSegments];
  __shared__ uint32_t append_sh[2 * kDirBins];
  stage_segments(segs, wt);
  append_init(append_sh);
  const uint32_t n = pb.counts[bounce];
  const bool odd = (bounce & 1) != 0;
  const float4* __restrict__ in_o = odd ? pb.q_o[1] : pb.q_o[0];
  const float4* __restrict__ in_d = odd ? pb.q_d[1] : pb.q_d[0];
  const float4* __restrict__ in_t = odd ? pb.q_t[1] : pb.q_t[0];
  float4* __restrict__ out_o = odd ? pb.q_o[0] : pb.q_o[1];
  float4* __restrict__ out_d = odd ? pb.q_d[0] : pb.q_d[1];
  float4* __restrict__ out_t = odd ? pb.q_t[0] : pb.q_t[1];
  const uint32_t stride = gridDim.x * blockDim.x;
  const float kInf = __int_as_float(0x7f800000);
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    bool cont = false, shadow = false;
    float4 next_o = make_float4(0.f, 0.f, 0.f, 0.f), next_d = next_o, next_t = next_o;
    float4 sh_o = next_o, sh_d = next_o, sh_c = next_o;
    if (i < n) {
      const float4 O = in_o[i], D = in_d[i], H = pb.hits[i];
      const float4 Tq = bounce == 0 ? make_float4(1.0f, 1.0f, 1.0f, 0.0f) : in_t[i];
      const uint32_t id = __float_as_uint(O.w);
      const Segment sg = segs[find_segment<false>(segs, wt.n_segs, id)];
      const JobParams& jp = wt.jobs[sg.job];
      const DevScene& s = wt.scenes[jp.scene];
      V3 T = xyz(Tq);
      const V3 rdir = xyz(D);
      if (H.x == kNoHit) {
        V3 L = T * env_lookup(jp.env, rdir);
        const float q = Tq.w;  // density of the lobe sample that made this ray (bounce > 0)
        if (bounce > 0 && q < kInf) {
          const float pe = env_pdf(jp.env, normalize(rdir));
          L = L * (q * q / (q * q + pe * pe));
        }
        const float4 c = pb.radiance[id];
        pb.radiance[id] = make_float4(c.x + L.x, c.y + L.y, c.z + L.z, 0.0f);
      } else {
        HitSurface hs;
        load_hit_surface(s, pb.hit_inst[i], O, H, rdir, hs);
        if (hs.emissive) {
          const V3 L = T * hs.color;
          const float4 c = pb.radiance[id];
          pb.radiance[id] = make_float4(c.x + L.x, c.y + L.y, c.z + L.z, 0.0f);
        } else {
          const uint32_t local = id - sg.path_begin;
          const uint32_t pix = local % jp.npix;
          const uint32_t sample = sg.first_sample + local / jp.npix;
          const float4 shift = hash4f(pix % jp.width, pix / jp.width);
          float4 s0, s1;
          bounce_samples(pb, sample, bounce, shift, s0, s1);
          const BsdfSample bs = sample_bsdf<true>(hs, rdir, s0, s1);
          // jobs without the flag take the plain estimator's exact path (one contribution
          // added onto zero, lobe samples at full weight)
          const bool nee_ok = (jp.flags & nb::kJobEnvNee) && bs.cos_o > 0.0f;
          if (nee_ok) {
            const uint32_t sb = sample * kLdsStride + 1u + bounce * kLdsPerBounce;
            const float u1 = fract(sobol_read(pb.sobol, pb.sobol_entries, sb).w + shift.w);
            const float u2 = fract(sobol_read(pb.sobol, pb.sobol_entries, sb + 1u).x + shift.x);
            const V3 we = env_sample_dir(jp.env, u1, u2);
            const float pe = env_pdf(jp.env, we);
            if (pe > 0.0f && dot(we, bs.n) > 0.0f) {
              const BsdfEval ev = eval_bsdf(hs, bs, we);
              const float pe2 = pe * pe;
              const float ws = pe2 / (ev.q_spec * ev.q_spec + pe2), wd = pe2 / (ev.q_diff * ev.q_diff + pe2);
              const V3 C = T * env_lookup(jp.env, we) * (ev.spec * ws + ev.diff * wd) / pe;
              if (finite3(C) && (C.x > 0.0f || C.y > 0.0f || C.z > 0.0f)) {
                shadow = true;
                sh_o = make_float4(hs.pos.x, hs.pos.y, hs.pos.z, O.w);
                sh_d = make_float4(we.x, we.y, we.z, D.w);
                sh_c = make_float4(C.x, C.y, C.z, 0.0f);
              }
            }
          }
          T = T * bs.weight;
          const float p_continue = rr_continue(bounce, jp, T);
          if (s0.z < p_continue && bounce < jp.bounces) {
            T = T / p_continue;
            cont = true;
            const float q = (nee_ok && dot(bs.wi, bs.n) > 0.0f) ? bs.pdf : kInf;
            next_o = make_float4(hs.pos.x, hs.pos.y, hs.pos.z, O.w);
            next_d = make_float4(bs.wi.x, bs.wi.y, bs.wi.z, D.w);
            next_t = make_float4(T.x, T.y, T.z, q);
          }
        }
      }
    }
    const uint32_t slot = block_append_binned(pb.counts + bounce + 1, cont, next_d, append_sh);
    if (cont) {
      out_o[slot] = next_o;
      out_d[slot] = next_d;
      out_t[slot] = next_t;
    }
    const uint32_t ss = warp_append(sq.counts + bounce, shadow);
    if (shadow) {
      sq.o[ss] = sh_o;
      sq.d[ss] = sh_d;
      sq.c[ss] = sh_c;
    }
  }
}

// Shadow rays of one bounce: an any-hit query each (raytracing_sw.wgsl's triangle test and
// BIAS, so the ray leaves its own surface like the reference's extension rays), with lane
// refill (trace_refill); unoccluded rays add their contribution to the path.  A path has at most one shadow ray per bounce, so
// each radiance entry has one writer per launch.  .w of a shadow ray's direction is the index
// of its scene in the wave.
__global__ void __launch_bounds__(kTraceThreads, 8) k_trace_shadow(PathBatch pb, const WaveTables wt, const ShadowQueue sq,
                                                      uint32_t bounce) {
  __shared__ DevScene scenes[nb::kMaxWaveScenes];
  for (uint32_t i = threadIdx.x; i < wt.n_scenes; i += blockDim.x) scenes[i] = wt.scenes[i];
  __syncthreads();
  __shared__ float world[kTraceWarps][kWorldFloats];
  const uint32_t n = sq.counts[bounce];
  const uint32_t st = trace_refill<true, false>(
      sq.fetch + bounce, n,
      [&](uint32_t r, V3& o, V3& d, uint32_t& sidx) {
        const float4 d4 = sq.d[r];
        o = xyz(sq.o[r]);
        d = xyz(d4);
        sidx = __float_as_uint(d4.w);
      },
      [&](uint32_t sidx) -> const DevScene& { return scenes[sidx]; },
      [&](uint32_t r, float t_hit, uint2, uint2) {
        if (t_hit == kNoHit) {
          const uint32_t id = __float_as_uint(sq.o[r].w);
          const float4 c = sq.c[r], rr = pb.radiance[id];
          pb.radiance[id] = make_float4(rr.x + c.x, rr.y + c.y, rr.z + c.z, 0.0f);
        }
      },
      nullptr, world[threadIdx.x >> 5]);
  if (st) atomicOr(pb.status, st);
}

__global__ void k_env_sample(const DevEnv env, const float* __restrict__ u, uint32_t n, float4* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const V3 d = env_sample_dir(env, u[2 * i], u[2 * i + 1]);
    out[i] = make_float4(d.x, d.y, d.z, env_pdf(env, d));
  }
}

// running mean in sample order: out = mix(out, L_k, 1/k) (pathtracing.wgsl:246-260).  Each job
// has at most one segment per wave, so every pixel has one writer.
__global__ void __launch_bounds__(256) k_accumulate(PathBatch pb, const WaveTables wt) {
  __shared__ Segment segs[nb::kMaxWaveSegments];
  stage_segments(segs, wt);
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < wt.n_pix; t += gridDim.x * blockDim.x) {
    const Segment sg = segs[find_segment<true>(segs, wt.n_segs, t)];
    const JobParams& jp = wt.jobs[sg.job];
    const uint32_t pix = t - sg.pix_begin;
    float4 c = jp.out[pix];
    for (uint32_t k = 0; k < sg.n_samples; ++k) {
      const float w = 1.0f / (float)(sg.first_sample + k);
      const float4 L = pb.radiance[(size_t)sg.path_begin + (size_t)k * jp.npix + pix];
      c.x = c.x * (1.0f - w) + L.x * w;
      c.y = c.y * (1.0f - w) + L.y * w;
      c.z = c.z * (1.0f - w) + L.z * w;
    }
    jp.out[pix] = make_float4(c.x, c.y, c.z, 1.0f);
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

cudaError_t launch_trace_rays(const nbd::DevScene& s, const float* rays, uint32_t n, bool any, bool refill,
                              float* hits, uint32_t* inst, uint32_t* fetch, uint32_t* status, int sms,
                              cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(fetch, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
#define NB_TRACE_RAYS(A, R)                                                                            \
  {                                                                                                    \
    static const int g = blocks_for((const void*)nbd::k_trace_rays<A, R>, nbd::kTraceThreads, sms);                  \
    nbd::k_trace_rays<A, R><<<g, nbd::kTraceThreads, 0, st>>>(s, (const float4*)rays, n, (float4*)hits, inst, fetch, status); \
  }
  if (any) {
    if (refill) NB_TRACE_RAYS(true, true) else NB_TRACE_RAYS(true, false)
  } else {
    if (refill) NB_TRACE_RAYS(false, true) else NB_TRACE_RAYS(false, false)
  }
#undef NB_TRACE_RAYS
  return cudaGetLastError();
}

cudaError_t launch_raygen(const PathBatch& pb, const WaveTables& wt, int sms, cudaStream_t st) {
  int g = (wt.flags & kWaveZeroRadiance) ? (int)std::min<uint64_t>((wt.n_paths + 255) / 256, (uint64_t)sms * 16) : 1;
  nbd::k_raygen<<<g < 1 ? 1 : g, 256, 0, st>>>(pb, wt);
  return cudaGetLastError();
}

cudaError_t launch_trace_wave(const PathBatch& pb, const WaveTables& wt, bool single_scene, uint32_t bounce,
                              unsigned long long* ray_total, int sms, cudaStream_t st,
                              unsigned long long* counters) {
  const bool refill = bounce >= 1;
#define NB_TRACE_WAVE(S, C, R)                                                                \
  {                                                                                           \
    static const int g = blocks_for((const void*)nbd::k_trace_wave<S, C, R>, nbd::kTraceThreads, sms);       \
    nbd::k_trace_wave<S, C, R><<<g, nbd::kTraceThreads, 0, st>>>(pb, wt, bounce, ray_total, counters);      \
  }
  if (counters) {
    if (single_scene) {
      if (refill) NB_TRACE_WAVE(true, true, true) else NB_TRACE_WAVE(true, true, false)
    } else {
      if (refill) NB_TRACE_WAVE(false, true, true) else NB_TRACE_WAVE(false, true, false)
    }
  } else if (single_scene) {
    if (refill) NB_TRACE_WAVE(true, false, true) else NB_TRACE_WAVE(true, false, false)
  } else {
    if (refill) NB_TRACE_WAVE(false, false, true) else NB_TRACE_WAVE(false, false, false)
  }
#undef NB_TRACE_WAVE
  return cudaGetLastError();
}

cudaError_t launch_shade(const PathBatch& pb, const WaveTables& wt, uint32_t bounce, int sms, cudaStream_t st) {
  static const int g = blocks_for((const void*)nbd::k_shade, nbd::kShadeThreads, sms);
  nbd::k_shade<<<g, nbd::kShadeThreads, 0, st>>>(pb, wt, bounce);
  return cudaGetLastError();
}

cudaError_t launch_shade_cache(const PathBatch& pb, const WaveTables& wt, const CacheWave& cw, uint32_t bounce,
                               int sms, cudaStream_t st) {
  static const int g = blocks_for((const void*)nbd::k_shade_cache, nbd::kShadeExtThreads, sms);
  nbd::k_shade_cache<<<g, nbd::kShadeExtThreads, 0, st>>>(pb, wt, cw, bounce);
  return cudaGetLastError();
}

cudaError_t launch_shade_nee(const PathBatch& pb, const WaveTables& wt, const ShadowQueue& sq, uint32_t bounce,
                             int sms, cudaStream_t st) {
  static const int g = blocks_for((const void*)nbd::k_shade_nee, nbd::kShadeExtThreads, sms);
  nbd::k_shade_nee<<<g, nbd::kShadeExtThreads, 0, st>>>(pb, wt, sq, bounce);
  return cudaGetLastError();
}

cudaError_t launch_trace_shadow(const PathBatch& pb, const WaveTables& wt, const ShadowQueue& sq, uint32_t bounce,
                                int sms, cudaStream_t st) {
  static const int g = blocks_for((const void*)nbd::k_trace_shadow, nbd::kTraceThreads, sms);
  nbd::k_trace_shadow<<<g, nbd::kTraceThreads, 0, st>>>(pb, wt, sq, bounce);
  return cudaGetLastError();
}

cudaError_t launch_env_sample(const nbd::DevEnv& env, const float* u, uint32_t n, float4* out, int sms,
                              cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int g = (int)std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
  nbd::k_env_sample<<<g, 256, 0, st>>>(env, u, n, out);
  return cudaGetLastError();
}

cudaError_t launch_accumulate(const PathBatch& pb, const WaveTables& wt, int sms, cudaStream_t st) {
  int g = (int)std::min<uint64_t>((wt.n_pix + 255) / 256, (uint64_t)sms * 16);
  nbd::k_accumulate<<<g < 1 ? 1 : g, 256, 0, st>>>(pb, wt);
  return cudaGetLastError();
}

}  // namespace nb

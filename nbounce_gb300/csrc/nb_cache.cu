// Radiance cache: fused BF16 tensor-core MLP (inference, training, Adam) and the cache-mode
// wave driver behind the nb_cache_* C ABI.
//
// The reference has no radiance cache (its README lists neural radiance caching as planned);
// the method is Mueller, Rousselle, Novak, Keller 2021, "Real-time Neural Radiance Caching for
// Path Tracing": a 64-wide, 5-hidden-layer ReLU MLP that maps a vertex (position, directions,
// material) to outgoing radiance, trained online on radiance estimated by a sparse set of
// longer training paths, queried where the other paths end their short prefix.
//
// Kernels (mma.sync m16n8k16, BF16 operands, FP32 accumulation; weights resident in shared
// memory as 336 rows x 64 inputs, rows padded to 72 elements so that ldmatrix is
// conflict-free):
//   k_cache_infer_tc tcgen05.mma (5th-generation tensor cores): operands in shared memory,
//                    FP32 accumulators in tensor memory, 4 groups of 128 rows per CTA
//   k_cache_infer_*  mma.sync: one warp evaluates 32 rows, the activations never leave
//                    registers (the C fragment of layer l, ReLU'd and packed to BF16, is the A
//                    fragment of layer l + 1)
//   k_cache_grad_tc  tcgen05.mma training (the default path): one warpgroup per 128 rows,
//                    forward, backward and weight-gradient GEMMs with TMEM accumulators
//   k_cache_grad     mma.sync training: one CTA of 8 warps takes 128 rows: forward with the activations kept in
//                    shared memory, relative L2 loss (p - y)^2 / (p^2 + 0.01) with the
//                    denominator held constant, backward through the 6 layers; each layer's
//                    weight gradient dZ^T H is a 128-deep GEMM across the CTA's rows written
//                    as a per-CTA FP32 partial (no atomics)
//   k_cache_adam     sums the partials in CTA order (deterministic), Adam update of the FP32
//                    master weights and of their BF16 copy
//   k_cache_count / _offsets / _gather  turn the training paths' vertex chains into records:
//                    radiance targets by a backward walk over the throughput factors, encoded
//                    inputs, reflectance-factorised targets; adapt the training-path density
//                    to the record budget
// The whole per-frame sequence runs without host synchronisation.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include <cuda_bf16.h>

#include "nb_mlp.cuh"
#include "nb_runtime.h"

namespace nbd {

using nb::CacheBounds;
using nb::CacheFeatures;
using nb::CacheQuery;
using nb::kMlpParams;
using nb::kMlpRows;
using nb::TrainVertex;
typedef __nv_bfloat16 bf16;

constexpr int kRS = 72;                                              // shared row stride (elements)
constexpr size_t kWSmem = (size_t)kMlpRows * kRS * sizeof(bf16);     // 48,384 B
constexpr int kInferWarps = 8;
constexpr size_t kInferSmem = kWSmem + (size_t)kInferWarps * 32 * kRS * sizeof(bf16);  // 85,248 B
constexpr int kGradRows = 128;
constexpr size_t kGradSmem = kWSmem + (size_t)8 * kGradRows * kRS * sizeof(bf16);      // 195,840 B
constexpr uint32_t kLiveEnd = 5 * 4096 + 3 * 64;  // parameters past this are padding rows of W_5

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm4(uint32_t a, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
__device__ __forceinline__ void ldsm4t(uint32_t a, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
// D = A (16x16, row-major) * B (16x8) + D, BF16 in, FP32 accumulate
__device__ __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float relu(float x) { return fmaxf(x, 0.0f); }
// x where the bf16 activation h (low or high half of u) is positive, else 0
__device__ __forceinline__ float gate_lo(float x, uint32_t u) {
  return __bfloat162float(__ushort_as_bfloat16((unsigned short)(u & 0xFFFFu))) > 0.0f ? x : 0.0f;
}
__device__ __forceinline__ float gate_hi(float x, uint32_t u) {
  return __bfloat162float(__ushort_as_bfloat16((unsigned short)(u >> 16))) > 0.0f ? x : 0.0f;
}

// Fragment coordinates: lane = 4 g + t.  A (16x16): a0 (g, 2t..), a1 (g+8, 2t..), a2 (g, 2t+8..),
// a3 (g+8, 2t+8..).  B (16x8): b0 (k 2t.., n g), b1 (k 2t+8.., n g).  C (16x8): c0,c1 (g, 2t..),
// c2,c3 (g+8, 2t..).  The C fragments of two adjacent n-tiles are, after packing, the A
// fragment of one k-tile of the next layer.

// A fragments of rows [r0, r0+16) x 64 inputs of a shared row block
__device__ __forceinline__ void load_a(const bf16* rows, int r0, int lane, uint32_t (&a)[4][4]) {
  const int q = lane >> 3, r = lane & 7;
#pragma unroll
  for (int kt = 0; kt < 4; ++kt)
    ldsm4(saddr(rows + (r0 + r + 8 * (q & 1)) * kRS + 16 * kt + 8 * (q >> 1)), a[kt][0], a[kt][1], a[kt][2],
          a[kt][3]);
}

// H' = relu(H W^T) for a 64x64 layer W ([out][in] rows in shared memory), MT row tiles
template <int MT>
__device__ __forceinline__ void layer_fwd(const bf16* W, int lane, const uint32_t (&a)[MT][4][4],
                                          uint32_t (&h)[MT][4][4]) {
  const int q = lane >> 3, r = lane & 7;
#pragma unroll
  for (int jp = 0; jp < 4; ++jp) {
    float c[MT][2][4];
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int e = 0; e < 4; ++e) c[m][0][e] = c[m][1][e] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      uint32_t b0, b1, b2, b3;  // (n-tile 2jp: k lo, k hi), (n-tile 2jp+1: k lo, k hi)
      ldsm4(saddr(W + (16 * jp + r + 8 * (q >> 1)) * kRS + 16 * kt + 8 * (q & 1)), b0, b1, b2, b3);
#pragma unroll
      for (int m = 0; m < MT; ++m) {
        mma(c[m][0], a[m][kt], b0, b1);
        mma(c[m][1], a[m][kt], b2, b3);
      }
    }
#pragma unroll
    for (int m = 0; m < MT; ++m) {
      h[m][jp][0] = pack2(relu(c[m][0][0]), relu(c[m][0][1]));
      h[m][jp][1] = pack2(relu(c[m][0][2]), relu(c[m][0][3]));
      h[m][jp][2] = pack2(relu(c[m][1][0]), relu(c[m][1][1]));
      h[m][jp][3] = pack2(relu(c[m][1][2]), relu(c[m][1][3]));
    }
  }
}

// outputs 0..7 of the 16-row output layer (only 0..2 are live)
template <int MT>
__device__ __forceinline__ void layer_out(const bf16* W5, int lane, const uint32_t (&h)[MT][4][4], float (&o)[MT][4]) {
  const int q = lane >> 3, r = lane & 7;
#pragma unroll
  for (int m = 0; m < MT; ++m) o[m][0] = o[m][1] = o[m][2] = o[m][3] = 0.0f;
#pragma unroll
  for (int kp = 0; kp < 2; ++kp) {
    uint32_t b0, b1, b2, b3;  // k-tiles 2kp (lo, hi), 2kp+1 (lo, hi)
    ldsm4(saddr(W5 + r * kRS + 32 * kp + 8 * q), b0, b1, b2, b3);
#pragma unroll
    for (int m = 0; m < MT; ++m) {
      mma(o[m], h[m][2 * kp], b0, b1);
      mma(o[m], h[m][2 * kp + 1], b2, b3);
    }
  }
}

template <int MT>
__device__ __forceinline__ void mlp_forward(const bf16* Ws, const bf16* rows, int lane, float (&o)[MT][4]) {
  uint32_t a[MT][4][4], h[MT][4][4];
#pragma unroll
  for (int m = 0; m < MT; ++m) load_a(rows, 16 * m, lane, a[m]);
  layer_fwd<MT>(Ws, lane, a, h);
  layer_fwd<MT>(Ws + 64 * kRS, lane, h, a);
  layer_fwd<MT>(Ws + 128 * kRS, lane, a, h);
  layer_fwd<MT>(Ws + 192 * kRS, lane, h, a);
  layer_fwd<MT>(Ws + 256 * kRS, lane, a, h);
  layer_out<MT>(Ws + 320 * kRS, lane, h, o);
}

// outputs of a 32-row warp tile into out[32][4] (floats, column 3 unused)
__device__ __forceinline__ void store_outputs(float* out, const float (&o)[2][4], int lane) {
  const int g = lane >> 2, t = lane & 3;
  if (t < 2) {
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      out[(16 * m + g) * 4 + 2 * t] = o[m][0];
      out[(16 * m + g) * 4 + 2 * t + 1] = o[m][1];
      out[(16 * m + g + 8) * 4 + 2 * t] = o[m][2];
      out[(16 * m + g + 8) * 4 + 2 * t + 1] = o[m][3];
    }
  }
}

__device__ __forceinline__ void load_weights(bf16* Ws, const bf16* __restrict__ W) {
  for (int i = threadIdx.x; i < kMlpRows * 8; i += blockDim.x)
    *reinterpret_cast<uint4*>(Ws + (i >> 3) * kRS + 8 * (i & 7)) = __ldg(reinterpret_cast<const uint4*>(W) + i);
}

// 64 features of a vertex, packed to bf16, into one shared row
__device__ __forceinline__ void encode_row(const CacheFeatures& v, const CacheBounds& b, bf16* row) {
  float f[64];
  cache_encode(v, b, f);
  uint4* dst = reinterpret_cast<uint4*>(row);
#pragma unroll
  for (int c = 0; c < 8; ++c)
    dst[c] = make_uint4(pack2(f[8 * c], f[8 * c + 1]), pack2(f[8 * c + 2], f[8 * c + 3]),
                        pack2(f[8 * c + 4], f[8 * c + 5]), pack2(f[8 * c + 6], f[8 * c + 7]));
}

// ---- inference ---------------------------------------------------------------------------

// rows of encoded inputs (bf16 [n][64]) -> out [n][3]
__global__ void __launch_bounds__(256, 2) k_cache_infer_rows(const bf16* __restrict__ W, const bf16* __restrict__ X,
                                                             uint32_t n, float* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  bf16* Ws = reinterpret_cast<bf16*>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  bf16* rows = Ws + kMlpRows * kRS + warp * 32 * kRS;
  load_weights(Ws, W);
  __syncthreads();
  const uint32_t groups = (n + 31) / 32;
  for (uint32_t grp = blockIdx.x * kInferWarps + warp; grp < groups; grp += gridDim.x * kInferWarps) {
    const uint32_t r0 = grp * 32;
    for (int k = lane; k < 256; k += 32) {
      const uint32_t row = r0 + (k >> 3);
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (row < n) v = __ldg(reinterpret_cast<const uint4*>(X + (size_t)row * 64) + (k & 7));
      *reinterpret_cast<uint4*>(rows + (k >> 3) * kRS + 8 * (k & 7)) = v;
    }
    __syncwarp();
    float o[2][4];
    mlp_forward<2>(Ws, rows, lane, o);
    __syncwarp();
    float* outs = reinterpret_cast<float*>(rows);
    store_outputs(outs, o, lane);
    __syncwarp();
    const uint32_t row = r0 + lane;
    if (row < n) {
      out[3 * (size_t)row] = outs[4 * lane];
      out[3 * (size_t)row + 1] = outs[4 * lane + 1];
      out[3 * (size_t)row + 2] = outs[4 * lane + 2];
    }
    __syncwarp();
  }
}

// cache queries of a wave: image queries add T * L to their path's radiance, tail queries
// set the radiance that closes their training path's chain
__global__ void __launch_bounds__(256, 2) k_cache_infer_queries(const bf16* __restrict__ W,
                                                                const CacheQuery* __restrict__ queries,
                                                                const uint32_t* __restrict__ n_queries,
                                                                uint32_t max_queries, CacheBounds bounds,
                                                                float4* __restrict__ radiance,
                                                                float4* __restrict__ tail) {
  extern __shared__ __align__(16) unsigned char smem[];
  bf16* Ws = reinterpret_cast<bf16*>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  bf16* rows = Ws + kMlpRows * kRS + warp * 32 * kRS;
  load_weights(Ws, W);
  __syncthreads();
  const uint32_t n = min(*n_queries, max_queries);
  const uint32_t groups = (n + 31) / 32;
  for (uint32_t grp = blockIdx.x * kInferWarps + warp; grp < groups; grp += gridDim.x * kInferWarps) {
    const uint32_t row = grp * 32 + lane;
    uint32_t tag = 0;
    float4 T = make_float4(0.f, 0.f, 0.f, 0.f);
    V3 fac{0.0f, 0.0f, 0.0f};
    if (row < n) {
      const CacheQuery q = queries[row];
      tag = q.f.tag;
      T = q.T;
      fac = cache_factor(q.f);
      encode_row(q.f, bounds, rows + lane * kRS);
    } else {
      uint4* dst = reinterpret_cast<uint4*>(rows + lane * kRS);
#pragma unroll
      for (int c = 0; c < 8; ++c) dst[c] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncwarp();
    float o[2][4];
    mlp_forward<2>(Ws, rows, lane, o);
    __syncwarp();
    float* outs = reinterpret_cast<float*>(rows);
    store_outputs(outs, o, lane);
    __syncwarp();
    if (row < n) {
      const V3 L{fmaxf(outs[4 * lane], 0.0f) * fac.x, fmaxf(outs[4 * lane + 1], 0.0f) * fac.y,
                 fmaxf(outs[4 * lane + 2], 0.0f) * fac.z};
      if (tag & nb::kCacheTailBit) {
        tail[tag & ~nb::kCacheTailBit] = make_float4(L.x, L.y, L.z, 0.0f);
      } else {
        float4 c = radiance[tag];
        c.x = c.x + T.x * L.x;
        c.y = c.y + T.y * L.y;
        c.z = c.z + T.z * L.z;
        radiance[tag] = c;
      }
    }
    __syncwarp();
  }
}

// ---- inference on the 5th-generation tensor cores (tcgen05) ------------------------------
//
// A CTA is two warpgroups of 4 warps; each warpgroup keeps two groups of 128 rows in flight,
// so an SM (2 CTAs) runs 8 independent layer chains and one chain's MMA round trip hides
// behind the others' epilogues.  The MMA operands sit in shared memory in the no-swizzle
// K-major canonical layout of tcgen05.mma: 8-row x 16-byte core matrices of 128 B, the core
// matrices of one 8-row group along K contiguous (leading byte offset 128 B), 8-row groups
// 1 KB apart (stride byte offset 1 KB).  Each group's accumulator (128 lanes x 64 FP32 columns)
// lives in tensor memory.  Per layer and group the warpgroup's first thread issues four
// K = 16 MMAs and commits them to the group's mbarrier; once they completed, the warps read
// their 32 accumulator rows (tcgen05.ld), apply ReLU, pack to BF16 and overwrite the group's
// operand with the next layer's (the MMA that read it is done).  The warp-collective
// (.sync.aligned) tcgen05 instructions - alloc, ld, dealloc - run on whole converged warps.
// Waits poll the mbarrier a bounded number of times: on a timeout the warpgroup raises
// kStatusCacheTimeout (bits 16.. = 1 + the layer it waited for) and stops; the CTA frees its
// TMEM before it exits.

constexpr int kTcRows = 128;                                   // rows per group (= TMEM lanes)
constexpr int kTcThreads = 256;                                // two warpgroups
constexpr uint32_t kTcCols = 256;                              // TMEM columns: 64 per group, 4 groups
constexpr uint32_t kTcLayerBytes = 8192;                       // one 64 x 64 layer, canonical
constexpr size_t kTcWBytes = 5 * kTcLayerBytes + 2048;         // + the 16 x 64 output layer
constexpr size_t kTcActBytes = (size_t)kTcRows * 64 * sizeof(bf16);  // 16 KB per group operand
constexpr size_t kTcSmem = kTcWBytes + 4 * kTcActBytes;        // 108,544 B (2 CTAs per SM)
constexpr uint32_t kTcWaitLimit = 1u << 22;                    // mbarrier polls per wait
constexpr uint32_t kStatusCacheTimeout = 1u << 8;

// byte offset of element (row, k) of a canonical K-major operand (rows x 64)
__host__ __device__ __forceinline__ uint32_t canon_off(uint32_t row, uint32_t k) {
  return (row >> 3) * 1024u + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// shared-memory matrix descriptor: start address, LBO 128 B, SBO 1024 B, descriptor version 1,
// no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(1024u >> 4) << 32) |
         (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}
// polls (non-blocking test_wait) until the phase of the given parity completed
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (uint32_t k = 0; k < kTcWaitLimit; ++k) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// barrier over the 128 threads of one warpgroup (named barrier 1 + wg); returns the OR of pred
__device__ __forceinline__ bool wg_barrier_or(uint32_t wg, bool pred) {
  uint32_t out;
  asm volatile(
      "{\n\t.reg .pred q, p;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, %2, 128, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(out)
      : "r"((uint32_t)pred), "r"(1u + wg)
      : "memory");
  return out != 0;
}
// 16 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  __syncwarp();  // warp-collective: lanes may leave the mbarrier poll at different times
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n\t"
               "tcgen05.wait::ld.sync.aligned;\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 64 consecutive FP32 accumulator columns of this thread's TMEM lane: one load, one wait
// (four 16-column loads each waited for would take four round trips to tensor memory)
__device__ __forceinline__ void tc_ld64(uint32_t taddr, float (&v)[64]) {
  uint32_t r[64];
  __syncwarp();  // warp-collective
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];\n\t"
               "tcgen05.wait::ld.sync.aligned;\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

// kQueries: the rows are a wave's cache queries (encoded here; results go to radiance / tail);
// else rows of encoded inputs X (bf16 [n][64]) with results in out[n][3].
template <bool kQueries>
__global__ void __launch_bounds__(kTcThreads, 2) k_cache_infer_tc(const bf16* __restrict__ W,
                                                                  const bf16* __restrict__ X,
                                                                  const CacheQuery* __restrict__ queries,
                                                                  const uint32_t* __restrict__ n_dev, uint32_t n_host,
                                                                  CacheBounds bounds, float* __restrict__ out,
                                                                  float4* __restrict__ radiance,
                                                                  float4* __restrict__ tail,
                                                                  uint32_t* __restrict__ status) {
  extern __shared__ __align__(128) unsigned char smem_tc[];
  __shared__ __align__(8) uint64_t mbar_slot[4];
  __shared__ uint32_t tmem_slot;
  unsigned char* Wc = smem_tc;
  const uint32_t warp = threadIdx.x >> 5, wg = threadIdx.x >> 7, tid = threadIdx.x & 127u;
  // group j of warpgroup wg: operand at act + j * kTcActBytes, mbarrier mbar + 8 j, accumulator
  // columns 128 wg + 64 j
  unsigned char* act = smem_tc + kTcWBytes + 2u * wg * kTcActBytes;
  const uint32_t mbar = saddr(&mbar_slot[2 * wg]);
  const uint32_t n = kQueries ? min(*n_dev, n_host) : n_host;

  // weights into the canonical layout: row r of layer l = global row 64 l + r.  Consecutive
  // threads take consecutive rows of one 16-byte column chunk, so each quarter-warp stores 128
  // contiguous bytes (a thread per chunk of one row would hit one bank group 8 times)
  for (uint32_t i = threadIdx.x; i < (uint32_t)kMlpRows * 8u; i += blockDim.x) {
    const uint32_t row = i % (uint32_t)kMlpRows, c = i / (uint32_t)kMlpRows, l = row >> 6, r = row & 63u;
    *reinterpret_cast<uint4*>(Wc + l * kTcLayerBytes + canon_off(r, 8u * c)) =
        __ldg(reinterpret_cast<const uint4*>(W) + 8u * row + c);
  }
  if (threadIdx.x == 0) {
    for (uint32_t k = 0; k < 4; ++k)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(&mbar_slot[k])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    __syncwarp();  // alloc is .sync.aligned: the whole warp, converged
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(&tmem_slot)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot + 128u * wg;            // this warpgroup's two accumulators
  const uint32_t lane_base = (32u * (warp & 3u)) << 16;  // this warp's 32 TMEM lanes
  uint32_t phase[2] = {0u, 0u};
  uint32_t fail_layer = 0;
  bool failed = false;

  // layer l of group j: four K = 16 MMAs into the group's 64 accumulator columns
  auto issue = [&](uint32_t j, int l) {
    const uint32_t a_base = saddr(act + j * kTcActBytes);
    const uint32_t b_base = saddr(Wc + l * kTcLayerBytes);
    const uint32_t idesc = tc_idesc(kTcRows, l < 5 ? 64u : 16u);
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k)
      tc_mma(tmem + 64u * j, tc_desc(a_base + 256u * k), tc_desc(b_base + 256u * k), idesc, k);
    tc_commit(mbar + 8u * j);
  };

  const uint32_t groups = (n + kTcRows - 1) / kTcRows;
  // round q covers row groups 4 q .. 4 q + 3 (warpgroup wg takes 4 q + 2 wg + j); rounds are
  // dealt to the CTAs round-robin
  for (uint32_t q = blockIdx.x; 4u * q + 2u * wg < groups && !failed; q += gridDim.x) {
    uint32_t tag[2] = {0u, 0u};
    float4 T[2];
    V3 fac[2];
#pragma unroll
    for (uint32_t j = 0; j < 2; ++j) {
      const uint32_t row = (4u * q + 2u * wg + j) * kTcRows + tid;
      T[j] = make_float4(0.f, 0.f, 0.f, 0.f);
      fac[j] = V3{0.0f, 0.0f, 0.0f};
      uint4 ch[8];
      if (row < n) {
        if (kQueries) {
          const CacheQuery qr = queries[row];
          tag[j] = qr.f.tag;
          T[j] = qr.T;
          fac[j] = cache_factor(qr.f);
          float f[64];
          cache_encode(qr.f, bounds, f);
#pragma unroll
          for (int c = 0; c < 8; ++c)
            ch[c] = make_uint4(pack2(f[8 * c], f[8 * c + 1]), pack2(f[8 * c + 2], f[8 * c + 3]),
                               pack2(f[8 * c + 4], f[8 * c + 5]), pack2(f[8 * c + 6], f[8 * c + 7]));
        } else {
#pragma unroll
          for (int c = 0; c < 8; ++c) ch[c] = __ldg(reinterpret_cast<const uint4*>(X + (size_t)row * 64) + c);
        }
      } else {
#pragma unroll
        for (int c = 0; c < 8; ++c) ch[c] = make_uint4(0u, 0u, 0u, 0u);
      }
      unsigned char* a = act + j * kTcActBytes;
#pragma unroll
      for (int c = 0; c < 8; ++c) *reinterpret_cast<uint4*>(a + canon_off(tid, 8u * c)) = ch[c];
    }
    fence_async_smem();
    tc_fence_before();
    wg_barrier_or(wg, false);
    tc_fence_after();
    if (tid == 0) {
      issue(0, 0);
      issue(1, 0);
    }
#pragma unroll 1
    for (int l = 0; l < 6 && !failed; ++l) {
#pragma unroll
      for (uint32_t j = 0; j < 2; ++j) {
        const bool ok = mbar_wait(mbar + 8u * j, phase[j]);
        phase[j] ^= 1u;
        tc_fence_after();
        const uint32_t t_row = tmem + 64u * j + lane_base;
        if (l < 5) {
          unsigned char* a = act + j * kTcActBytes;  // its MMA is complete: overwrite in place
          float v[64];
          tc_ld64(t_row, v);
#pragma unroll
          for (int c = 0; c < 8; ++c)
            *reinterpret_cast<uint4*>(a + canon_off(tid, 8u * c)) =
                make_uint4(pack2(relu(v[8 * c]), relu(v[8 * c + 1])), pack2(relu(v[8 * c + 2]), relu(v[8 * c + 3])),
                           pack2(relu(v[8 * c + 4]), relu(v[8 * c + 5])), pack2(relu(v[8 * c + 6]), relu(v[8 * c + 7])));
          fence_async_smem();
        } else {
          // every lane of every warp runs the (warp-collective) accumulator load; only rows
          // of the batch use it
          float v[16];
          tc_ld16(t_row, v);
          const uint32_t row = (4u * q + 2u * wg + j) * kTcRows + tid;
          if (!ok || row >= n) {
          } else if (kQueries) {
            const V3 L{fmaxf(v[0], 0.0f) * fac[j].x, fmaxf(v[1], 0.0f) * fac[j].y, fmaxf(v[2], 0.0f) * fac[j].z};
            if (tag[j] & nb::kCacheTailBit) {
              tail[tag[j] & ~nb::kCacheTailBit] = make_float4(L.x, L.y, L.z, 0.0f);
            } else {
              float4 c = radiance[tag[j]];
              c.x = c.x + T[j].x * L.x;
              c.y = c.y + T[j].y * L.y;
              c.z = c.z + T[j].z * L.z;
              radiance[tag[j]] = c;
            }
          } else {
            out[3 * (size_t)row] = v[0];
            out[3 * (size_t)row + 1] = v[1];
            out[3 * (size_t)row + 2] = v[2];
          }
        }
        tc_fence_before();
        failed = wg_barrier_or(wg, !ok);
        tc_fence_after();
        if (failed) {
          fail_layer = (uint32_t)l + 1u;
          break;
        }
        if (l < 5 && tid == 0) issue(j, l + 1);
      }
    }
  }
  if (failed && tid == 0) {
    atomicOr(status, kStatusCacheTimeout | (fail_layer << 16));
    // give outstanding MMAs a bounded chance to finish before the memory is released
    mbar_wait(mbar, phase[0] ^ 1u);
    mbar_wait(mbar + 8u, phase[1] ^ 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();  // dealloc is .sync.aligned
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem_slot), "r"(kTcCols)
                 : "memory");
  }
}

// ---- training ----------------------------------------------------------------------------

// bf16 pairs of a C-fragment-derived A fragment (16 rows from r0) into shared rows
__device__ __forceinline__ void store_frag(bf16* rows, int r0, int lane, const uint32_t (&h)[4][4]) {
  const int g = lane >> 2, t = lane & 3;
  uint32_t* base = reinterpret_cast<uint32_t*>(rows);
#pragma unroll
  for (int jp = 0; jp < 4; ++jp) {
    base[((r0 + g) * kRS + 16 * jp + 2 * t) >> 1] = h[jp][0];
    base[((r0 + g + 8) * kRS + 16 * jp + 2 * t) >> 1] = h[jp][1];
    base[((r0 + g) * kRS + 16 * jp + 8 + 2 * t) >> 1] = h[jp][2];
    base[((r0 + g + 8) * kRS + 16 * jp + 8 + 2 * t) >> 1] = h[jp][3];
  }
}
__device__ __forceinline__ uint32_t ld_pair(const bf16* rows, int row, int col) {
  return reinterpret_cast<const uint32_t*>(rows)[(row * kRS + col) >> 1];
}

// Gradient of the mean relative L2 loss of rows [row0, min(row0 + rows_per_step, n)) times
// 3 * rows: each CTA writes the FP32 partial weight gradient of its 128 rows (unscaled) and its
// partial loss.  Rows whose target .w is 0 are skipped (invalid target).  clip > 0 bounds the
// loss gradient per record and channel.
__global__ void __launch_bounds__(256, 1) k_cache_grad(const bf16* __restrict__ W, const bf16* __restrict__ X,
                                                       const float4* __restrict__ Y,
                                                       const uint32_t* __restrict__ n_dev, uint32_t n_host,
                                                       uint32_t row0, uint32_t rows_per_step, float clip,
                                                       float* __restrict__ part_dw, float* __restrict__ part_loss) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float warp_loss[8];
  bf16* Ws = reinterpret_cast<bf16*>(smem);
  bf16* Hs = Ws + kMlpRows * kRS;           // H_0 (inputs) .. H_5, 128 rows each
  bf16* dZs = Hs + 6 * kGradRows * kRS;     // two 128-row buffers of output gradients
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3, q = lane >> 3, r = lane & 7;
  const uint32_t n_total = n_dev ? *n_dev : n_host;
  const uint32_t end = n_total > row0 ? row0 + min(n_total - row0, rows_per_step) : row0;
  const uint32_t cta0 = row0 + blockIdx.x * kGradRows;
  float* dw = part_dw + (size_t)blockIdx.x * kMlpParams;

  load_weights(Ws, W);
  for (int k = threadIdx.x; k < kGradRows * 8; k += blockDim.x) {
    const uint32_t row = cta0 + (k >> 3);
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (row < end) v = __ldg(reinterpret_cast<const uint4*>(X + (size_t)row * 64) + (k & 7));
    *reinterpret_cast<uint4*>(Hs + (k >> 3) * kRS + 8 * (k & 7)) = v;
  }
  __syncthreads();

  // forward over this warp's 16 rows; H_1..H_5 kept for the backward pass
  const int wr = 16 * warp;
  uint32_t a[1][4][4], h[1][4][4];
  load_a(Hs, wr, lane, a[0]);
#pragma unroll
  for (int l = 0; l < 5; ++l) {
    layer_fwd<1>(Ws + 64 * l * kRS, lane, a, h);
    store_frag(Hs + (l + 1) * kGradRows * kRS, wr, lane, h[0]);
#pragma unroll
    for (int kt = 0; kt < 4; ++kt)
#pragma unroll
      for (int e = 0; e < 4; ++e) a[0][kt][e] = h[0][kt][e];
  }
  float o[1][4];
  layer_out<1>(Ws + 320 * kRS, lane, a, o);

  // dL/dp = 2 (p - y) / (p^2 + 0.01), denominator treated as a constant
  float lsum = 0.0f, gz[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const uint32_t row = cta0 + wr + g + (e >= 2 ? 8 : 0);
    const int col = 2 * t + (e & 1);
    gz[e] = 0.0f;
    if (col < 3 && row < end) {
      const float4 y4 = __ldg(Y + row);
      if (y4.w != 0.0f) {
        const float y = col == 0 ? y4.x : (col == 1 ? y4.y : y4.z);
        const float p = o[0][e];
        const float d = p - y;
        const float den = p * p + 0.01f;
        lsum += d * d / den;
        gz[e] = 2.0f * d / den;
        if (clip > 0.0f) gz[e] = fminf(fmaxf(gz[e], -clip), clip);
      }
    }
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) lsum += __shfl_xor_sync(0xFFFFFFFFu, lsum, s);
  if (lane == 0) warp_loss[warp] = lsum;

  // ---- layer 5 (16 x 64): dZ6 has one k-tile (outputs 0..15, 3..15 zero)
  uint32_t dz6[4] = {pack2(gz[0], gz[1]), pack2(gz[2], gz[3]), 0u, 0u};
  uint32_t dz[4][4];
  {
    bf16* D = dZs + kGradRows * kRS;  // buffer 1
    uint32_t* Db = reinterpret_cast<uint32_t*>(D);
    Db[((wr + g) * kRS + 2 * t) >> 1] = dz6[0];
    Db[((wr + g + 8) * kRS + 2 * t) >> 1] = dz6[1];
    Db[((wr + g) * kRS + 8 + 2 * t) >> 1] = 0u;
    Db[((wr + g + 8) * kRS + 8 + 2 * t) >> 1] = 0u;
    const bf16* H5 = Hs + 5 * kGradRows * kRS;
    // dH5 = dZ6 W5, gated by H5 > 0
#pragma unroll
    for (int jp = 0; jp < 4; ++jp) {
      float c[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
      uint32_t b0, b1, b2, b3;
      ldsm4t(saddr(Ws + (320 + r + 8 * (q & 1)) * kRS + 16 * jp + 8 * (q >> 1)), b0, b1, b2, b3);
      mma(c[0], dz6, b0, b1);
      mma(c[1], dz6, b2, b3);
      const uint32_t m00 = ld_pair(H5, wr + g, 16 * jp + 2 * t), m01 = ld_pair(H5, wr + g + 8, 16 * jp + 2 * t);
      const uint32_t m10 = ld_pair(H5, wr + g, 16 * jp + 8 + 2 * t),
                     m11 = ld_pair(H5, wr + g + 8, 16 * jp + 8 + 2 * t);
      dz[jp][0] = pack2(gate_lo(c[0][0], m00), gate_hi(c[0][1], m00));
      dz[jp][1] = pack2(gate_lo(c[0][2], m01), gate_hi(c[0][3], m01));
      dz[jp][2] = pack2(gate_lo(c[1][0], m10), gate_hi(c[1][1], m10));
      dz[jp][3] = pack2(gate_lo(c[1][2], m11), gate_hi(c[1][3], m11));
    }
    __syncthreads();
    // dW5 = dZ6^T H5 over the 128 rows: warp w takes inputs 8w..8w+7
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kp = 0; kp < 4; ++kp) {
      uint32_t b0, b1, b2, b3;  // k-tiles 2kp, 2kp+1 of H5 columns 8w..
      ldsm4t(saddr(H5 + (32 * kp + r + 8 * q) * kRS + 8 * warp), b0, b1, b2, b3);
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const int kt = 2 * kp + s;
        uint32_t av[4];
        ldsm4t(saddr(D + (16 * kt + r + 8 * (q >> 1)) * kRS + 8 * (q & 1)), av[0], av[1], av[2], av[3]);
        mma(acc, av, s ? b2 : b0, s ? b3 : b1);
      }
    }
    float* d5 = dw + 5 * 4096;
    *reinterpret_cast<float2*>(d5 + g * 64 + 8 * warp + 2 * t) = make_float2(acc[0], acc[1]);
    *reinterpret_cast<float2*>(d5 + (g + 8) * 64 + 8 * warp + 2 * t) = make_float2(acc[2], acc[3]);
  }

  // ---- layers 4..0 (64 x 64)
#pragma unroll 1
  for (int l = 4; l >= 0; --l) {
    bf16* D = dZs + (l & 1) * kGradRows * kRS;
    store_frag(D, wr, lane, dz);
    const bf16* Hl = Hs + l * kGradRows * kRS;
    uint32_t dzn[4][4];
    if (l >= 1) {
      const bf16* Wl = Ws + 64 * l * kRS;
#pragma unroll
      for (int jp = 0; jp < 4; ++jp) {
        float c[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
          uint32_t b0, b1, b2, b3;
          ldsm4t(saddr(Wl + (16 * kt + r + 8 * (q & 1)) * kRS + 16 * jp + 8 * (q >> 1)), b0, b1, b2, b3);
          mma(c[0], dz[kt], b0, b1);
          mma(c[1], dz[kt], b2, b3);
        }
        const uint32_t m00 = ld_pair(Hl, wr + g, 16 * jp + 2 * t), m01 = ld_pair(Hl, wr + g + 8, 16 * jp + 2 * t);
        const uint32_t m10 = ld_pair(Hl, wr + g, 16 * jp + 8 + 2 * t),
                       m11 = ld_pair(Hl, wr + g + 8, 16 * jp + 8 + 2 * t);
        dzn[jp][0] = pack2(gate_lo(c[0][0], m00), gate_hi(c[0][1], m00));
        dzn[jp][1] = pack2(gate_lo(c[0][2], m01), gate_hi(c[0][3], m01));
        dzn[jp][2] = pack2(gate_lo(c[1][0], m10), gate_hi(c[1][1], m10));
        dzn[jp][3] = pack2(gate_lo(c[1][2], m11), gate_hi(c[1][3], m11));
      }
    }
    __syncthreads();
    // dW_l = dZ_{l+1}^T H_l: warp w takes outputs 16 (w >> 1).., inputs 32 (w & 1)..
    const int mt = warp >> 1, nb0 = 4 * (warp & 1);
    float acc[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < 8; ++kt) {
      uint32_t av[4];
      ldsm4t(saddr(D + (16 * kt + r + 8 * (q >> 1)) * kRS + 16 * mt + 8 * (q & 1)), av[0], av[1], av[2], av[3]);
#pragma unroll
      for (int np = 0; np < 2; ++np) {
        const int j = nb0 + 2 * np;
        uint32_t b0, b1, b2, b3;
        ldsm4t(saddr(Hl + (16 * kt + r + 8 * (q & 1)) * kRS + 8 * (j + (q >> 1))), b0, b1, b2, b3);
        mma(acc[2 * np], av, b0, b1);
        mma(acc[2 * np + 1], av, b2, b3);
      }
    }
    float* dl = dw + l * 4096;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = 8 * (nb0 + j) + 2 * t;
      *reinterpret_cast<float2*>(dl + (16 * mt + g) * 64 + col) = make_float2(acc[j][0], acc[j][1]);
      *reinterpret_cast<float2*>(dl + (16 * mt + g + 8) * 64 + col) = make_float2(acc[j][2], acc[j][3]);
    }
    if (l >= 1) {
#pragma unroll
      for (int jp = 0; jp < 4; ++jp)
#pragma unroll
        for (int e = 0; e < 4; ++e) dz[jp][e] = dzn[jp][e];
    }
  }
  // padding rows 16..: W_5 has rows 0..15 only; nothing else to clear
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int w = 0; w < 8; ++w) s += warp_loss[w];
    part_loss[blockIdx.x] = s;
  }
}

// ---- training on the 5th-generation tensor cores (tcgen05) -------------------------------
//
// One warpgroup per 128-row group (thread = row = tensor-memory lane), every GEMM a
// tcgen05.mma with M = 128 and FP32 accumulators in tensor memory, issued by one thread and
// committed to one mbarrier:
//   forward    Z_{l+1} = H_l W_l^T          A = H_l (rows x in, K-major), B = W_l (out x in)
//   backward   dH_l = dZ_{l+1} W_l           A = dZ_{l+1} (rows x out), B = W_l^T (in x out)
//   weights    dW_l = dZ_{l+1}^T H_l         A = dZ_{l+1}, B = H_l, both read through MN-major
//                                            descriptors (M = out, N = in, K = the 128 rows)
// so the activations H_0..H_5 and the output gradient are stored once, row-major in the
// canonical layout, and serve both as K-major operands (rows x features) and as MN-major ones
// (features x rows).  M is 128 for the weight GEMMs too: rows out >= 64 (>= 16 for the output
// layer) read whatever follows in shared memory and land in accumulator lanes nobody reads.
// The backward GEMM of a layer and its weight GEMM read the same dZ and are issued together.
// Rounding points are those of k_cache_grad (BF16 activations and output gradients, FP32
// accumulation), and the partials have its layout, so k_cache_adam serves both.
constexpr uint32_t kTrRows = 128;
constexpr size_t kTrWf = 5 * 8192 + 2048;              // W_0..W_4 (64 x 64), W_5 (16 x 64)
constexpr size_t kTrWb = 4 * 8192 + 2048;              // W_1^T..W_4^T (64 x 64), W_5^T (64 x 16)
constexpr size_t kTrAct = (size_t)kTrRows * 64 * 2;    // one 128 x 64 BF16 tile
// 128 x 16 output gradient (4 KB) + slack: the padded weight GEMMs read up to ~29 KB past the
// start of dZ and ~7.5 KB past dZ6, all inside this allocation
constexpr size_t kTrDz6 = 14336;
constexpr size_t kTrSmem = kTrWf + kTrWb + 7 * kTrAct + kTrDz6;  // H_0..H_5, dZ: 206,848 B
constexpr uint32_t kTrCols = 256;                      // TMEM: [0, 64) layer GEMMs, [64, 192) two weight-GEMM buffers
constexpr size_t kTrStage = kTrWf + kTrWb;             // the weight image the training kernel copies in

// Where parameter p (rows [out][in] per layer) sits in the training kernel's weight image:
// *f in the forward operands W_l (out x in), *b in the backward ones W_l^T (in x out), or
// 0xFFFFFFFF for the first layer, whose transpose no GEMM needs.  Adam keeps the image current.
__host__ __device__ __forceinline__ void stage_offsets(uint32_t p, uint32_t* f, uint32_t* b) {
  const uint32_t l = p >> 12, r = p & 4095u, out = r >> 6, in = r & 63u;
  *f = l * 8192u + canon_off(out, in);
  if (l == 0) *b = 0xFFFFFFFFu;
  else if (l < 5) *b = (uint32_t)kTrWf + (l - 1u) * 8192u + canon_off(in, out);
  else *b = (uint32_t)kTrWf + 4u * 8192u + (in >> 3) * 256u + (out >> 3) * 128u + (in & 7u) * 16u + (out & 7u) * 2u;
}

// shared-memory matrix descriptor with explicit leading / stride byte offsets, no swizzle
__device__ __forceinline__ uint64_t tc_desc2(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// kind::f16 instruction descriptor with the operands' major-ness (bit 15: A MN-major, 16: B)
__host__ __device__ constexpr uint32_t tc_idesc2(uint32_t M, uint32_t N, bool a_mn, bool b_mn) {
  return tc_idesc(M, N) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}
// A row-major canonical tile (8-feature chunks of 16 B, 8-row groups G bytes apart) read as an
// MN-major operand (features x rows): leading byte offset G (between 8-row groups, along K),
// stride byte offset 128 B (between 8-feature chunks, along M or N).

__global__ void __launch_bounds__(128, 1) k_cache_grad_tc(const unsigned char* __restrict__ stage,
                                                          const bf16* __restrict__ X,
                                                          const float4* __restrict__ Y,
                                                          const uint32_t* __restrict__ n_dev, uint32_t n_host,
                                                          uint32_t row0, uint32_t rows_per_step, float clip,
                                                          float* __restrict__ part_dw, float* __restrict__ part_loss,
                                                          uint32_t* __restrict__ status) {
  extern __shared__ __align__(128) unsigned char smem_tr[];
  __shared__ __align__(8) uint64_t mbar_slot, copy_slot;
  __shared__ uint32_t tmem_slot;
  __shared__ float warp_loss[4];
  unsigned char* Wf = smem_tr;
  unsigned char* Wb = Wf + kTrWf;
  unsigned char* H = Wb + kTrWb;          // H_l at H + l * kTrAct
  unsigned char* dZ = H + 6 * kTrAct;     // 128 x 64 output gradient of the layer being done
  unsigned char* dZ6 = dZ + kTrAct;       // 128 x 16 gradient of the output layer
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  const uint32_t mbar = saddr(&mbar_slot);
  const uint32_t n_total = n_dev ? *n_dev : n_host;
  const uint32_t end = n_total > row0 ? row0 + min(n_total - row0, rows_per_step) : row0;
  const uint32_t row = row0 + blockIdx.x * kTrRows + tid;
  float* dw = part_dw + (size_t)blockIdx.x * kMlpParams;

  // the weight image (W_l and W_l^T already in the canonical layout): bulk asynchronous
  // copies of 16 KB or less, completing on copy_slot
  const uint32_t copy_bar = saddr(&copy_slot);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(copy_bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(copy_bar), "r"((uint32_t)kTrStage)
                 : "memory");
    for (uint32_t off = 0; off < (uint32_t)kTrStage; off += 16384u) {
      const uint32_t bytes = min(16384u, (uint32_t)kTrStage - off);
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                       saddr(Wf + off)),
                   "l"(stage + off), "r"(bytes), "r"(copy_bar)
                   : "memory");
    }
  }
  // this thread's input row
  {
    const bool live = row < end;
#pragma unroll
    for (uint32_t c = 0; c < 8; ++c) {
      const uint4 v = live ? __ldg(reinterpret_cast<const uint4*>(X + (size_t)row * 64) + c) : make_uint4(0u, 0u, 0u, 0u);
      *reinterpret_cast<uint4*>(H + canon_off(tid, 8u * c)) = v;
    }
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(&tmem_slot)),
                 "r"(kTrCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const bool staged = mbar_wait(copy_bar, 0u);  // the weight image has landed
  const uint32_t tmem = tmem_slot, lane_base = (32u * warp) << 16;
  const uint32_t d_layer = tmem;  // weight GEMMs alternate between tmem + 64 and tmem + 128
  uint32_t phase = 0;
  bool failed = false;
  uint32_t fail_round = 0, round = 0;

  // waits for the committed MMAs; every thread learns whether any wait gave up
  auto wait_all = [&]() {
    const bool ok = mbar_wait(mbar, phase);
    phase ^= 1u;
    ++round;
    tc_fence_after();
    return ok;
  };
  // ends a round of shared-memory writes that the next MMAs read
  auto publish = [&](bool bad) {
    fence_async_smem();
    tc_fence_before();
    const bool any_bad = __syncthreads_or(bad ? 1 : 0) != 0;
    tc_fence_after();
    if (any_bad && !failed) {
      failed = true;
      fail_round = round;
    }
  };
  publish(!staged);

  // ---- forward: H_1..H_5, then the output layer
  for (int l = 0; l < 6 && !failed; ++l) {
    if (tid == 0) {
      const uint32_t a = saddr(H + l * kTrAct), b = saddr(Wf + l * 8192u);
      const uint32_t idesc = tc_idesc(kTrRows, l < 5 ? 64u : 16u);
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k)
        tc_mma(d_layer, tc_desc2(a + 256u * k, 128u, 1024u), tc_desc2(b + 256u * k, 128u, 1024u), idesc, k);
      tc_commit(mbar);
    }
    const bool ok = wait_all();
    if (l < 5) {
      unsigned char* h = H + (l + 1) * kTrAct;
      float v[64];
      tc_ld64(d_layer + lane_base, v);
#pragma unroll
      for (uint32_t c = 0; c < 8; ++c)
        *reinterpret_cast<uint4*>(h + canon_off(tid, 8u * c)) =
            make_uint4(pack2(relu(v[8 * c]), relu(v[8 * c + 1])), pack2(relu(v[8 * c + 2]), relu(v[8 * c + 3])),
                       pack2(relu(v[8 * c + 4]), relu(v[8 * c + 5])), pack2(relu(v[8 * c + 6]), relu(v[8 * c + 7])));
    } else {
      // output layer: dL/dp = 2 (p - y) / (p^2 + 0.01) with the denominator held constant
      float v[16];
      tc_ld16(d_layer + lane_base, v);
      float gz[3] = {0.0f, 0.0f, 0.0f}, lsum = 0.0f;
      if (row < end) {
        const float4 y4 = __ldg(Y + row);
        if (y4.w != 0.0f) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float y = c == 0 ? y4.x : (c == 1 ? y4.y : y4.z);
            const float d = v[c] - y;
            const float den = v[c] * v[c] + 0.01f;
            lsum += d * d / den;
            gz[c] = 2.0f * d / den;
            if (clip > 0.0f) gz[c] = fminf(fmaxf(gz[c], -clip), clip);
          }
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xFFFFFFFFu, lsum, o);
      if ((tid & 31u) == 0) warp_loss[warp] = lsum;
      // dZ6: 128 x 16 (outputs 3..15 zero), 8-row groups 256 B apart
      unsigned char* d6 = dZ6 + (tid >> 3) * 256u + (tid & 7u) * 16u;
      *reinterpret_cast<uint4*>(d6) = make_uint4(pack2(gz[0], gz[1]), pack2(gz[2], 0.0f), 0u, 0u);
      *reinterpret_cast<uint4*>(d6 + 128u) = make_uint4(0u, 0u, 0u, 0u);
    }
    publish(!ok);
  }

  // ---- backward: layer 5 (16 x 64), then 4 .. 0 (64 x 64).  The MMAs of layer l - 1 are
  // issued as soon as dZ_l is in shared memory; meanwhile the warps read layer l's weight
  // gradient out of the other tensor-memory buffer and store it.
  // issues dH_l = dZ_{l+1} W_l (l >= 1) and dW_l = dZ_{l+1}^T H_l, then commits
  auto issue_backward = [&](int l) {
    if (tid != 0) return;
    const bool out_layer = l == 5;
    const uint32_t dz_group = out_layer ? 256u : 1024u;  // bytes between 8-row groups of dZ
    const uint32_t a = saddr(out_layer ? dZ6 : dZ), h = saddr(H + l * kTrAct);
    if (l >= 1) {  // K = 16 (output layer) or 64
      const uint32_t b = out_layer ? saddr(Wb + 4u * 8192u) : saddr(Wb + (l - 1) * 8192u);
      const uint32_t idesc = tc_idesc(kTrRows, 64u);
      const uint32_t kk = out_layer ? 1u : 4u;
      for (uint32_t k = 0; k < kk; ++k)
        tc_mma(d_layer, tc_desc2(a + 256u * k, 128u, dz_group), tc_desc2(b + 256u * k, 128u, out_layer ? 256u : 1024u),
               idesc, k);
    }
    // M = out (padded to 128), N = in, K = 128 rows in 8 steps of 16
    const uint32_t d_w = tmem + 64u + 64u * (uint32_t)(l & 1);
    const uint32_t idesc = tc_idesc2(kTrRows, 64u, true, true);
#pragma unroll
    for (uint32_t k = 0; k < 8; ++k)
      tc_mma(d_w, tc_desc2(a + 2u * k * dz_group, dz_group, 128u), tc_desc2(h + 2u * k * 1024u, 1024u, 128u), idesc, k);
    tc_commit(mbar);
  };
  if (!failed) issue_backward(5);
  for (int l = 5; l >= 0 && !failed; --l) {
    const bool ok = wait_all();
    if (l >= 1) {
      // dZ_l = dH_l where H_l > 0 (BF16 activation), written over dZ (its MMAs are complete)
      const unsigned char* hl = H + l * kTrAct;
      float v[64];
      tc_ld64(d_layer + lane_base, v);
#pragma unroll
      for (uint32_t c = 0; c < 8; ++c) {
        const uint4 m = *reinterpret_cast<const uint4*>(hl + canon_off(tid, 8u * c));
        const float* x = v + 8 * c;
        *reinterpret_cast<uint4*>(dZ + canon_off(tid, 8u * c)) =
            make_uint4(pack2(gate_lo(x[0], m.x), gate_hi(x[1], m.x)), pack2(gate_lo(x[2], m.y), gate_hi(x[3], m.y)),
                       pack2(gate_lo(x[4], m.z), gate_hi(x[5], m.z)), pack2(gate_lo(x[6], m.w), gate_hi(x[7], m.w)));
      }
    }
    publish(!ok);
    if (l >= 1 && !failed) issue_backward(l - 1);
    // weight gradient of layer l: accumulator lane = output unit (< 16 or < 64 live), columns =
    // inputs; warps without live units skip the (warp-collective) loads
    if (!failed && 32u * warp < (l == 5 ? 16u : 64u)) {
      const uint32_t outs = l == 5 ? 16u : 64u;
      const uint32_t d_w = tmem + 64u + 64u * (uint32_t)(l & 1);
      float* d = dw + (size_t)l * 4096u + (size_t)tid * 64u;
      float v[64];
      tc_ld64(d_w + lane_base, v);
      if (tid < outs) {
#pragma unroll
        for (int q = 0; q < 16; ++q)
          *reinterpret_cast<float4*>(d + 4u * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
    }
    // the next round's epilogue overwrites dZ only after its wait, i.e. after these loads
  }
  if (tid == 0) {
    part_loss[blockIdx.x] = warp_loss[0] + warp_loss[1] + warp_loss[2] + warp_loss[3];
    if (failed) {
      atomicOr(status, kStatusCacheTimeout | ((100u + fail_round) << 16));
      mbar_wait(mbar, phase ^ 1u);  // give MMAs still in flight a bounded chance to finish
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem_slot), "r"(kTrCols) : "memory");
  }
}

struct AdamArgs {
  float lr, beta1, beta2, eps;
  float bc1, bc2;  // 1 - beta^t
  float ema;       // decay of the weight average (0: none)
  float ec;        // 1 - ema^t: bias correction of the average (it starts from zero)
  int update;
};

// Sums the per-CTA partials and applies one Adam step (update != 0), or only writes the mean
// gradient to grad_out.  A block takes 32 parameters: its 8 warps each sum every 8th partial
// (partials k, k + 8, ... for warp k, two running sums), and the 8 sums are combined in a fixed
// order, so the result does not depend on scheduling.  With ema > 0 it also advances the
// weight average that renders query (Mueller et al. 2021 average the weights the same way).
constexpr uint32_t kAdamParams = 32;  // parameters per block (one per lane)
__global__ void __launch_bounds__(256) k_cache_adam(float* __restrict__ w, bf16* __restrict__ wb,
                                                    unsigned char* __restrict__ stage,
                                                    float* __restrict__ we, bf16* __restrict__ web,
                                                    float* __restrict__ m, float* __restrict__ v,
                                                    const float* __restrict__ part_dw,
                                                    const float* __restrict__ part_loss,
                                                    const uint32_t* __restrict__ n_dev, uint32_t n_host,
                                                    uint32_t row0, uint32_t rows_per_step, AdamArgs args,
                                                    float* __restrict__ grad_out, float* __restrict__ loss_out) {
  __shared__ float red[8][kAdamParams];
  const uint32_t n_total = n_dev ? *n_dev : n_host;
  const uint32_t rows = n_total > row0 ? min(n_total - row0, rows_per_step) : 0u;
  const uint32_t lane = threadIdx.x & 31u, grp = threadIdx.x >> 5;
  const uint32_t p = blockIdx.x * kAdamParams + lane;
  const uint32_t parts = (rows + kGradRows - 1) / kGradRows;
  const float scale = rows ? 1.0f / (3.0f * (float)rows) : 0.0f;
  if (blockIdx.x == 0 && threadIdx.x == 0 && loss_out) {
    float s = 0.0f;
    for (uint32_t c = 0; c < parts; ++c) s += part_loss[c];
    *loss_out = s * scale;
  }
  float a0 = 0.0f, a1 = 0.0f;
  if (p < (uint32_t)kMlpParams) {
    uint32_t c = grp;
    for (; c + 8 < parts; c += 16) {
      a0 += part_dw[(size_t)c * kMlpParams + p];
      a1 += part_dw[(size_t)(c + 8) * kMlpParams + p];
    }
    if (c < parts) a0 += part_dw[(size_t)c * kMlpParams + p];
  }
  red[grp][lane] = a0 + a1;
  __syncthreads();
  if (grp != 0 || p >= (uint32_t)kMlpParams) return;
  const float gsum = ((red[0][lane] + red[1][lane]) + (red[2][lane] + red[3][lane])) +
                     ((red[4][lane] + red[5][lane]) + (red[6][lane] + red[7][lane]));
  const bool live = p < kLiveEnd;
  const float gr = live ? gsum * scale : 0.0f;
  if (grad_out) grad_out[p] = gr;
  if (!args.update || !live || rows == 0) return;
  const float mm = args.beta1 * m[p] + (1.0f - args.beta1) * gr;
  const float vv = args.beta2 * v[p] + (1.0f - args.beta2) * (gr * gr);
  m[p] = mm;
  v[p] = vv;
  const float wn = w[p] - args.lr * (mm / args.bc1) / (sqrtf(vv / args.bc2) + args.eps);
  w[p] = wn;
  const bf16 b16 = __float2bfloat16_rn(wn);
  wb[p] = b16;
  uint32_t of, ob;
  stage_offsets(p, &of, &ob);
  *reinterpret_cast<bf16*>(stage + of) = b16;
  if (ob != 0xFFFFFFFFu) *reinterpret_cast<bf16*>(stage + ob) = b16;
  if (args.ema > 0.0f) {
    const float e = args.ema * we[p] + (1.0f - args.ema) * wn;
    we[p] = e;
    web[p] = __float2bfloat16_rn(e / args.ec);
  }
}

// ---- training records --------------------------------------------------------------------

// counters: [0] queries, [1] records found, [2] records used, [3] slots of the wave.
// The exclusive scan of the per-slot vertex counts runs in two passes over tiles of
// kScanTile slots (one tile per block): block sums, then each tile's scan plus the sum of the
// tiles before it.  The order of the records is fixed by the slots, so training stays
// deterministic.
constexpr int kScanThreads = 512;
constexpr int kScanPer = 8;
constexpr int kScanTile = kScanThreads * kScanPer;  // 4096 slots per block

// exclusive scan of one value per thread over a kScanThreads block; *total = block sum
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t ws = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, ws, d);
      if (lane >= d) ws += y;
    }
    warp_sums[lane] = ws;  // inclusive over warps
  }
  __syncthreads();
  *total = warp_sums[kScanThreads / 32 - 1];
  return incl - v + (warp > 0 ? warp_sums[warp - 1] : 0u);
}

// Pass 1: the wave's slot count (from the stride its shade kernels used) and each tile's sum.
__global__ void __launch_bounds__(kScanThreads) k_cache_count(const uint32_t* __restrict__ vert_count,
                                                              uint32_t max_slots, uint32_t n_paths,
                                                              const uint32_t* __restrict__ stride,
                                                              uint32_t* __restrict__ block_sums,
                                                              uint32_t* __restrict__ counters) {
  __shared__ uint32_t warp_sums[32];
  const uint32_t G = *stride;
  const uint32_t n_slots = min(max_slots, (n_paths + G - 1) / G);
  if (blockIdx.x == 0 && threadIdx.x == 0) counters[3] = n_slots;
  const uint32_t base = blockIdx.x * (uint32_t)kScanTile;
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    const uint32_t i = base + (uint32_t)k * kScanThreads + threadIdx.x;
    if (i < n_slots) sum += vert_count[i];
  }
  uint32_t total;
  block_exclusive_scan(sum, warp_sums, &total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Pass 2: each slot's first record, the record totals and the next wave's stride.
__global__ void __launch_bounds__(kScanThreads) k_cache_offsets(const uint32_t* __restrict__ vert_count,
                                                                const uint32_t* __restrict__ block_sums,
                                                                uint32_t n_blocks, uint32_t max_slots,
                                                                uint32_t n_paths, uint32_t budget, uint32_t* stride,
                                                                uint32_t* __restrict__ offsets, uint32_t* counters) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t tile[kScanTile];
  __shared__ uint32_t prefix;
  const uint32_t n_slots = counters[3];
  const uint32_t base = blockIdx.x * (uint32_t)kScanTile;
  if (threadIdx.x == 0) {
    uint32_t p = 0;
    for (uint32_t b = 0; b < blockIdx.x; ++b) p += block_sums[b];
    prefix = p;
  }
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    const uint32_t j = (uint32_t)k * kScanThreads + threadIdx.x, i = base + j;
    tile[j] = i < n_slots ? vert_count[i] : 0u;
  }
  __syncthreads();
  uint32_t local[kScanPer], sum = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    local[k] = sum;
    sum += tile[threadIdx.x * kScanPer + k];
  }
  uint32_t total;
  const uint32_t before = block_exclusive_scan(sum, warp_sums, &total) + prefix;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) tile[threadIdx.x * kScanPer + k] = before + local[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    const uint32_t j = (uint32_t)k * kScanThreads + threadIdx.x, i = base + j;
    if (i < n_slots) offsets[i] = tile[j];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    uint32_t all = 0;
    for (uint32_t b = 0; b < n_blocks; ++b) all += block_sums[b];
    counters[1] = all;
    counters[2] = min(all, budget);
    // one training path per G paths gave `all` records: aim the next wave at the budget
    const uint32_t G = *stride;
    const uint32_t g_min = max(1u, (n_paths + max_slots - 1) / max_slots);
    double next = all ? (double)G * (double)all / (double)budget : (double)g_min;
    next = fmin(fmax(next, (double)g_min), (double)nb::kCacheMaxStride);
    *stride = (uint32_t)(next + 0.5);
  }
}

// One thread per slot: walks the chain backwards (L_k = w_k * L_{k+1}, L after the last vertex
// = tail) and writes the encoded inputs and reflectance-factorised targets of its records.
__global__ void __launch_bounds__(128) k_cache_gather(const TrainVertex* __restrict__ verts,
                                                      const uint32_t* __restrict__ vert_count,
                                                      const float4* __restrict__ tail,
                                                      const uint32_t* __restrict__ offsets,
                                                      const uint32_t* __restrict__ counters, CacheBounds bounds,
                                                      bf16* __restrict__ X, float4* __restrict__ Y) {
  const uint32_t n_slots = counters[3], used = counters[2];
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n_slots; s += gridDim.x * blockDim.x) {
    const uint32_t cnt = vert_count[s];
    if (cnt == 0) continue;
    const uint32_t off = offsets[s];
    const float4 t4 = tail[s];
    V3 L{t4.x, t4.y, t4.z};
    for (int k = (int)cnt - 1; k >= 0; --k) {
      const TrainVertex tv = verts[(size_t)s * nb::kCacheMaxVertices + k];
      L = L * V3{tv.w.x, tv.w.y, tv.w.z};
      const uint32_t row = off + (uint32_t)k;
      if (row >= used) continue;
      const V3 fac = cache_factor(tv.f);
      const V3 y = V3{L.x / fac.x, L.y / fac.y, L.z / fac.z};
      const bool ok = isfinite(y.x) && isfinite(y.y) && isfinite(y.z);
      Y[row] = make_float4(ok ? y.x : 0.0f, ok ? y.y : 0.0f, ok ? y.z : 0.0f, ok ? 1.0f : 0.0f);
      float f[64];
      cache_encode(tv.f, bounds, f);
      uint4* dst = reinterpret_cast<uint4*>(X + (size_t)row * 64);
#pragma unroll
      for (int c = 0; c < 8; ++c)
        dst[c] = make_uint4(pack2(f[8 * c], f[8 * c + 1]), pack2(f[8 * c + 2], f[8 * c + 3]),
                            pack2(f[8 * c + 4], f[8 * c + 5]), pack2(f[8 * c + 6], f[8 * c + 7]));
    }
  }
}

// ---- API helpers -------------------------------------------------------------------------

__global__ void k_to_bf16(const float* __restrict__ in, bf16* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(in[i]);
}
__global__ void k_targets(const float* __restrict__ in, float4* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = make_float4(in[3 * i], in[3 * i + 1], in[3 * i + 2], 1.0f);
}
__global__ void k_encode(const CacheFeatures* __restrict__ v, size_t n, CacheBounds b, float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float f[64];
    cache_encode(v[i], b, f);
#pragma unroll
    for (int k = 0; k < 64; ++k) out[64 * i + k] = f[k];
  }
}

}  // namespace nbd

// ==========================================================================================
// host side
// ==========================================================================================
using namespace nb;

struct nb_cache {
  nb_cache_config cfg{};
  DeviceArena arena;  // weights, optimiser state, gradient partials
  float* w = nullptr;
  nbd::bf16* wb = nullptr;
  float* we = nullptr;      // weight average, uncorrected (renders query web when cfg.ema > 0)
  nbd::bf16* web = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  uint32_t* status = nullptr;  // tensor-core wait timeouts of nb_cache_infer / training
  unsigned char* wstage = nullptr;  // training weight image (k_cache_grad_tc), kept by k_cache_adam
  float* part_dw = nullptr;
  float* part_loss = nullptr;
  uint32_t part_cap = 0;  // CTAs the partial buffers hold
  float* losses = nullptr;  // per step of the last frame
  uint32_t losses_cap = 0;
  uint64_t adam_steps = 0;
  CacheBounds bounds{};
  bool bounds_set = false;
  // per-wave buffers
  DeviceArena wave;
  uint32_t cap_paths = 0, cap_slots = 0, cap_records = 0;
  float4* q_x = nullptr;
  CacheQuery* queries = nullptr;
  uint32_t* counters = nullptr;  // queries, records found, records used, slots
  TrainVertex* verts = nullptr;
  uint32_t* vert_count = nullptr;
  float4* tail = nullptr;
  uint32_t* offsets = nullptr;
  uint32_t* block_sums = nullptr;  // per scan tile
  uint32_t* stride = nullptr;
  nbd::bf16* X = nullptr;
  float4* Y = nullptr;
  uint32_t frame = 0;
  uint32_t last_steps = 0;
  bool stride_init = false;
  // API scratch (encoded rows / targets of nb_cache_infer / _gradient / _train_step)
  DeviceArena scratch;
  size_t scratch_rows = 0;
  nbd::bf16* sx = nullptr;
  float4* sy = nullptr;
  std::mutex mu;
};

namespace {

// splitmix64: weight initialisation stream
uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int set_smem_limits() {
  static int rc = -1;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaError_t e = cudaFuncSetAttribute(nbd::k_cache_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)nbd::kGradSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(nbd::k_cache_infer_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)nbd::kInferSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(nbd::k_cache_infer_queries, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)nbd::kInferSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(nbd::k_cache_infer_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)nbd::kTcSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(nbd::k_cache_infer_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)nbd::kTcSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(nbd::k_cache_grad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)nbd::kTrSmem);
    rc = e == cudaSuccess ? NB_OK : cuda_fail(e, "cudaFuncSetAttribute(cache kernels)");
  });
  return rc;
}

int upload_weights(nb_cache* c, const float* w_host) {
  std::vector<nbd::bf16> b(kMlpParams);
  for (int i = 0; i < kMlpParams; ++i) b[i] = __float2bfloat16_rn(w_host[i]);
  NB_CUDA(cudaMemcpy(c->w, w_host, kMlpParams * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy(weights)");
  NB_CUDA(cudaMemcpy(c->wb, b.data(), kMlpParams * sizeof(nbd::bf16), cudaMemcpyHostToDevice), "cudaMemcpy(weights)");
  NB_CUDA(cudaMemset(c->we, 0, kMlpParams * sizeof(float)), "cudaMemset");
  NB_CUDA(cudaMemcpy(c->web, b.data(), kMlpParams * sizeof(nbd::bf16), cudaMemcpyHostToDevice), "cudaMemcpy(weights)");
  NB_CUDA(cudaMemset(c->m, 0, kMlpParams * sizeof(float)), "cudaMemset");
  NB_CUDA(cudaMemset(c->v, 0, kMlpParams * sizeof(float)), "cudaMemset");
  std::vector<unsigned char> img(nbd::kTrStage, 0);
  for (uint32_t p = 0; p < (uint32_t)kMlpParams; ++p) {
    uint32_t of, ob;
    nbd::stage_offsets(p, &of, &ob);
    std::memcpy(img.data() + of, &b[p], sizeof(nbd::bf16));
    if (ob != 0xFFFFFFFFu) std::memcpy(img.data() + ob, &b[p], sizeof(nbd::bf16));
  }
  NB_CUDA(cudaMemcpy(c->wstage, img.data(), img.size(), cudaMemcpyHostToDevice), "cudaMemcpy(weight image)");
  c->adam_steps = 0;
  return NB_OK;
}

int ensure_parts(nb_cache* c, uint32_t ctas) {
  if (ctas <= c->part_cap) return NB_OK;
  // grown in a separate arena entry; the old partials are simply left to the arena
  void* p = nullptr;
  int rc = c->arena.alloc((size_t)ctas * kMlpParams * sizeof(float), &p);
  if (rc) return rc;
  c->part_dw = (float*)p;
  rc = c->arena.alloc((size_t)ctas * sizeof(float), &p);
  if (rc) return rc;
  c->part_loss = (float*)p;
  c->part_cap = ctas;
  return NB_OK;
}

int ensure_losses(nb_cache* c, uint32_t steps) {
  if (steps <= c->losses_cap) return NB_OK;
  void* p = nullptr;
  int rc = c->arena.alloc((size_t)steps * sizeof(float), &p);
  if (rc) return rc;
  c->losses = (float*)p;
  c->losses_cap = steps;
  return NB_OK;
}

int ensure_scratch(nb_cache* c, size_t rows) {
  if (rows <= c->scratch_rows) return NB_OK;
  c->scratch.release();
  c->scratch_rows = 0;
  void* p = nullptr;
  int rc = c->scratch.alloc(rows * 64 * sizeof(nbd::bf16), &p);
  if (rc) return rc;
  c->sx = (nbd::bf16*)p;
  rc = c->scratch.alloc(rows * sizeof(float4), &p);
  if (rc) return rc;
  c->sy = (float4*)p;
  c->scratch_rows = rows;
  return NB_OK;
}

int grid_for(size_t n, int threads, int sms) {
  size_t g = (n + threads - 1) / threads;
  return (int)std::max<size_t>(1, std::min<size_t>(g, (size_t)sms * 8));
}

// one optimiser step (update) or gradient evaluation over rows [row0, row0 + rows_per_step)
// of (X, Y); n_dev (device row count) or n_host bounds the rows
cudaError_t train_launch(nb_cache* c, const nbd::bf16* X, const float4* Y, const uint32_t* n_dev, uint32_t n_host,
                         uint32_t row0, uint32_t rows_per_step, bool update, float* grad_out, float* loss_out,
                         cudaStream_t st) {
  const uint32_t ctas = (rows_per_step + nbd::kGradRows - 1) / nbd::kGradRows;
  if (c->cfg.tensor_path == NB_CACHE_TCGEN05)
    nbd::k_cache_grad_tc<<<ctas, 128, nbd::kTrSmem, st>>>(c->wstage, X, Y, n_dev, n_host, row0, rows_per_step,
                                                          c->cfg.grad_clip, c->part_dw, c->part_loss, c->status);
  else
    nbd::k_cache_grad<<<ctas, 256, nbd::kGradSmem, st>>>(c->wb, X, Y, n_dev, n_host, row0, rows_per_step,
                                                         c->cfg.grad_clip, c->part_dw, c->part_loss);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  nbd::AdamArgs a{};
  a.lr = c->cfg.learning_rate;
  a.beta1 = c->cfg.beta1;
  a.beta2 = c->cfg.beta2;
  a.eps = c->cfg.epsilon;
  a.ema = c->cfg.ema;
  a.update = update ? 1 : 0;
  if (update) {
    // Adam bias correction with the step number of this update; a step whose rows turn out to be
    // empty on the device skips the update but still counts here (it only shifts the correction)
    const double t = (double)(c->adam_steps + 1);
    a.bc1 = (float)(1.0 - std::pow((double)c->cfg.beta1, t));
    a.bc2 = (float)(1.0 - std::pow((double)c->cfg.beta2, t));
    a.ec = (float)(1.0 - std::pow((double)c->cfg.ema, t));
    c->adam_steps += 1;
  } else {
    a.bc1 = a.bc2 = a.ec = 1.0f;
  }
  nbd::k_cache_adam<<<(kMlpParams + nbd::kAdamParams - 1) / nbd::kAdamParams, 256, 0, st>>>(
      c->w, c->wb, c->wstage, c->we, c->web, c->m, c->v,
                                                              c->part_dw,
                                                              c->part_loss,
                                                              n_dev, n_host, row0, rows_per_step, a, grad_out,
                                                              loss_out);
  return cudaGetLastError();
}

}  // namespace

namespace nb {

// Buffers and wave state for a cache-mode wave of n_paths paths on `scene`.
int cache_wave_begin(nb_cache* c, const nb_scene* scene, uint32_t n_paths, CacheWave* cw, cudaStream_t st) {
  if (!c || !cw) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  int rc = set_smem_limits();
  if (rc) return rc;
  if (!c->bounds_set) {
    const std::vector<nb_bvh_node>& root = scene->host.has_tlas ? scene->host.tlas : scene->host.blas;
    if (root.empty()) return fail(NB_ERR_INVALID_ARG, "scene has no bounds");
    for (int a = 0; a < 3; ++a) {
      const float lo = root[0].min[a], hi = root[0].max[a];
      c->bounds.lo[a] = lo;
      c->bounds.inv_extent[a] = hi > lo ? 1.0f / (hi - lo) : 1.0f;
    }
    c->bounds_set = true;
  }
  const uint32_t budget = c->cfg.train_records;
  // training slots: up to one per path, at most 4 budgets' worth of training paths
  const uint32_t want_slots = std::max<uint32_t>(1024u, std::min<uint32_t>(n_paths, 4u * budget));
  if (n_paths > c->cap_paths || want_slots > c->cap_slots || budget > c->cap_records) {
    NB_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    const uint32_t P = std::max(n_paths, c->cap_paths), S = std::max(want_slots, c->cap_slots);
    const uint32_t R = std::max(budget, 1u);
    c->wave.release();
    c->cap_paths = c->cap_slots = c->cap_records = 0;
    void* p = nullptr;
    if ((rc = c->wave.alloc((size_t)2 * P * sizeof(float4), &p))) return rc;
    c->q_x = (float4*)p;
    if ((rc = c->wave.alloc((size_t)(P + S) * sizeof(CacheQuery), &p))) return rc;
    c->queries = (CacheQuery*)p;
    if ((rc = c->wave.alloc(8 * sizeof(uint32_t), &p))) return rc;
    c->counters = (uint32_t*)p;
    if ((rc = c->wave.alloc((size_t)S * kCacheMaxVertices * sizeof(TrainVertex), &p))) return rc;
    c->verts = (TrainVertex*)p;
    if ((rc = c->wave.alloc((size_t)S * sizeof(uint32_t), &p))) return rc;
    c->vert_count = (uint32_t*)p;
    if ((rc = c->wave.alloc((size_t)S * sizeof(float4), &p))) return rc;
    c->tail = (float4*)p;
    if ((rc = c->wave.alloc((size_t)S * sizeof(uint32_t), &p))) return rc;
    c->offsets = (uint32_t*)p;
    if ((rc = c->wave.alloc(((size_t)S + nbd::kScanTile - 1) / nbd::kScanTile * sizeof(uint32_t), &p))) return rc;
    c->block_sums = (uint32_t*)p;
    if ((rc = c->wave.alloc(sizeof(uint32_t), &p))) return rc;
    c->stride = (uint32_t*)p;
    if ((rc = c->wave.alloc((size_t)R * 64 * sizeof(nbd::bf16), &p))) return rc;
    c->X = (nbd::bf16*)p;
    if ((rc = c->wave.alloc((size_t)R * sizeof(float4), &p))) return rc;
    c->Y = (float4*)p;
    c->cap_paths = P;
    c->cap_slots = S;
    c->cap_records = R;
    c->stride_init = false;
  }
  if ((rc = ensure_parts(c, (c->cfg.train_records / std::max(1u, c->cfg.train_steps) + nbd::kGradRows - 1) /
                                   nbd::kGradRows + 1)))
    return rc;
  if ((rc = ensure_losses(c, std::max(1u, c->cfg.train_steps)))) return rc;
  if (!c->stride_init) {
    // first wave: guess three records per training path
    const uint64_t g_min = (n_paths + (uint64_t)c->cap_slots - 1) / c->cap_slots;
    uint64_t g = std::max<uint64_t>(1, (uint64_t)n_paths * 3 / std::max(1u, budget));
    g = std::min<uint64_t>(std::max<uint64_t>(g, std::max<uint64_t>(g_min, 1)), kCacheMaxStride);
    const uint32_t g32 = (uint32_t)g;
    NB_CUDA(cudaMemcpyAsync(c->stride, &g32, sizeof(g32), cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    NB_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    c->stride_init = true;
  }
  NB_CUDA(cudaMemsetAsync(c->counters, 0, 8 * sizeof(uint32_t), st), "cudaMemsetAsync");
  NB_CUDA(cudaMemsetAsync(c->vert_count, 0, (size_t)c->cap_slots * sizeof(uint32_t), st), "cudaMemsetAsync");
  cw->q_x[0] = c->q_x;
  cw->q_x[1] = c->q_x + c->cap_paths;
  cw->queries = c->queries;
  cw->n_queries = c->counters;
  cw->max_queries = c->cap_paths + c->cap_slots;
  cw->verts = c->verts;
  cw->vert_count = c->vert_count;
  cw->tail = c->tail;
  cw->stride = c->stride;
  cw->max_slots = c->cap_slots;
  cw->frame = c->frame;
  cw->spread_c = c->cfg.spread;
  cw->extra = c->cfg.extra_vertices;
  return NB_OK;
}

// After the last bounce: cache lookups of the wave's queries.
int cache_wave_infer(nb_cache* c, const PathBatch& pb, int sms, cudaStream_t st) {
  const nbd::bf16* w = c->cfg.ema > 0.0f ? c->web : c->wb;
  if (c->cfg.tensor_path == NB_CACHE_TCGEN05)
    nbd::k_cache_infer_tc<true><<<2 * sms, nbd::kTcThreads, nbd::kTcSmem, st>>>(
        w, nullptr, c->queries, c->counters, c->cap_paths + c->cap_slots, c->bounds, nullptr, pb.radiance, c->tail,
        pb.status);
  else
    nbd::k_cache_infer_queries<<<2 * sms, 256, nbd::kInferSmem, st>>>(w, c->queries, c->counters,
                                                                      c->cap_paths + c->cap_slots, c->bounds,
                                                                      pb.radiance, c->tail);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "cache lookup launch");
  return NB_OK;
}

// Then: training records from the training paths' chains and the optimiser steps.
int cache_wave_train(nb_cache* c, uint32_t n_paths, int sms, cudaStream_t st) {
  const uint32_t tiles = (c->cap_slots + nbd::kScanTile - 1) / nbd::kScanTile;
  nbd::k_cache_count<<<tiles, nbd::kScanThreads, 0, st>>>(c->vert_count, c->cap_slots, n_paths, c->stride,
                                                          c->block_sums, c->counters);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    nbd::k_cache_offsets<<<tiles, nbd::kScanThreads, 0, st>>>(c->vert_count, c->block_sums, tiles, c->cap_slots,
                                                              n_paths, c->cfg.train_records, c->stride, c->offsets,
                                                              c->counters);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    nbd::k_cache_gather<<<grid_for(c->cap_slots, 128, sms), 128, 0, st>>>(
        c->verts, c->vert_count, c->tail, c->offsets, c->counters, c->bounds, c->X, c->Y);
    e = cudaGetLastError();
  }
  const uint32_t steps = c->cfg.train_steps;
  const uint32_t per = steps ? (c->cfg.train_records + steps - 1) / steps : 0;
  for (uint32_t k = 0; k < steps && e == cudaSuccess; ++k)
    e = train_launch(c, c->X, c->Y, c->counters + 2, 0, k * per, per, c->cfg.learning_rate > 0.0f, nullptr,
                     c->losses + k, st);
  if (e != cudaSuccess) return cuda_fail(e, "cache wave launch");
  c->last_steps = steps;
  c->frame += 1;
  return NB_OK;
}

}  // namespace nb

// ==========================================================================================
// C ABI
// ==========================================================================================

void nb_cache_default_config(nb_cache_config* cfg) {
  if (!cfg) return;
  cfg->learning_rate = 1e-2f;
  cfg->beta1 = 0.9f;
  cfg->beta2 = 0.99f;
  cfg->epsilon = 1e-8f;
  cfg->spread = 0.01f;
  cfg->train_records = 65536;
  cfg->train_steps = 4;
  cfg->extra_vertices = 3;
  cfg->seed = 0x5EED0u;
  cfg->ema = 0.99f;
  cfg->grad_clip = 0.0f;
  cfg->tensor_path = NB_CACHE_TCGEN05;
}

int nb_cache_create(const nb_cache_config* cfg, nb_cache** out) {
  if (!out) return fail(NB_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  nb_cache_config c{};
  if (cfg) c = *cfg;
  else nb_cache_default_config(&c);
  if (!(c.learning_rate >= 0.0f) || !(c.beta1 >= 0.0f && c.beta1 < 1.0f) || !(c.beta2 >= 0.0f && c.beta2 < 1.0f) ||
      !(c.epsilon > 0.0f))
    return fail(NB_ERR_INVALID_ARG, "invalid optimiser settings");
  if (c.train_records > (1u << 24) || (c.train_steps == 0) != (c.train_records == 0) || c.train_steps > 64)
    return fail(NB_ERR_INVALID_ARG, "train_records must be <= 2^24 and train_steps in 1..64 (both 0 to freeze)");
  if (c.extra_vertices > nb::kCacheMaxVertices) return fail(NB_ERR_INVALID_ARG, "extra_vertices must be <= 8");
  if (!(c.ema >= 0.0f && c.ema < 1.0f) || !(c.grad_clip >= 0.0f))
    return fail(NB_ERR_INVALID_ARG, "ema must be in [0, 1) and grad_clip >= 0");
  if (c.tensor_path != NB_CACHE_TCGEN05 && c.tensor_path != NB_CACHE_MMA_SYNC)
    return fail(NB_ERR_INVALID_ARG, "unknown tensor_path");
  int n_dev = 0;
  if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0) return fail(NB_ERR_NO_DEVICE, "no CUDA device");
  nb_cache* h = new (std::nothrow) nb_cache();
  if (!h) return fail(NB_ERR_OOM, "host allocation failed");
  h->cfg = c;
  void* p[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  int rc = NB_OK;
  for (int k = 0; k < 6 && !rc; ++k)
    rc = h->arena.alloc(kMlpParams * ((k == 1 || k == 3) ? sizeof(nbd::bf16) : sizeof(float)), &p[k]);
  h->w = (float*)p[0];
  h->wb = (nbd::bf16*)p[1];
  h->we = (float*)p[2];
  h->web = (nbd::bf16*)p[3];
  h->m = (float*)p[4];
  h->v = (float*)p[5];
  if (!rc) rc = h->arena.alloc(sizeof(uint32_t), &p[6]);
  h->status = (uint32_t*)p[6];
  void* stage = nullptr;
  if (!rc) rc = h->arena.alloc(nbd::kTrStage, &stage);
  h->wstage = (unsigned char*)stage;
  if (!rc) {
    // He-uniform initialisation: U(-sqrt(6 / 64), sqrt(6 / 64)); padding rows of W_5 zero
    std::vector<float> w(kMlpParams, 0.0f);
    uint64_t s = c.seed;
    const double lim = std::sqrt(6.0 / 64.0);
    for (uint32_t i = 0; i < nbd::kLiveEnd; ++i)
      w[i] = (float)((double)(splitmix(s) >> 11) * 0x1.0p-53 * 2.0 * lim - lim);
    rc = upload_weights(h, w.data());
  }
  if (rc) {
    h->arena.release();
    delete h;
    return rc;
  }
  *out = h;
  return NB_OK;
}

void nb_cache_destroy(nb_cache* c) {
  if (!c) return;
  cudaDeviceSynchronize();
  c->arena.release();
  c->wave.release();
  c->scratch.release();
  delete c;
}

int nb_cache_get_config(const nb_cache* c, nb_cache_config* out) {
  if (!c || !out) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  *out = c->cfg;
  return NB_OK;
}

int nb_cache_set_bounds(nb_cache* c, const float lo[3], const float hi[3]) {
  if (!c || !lo || !hi) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  for (int a = 0; a < 3; ++a) {
    if (!(hi[a] >= lo[a])) return fail(NB_ERR_INVALID_ARG, "bounds: hi < lo");
    c->bounds.lo[a] = lo[a];
    c->bounds.inv_extent[a] = hi[a] > lo[a] ? 1.0f / (hi[a] - lo[a]) : 1.0f;
  }
  c->bounds_set = true;
  return NB_OK;
}

int nb_cache_get_weights(const nb_cache* c, float* w, size_t n) {
  if (!c || !w) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (n != (size_t)kMlpParams) return fail(NB_ERR_INVALID_ARG, "weights hold %d floats", kMlpParams);
  NB_CUDA(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
  NB_CUDA(cudaMemcpy(w, c->w, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost), "cudaMemcpy(weights)");
  return NB_OK;
}

int nb_cache_set_weights(nb_cache* c, const float* w, size_t n) {
  if (!c || !w) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (n != (size_t)kMlpParams) return fail(NB_ERR_INVALID_ARG, "weights hold %d floats", kMlpParams);
  std::lock_guard<std::mutex> lk(c->mu);
  NB_CUDA(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
  std::vector<float> cp(w, w + kMlpParams);
  for (int i = (int)nbd::kLiveEnd; i < kMlpParams; ++i) cp[i] = 0.0f;
  return upload_weights(c, cp.data());
}

int nb_cache_encode(nb_cache* c, const nb_cache_vertex* v, size_t n, float* out, void* stream) {
  if (!c || (!v && n) || (!out && n)) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (n == 0) return NB_OK;
  static_assert(sizeof(nb_cache_vertex) == sizeof(CacheFeatures), "nb_cache_vertex layout");
  nbd::k_encode<<<grid_for(n, 128, sm_count()), 128, 0, (cudaStream_t)stream>>>((const CacheFeatures*)v, n,
                                                                              c->bounds, out);
  NB_CUDA(cudaGetLastError(), "cache encode launch");
  return NB_OK;
}

int nb_cache_infer(nb_cache* c, const float* enc, size_t n, float* out, void* stream) {
  if (!c || (!enc && n) || (!out && n)) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (n == 0) return NB_OK;
  if (n > (1u << 30)) return fail(NB_ERR_INVALID_ARG, "too many rows");
  std::lock_guard<std::mutex> lk(c->mu);
  int rc = set_smem_limits();
  if (rc || (rc = ensure_scratch(c, n))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int sms = sm_count();
  nbd::k_to_bf16<<<grid_for(n * 64, 256, sms), 256, 0, st>>>(enc, c->sx, n * 64);
  if (c->cfg.tensor_path == NB_CACHE_TCGEN05) {
    NB_CUDA(cudaMemsetAsync(c->status, 0, sizeof(uint32_t), st), "cudaMemsetAsync");
    const size_t rounds = (n + 4 * nbd::kTcRows - 1) / (4 * nbd::kTcRows);
    nbd::k_cache_infer_tc<false><<<(unsigned)std::min<size_t>(rounds, 2 * (size_t)sms), nbd::kTcThreads,
                                   nbd::kTcSmem, st>>>(c->wb, c->sx, nullptr, nullptr, (uint32_t)n, c->bounds, out,
                                                       nullptr, nullptr, c->status);
  } else {
    nbd::k_cache_infer_rows<<<std::min<size_t>((n + 255) / 256, 2 * (size_t)sms), 256, nbd::kInferSmem, st>>>(
        c->wb, c->sx, (uint32_t)n, out);
  }
  NB_CUDA(cudaGetLastError(), "cache infer launch");
  if (c->cfg.tensor_path == NB_CACHE_TCGEN05) {
    uint32_t status = 0;
    NB_CUDA(cudaMemcpyAsync(&status, c->status, sizeof(status), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    NB_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (status & nbd::kStatusCacheTimeout)
      return fail(NB_ERR_TIMEOUT, "tensor-core wait timed out (layer %u)", (status >> 16) - 1u);
  }
  return NB_OK;
}

static int rows_op(nb_cache* c, const float* enc, const float* target, size_t n, bool update, float* grad,
                   float* loss, void* stream) {
  if (!c || (!enc && n) || (!target && n)) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (n == 0) return fail(NB_ERR_INVALID_ARG, "empty batch");
  if (n > (1u << 24)) return fail(NB_ERR_INVALID_ARG, "batch larger than 2^24 rows");
  std::lock_guard<std::mutex> lk(c->mu);
  int rc = set_smem_limits();
  if (rc || (rc = ensure_scratch(c, n))) return rc;
  const uint32_t ctas = (uint32_t)((n + nbd::kGradRows - 1) / nbd::kGradRows);
  if ((rc = ensure_parts(c, ctas)) || (rc = ensure_losses(c, 1))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int sms = sm_count();
  const bool tc = c->cfg.tensor_path == NB_CACHE_TCGEN05;
  cudaError_t e = tc ? cudaMemsetAsync(c->status, 0, sizeof(uint32_t), st) : cudaSuccess;
  if (e == cudaSuccess) {
    nbd::k_to_bf16<<<grid_for(n * 64, 256, sms), 256, 0, st>>>(enc, c->sx, n * 64);
    nbd::k_targets<<<grid_for(n, 256, sms), 256, 0, st>>>(target, c->sy, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = train_launch(c, c->sx, c->sy, nullptr, (uint32_t)n, 0, (uint32_t)n, update, grad, c->losses, st);
  if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, c->losses, sizeof(float), cudaMemcpyDeviceToHost, st);
  uint32_t status = 0;
  if (e == cudaSuccess && tc) e = cudaMemcpyAsync(&status, c->status, sizeof(status), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "cache training launch");
  if (status & nbd::kStatusCacheTimeout) return fail(NB_ERR_TIMEOUT, "tensor-core wait timed out in training");
  return NB_OK;
}

int nb_cache_gradient(nb_cache* c, const float* enc, const float* target, size_t n, float* grad, float* loss,
                      void* stream) {
  if (!grad) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  return rows_op(c, enc, target, n, false, grad, loss, stream);
}

int nb_cache_train_step(nb_cache* c, const float* enc, const float* target, size_t n, float* loss, void* stream) {
  return rows_op(c, enc, target, n, true, nullptr, loss, stream);
}

int nb_cache_get_stats(nb_cache* c, nb_cache_stats* out, void* stream) {
  if (!c || !out) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::memset(out, 0, sizeof(*out));
  out->frames = c->frame;
  out->adam_steps = c->adam_steps;
  if (!c->counters) return NB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t cnt[4] = {0, 0, 0, 0}, stride = 0;
  float losses[64] = {0};
  NB_CUDA(cudaMemcpyAsync(cnt, c->counters, sizeof(cnt), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
  NB_CUDA(cudaMemcpyAsync(&stride, c->stride, sizeof(stride), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
  const uint32_t steps = std::min<uint32_t>(c->last_steps, 64);
  if (steps)
    NB_CUDA(cudaMemcpyAsync(losses, c->losses, steps * sizeof(float), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
  NB_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  out->queries = cnt[0];
  out->records_found = cnt[1];
  out->records_used = cnt[2];
  out->training_groups = cnt[3];
  out->stride = stride;
  double s = 0.0;
  for (uint32_t k = 0; k < steps; ++k) s += losses[k];
  out->loss = steps ? (float)(s / steps) : 0.0f;
  return NB_OK;
}

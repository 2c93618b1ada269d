// BC6H (BPTC float) block decoding and DDS cube-map parsing: the environment format the
// reference loads (EnvMap::load, envmap.rs:12-17; Texture::create_cubemap, texture.rs:89-144,
// which accepts DXGI BC6H_UF16 only and samples mip 0 through textureSampleLevel,
// pathtracing.wgsl:168).  The reference leaves the decoding to the graphics hardware; here a
// kernel decodes mip 0 of the six faces once at ingest into the RGBA32F texel table the pass
// samples, so traversal and shading stay format-agnostic.
//
// The block format follows the published BC6H specification (Direct3D 11 "BC6H format";
// Khronos Data Format Specification, "BC6H"): a 128-bit little-endian block holds a 2- or
// 5-bit mode, endpoints whose bits are spread over the block in a mode-specific order, a
// 5-bit partition number for the two-subset modes, and 3-bit (two subsets) or 4-bit (one
// subset) texel indices whose anchor texels drop their top bit.  Endpoints of the transformed
// modes are deltas to the first endpoint; all are unquantised to 16 bits, interpolated with
// the 6-bit weights and scaled to half-float bits (31/64 unsigned, 31/32 signed).  Reserved
// modes decode to zero.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "nb_internal.h"
#include "nb_runtime.h"

namespace nb {
namespace {

// Endpoints: subset 0 uses (w, x), subset 1 uses (y, z).
enum : uint16_t { ew = 0, ex = 1, ey = 2, ez = 3 };
enum : uint16_t { cr = 0, cg = 1, cb = 2 };
// A run of n consecutive block bits that holds bits [lo, lo + n) of one endpoint channel.
// Runs marked reversed hold those bits highest first.
constexpr uint16_t run(uint16_t e, uint16_t c, uint16_t lo, uint16_t n) {
  return (uint16_t)(e << 12 | c << 10 | lo << 5 | n);
}
constexpr uint16_t rev(uint16_t e, uint16_t c, uint16_t lo, uint16_t n) {
  return (uint16_t)(1u << 14 | run(e, c, lo, n));
}

// The endpoint bit layout of each mode, in block order after the mode bits.
__constant__ const uint16_t kRuns[] = {
    // mode 1 (2-bit mode 00): 10-bit endpoints, deltas 5/5/5
    run(ey, cg, 4, 1), run(ey, cb, 4, 1), run(ez, cb, 4, 1), run(ew, cr, 0, 10), run(ew, cg, 0, 10),
    run(ew, cb, 0, 10), run(ex, cr, 0, 5), run(ez, cg, 4, 1), run(ey, cg, 0, 4), run(ex, cg, 0, 5),
    run(ez, cb, 0, 1), run(ez, cg, 0, 4), run(ex, cb, 0, 5), run(ez, cb, 1, 1), run(ey, cb, 0, 4),
    run(ey, cr, 0, 5), run(ez, cb, 2, 1), run(ez, cr, 0, 5), run(ez, cb, 3, 1),
    // mode 2 (01): 7-bit endpoints, deltas 6/6/6
    run(ey, cg, 5, 1), run(ez, cg, 4, 1), run(ez, cg, 5, 1), run(ew, cr, 0, 7), run(ez, cb, 0, 1),
    run(ez, cb, 1, 1), run(ey, cb, 4, 1), run(ew, cg, 0, 7), run(ey, cb, 5, 1), run(ez, cb, 2, 1),
    run(ey, cg, 4, 1), run(ew, cb, 0, 7), run(ez, cb, 3, 1), run(ez, cb, 5, 1), run(ez, cb, 4, 1),
    run(ex, cr, 0, 6), run(ey, cg, 0, 4), run(ex, cg, 0, 6), run(ez, cg, 0, 4), run(ex, cb, 0, 6),
    run(ey, cb, 0, 4), run(ey, cr, 0, 6), run(ez, cr, 0, 6),
    // mode 3 (00010): 11-bit endpoints, deltas 5/4/4
    run(ew, cr, 0, 10), run(ew, cg, 0, 10), run(ew, cb, 0, 10), run(ex, cr, 0, 5), run(ew, cr, 10, 1),
    run(ey, cg, 0, 4), run(ex, cg, 0, 4), run(ew, cg, 10, 1), run(ez, cb, 0, 1), run(ez, cg, 0, 4),
    run(ex, cb, 0, 4), run(ew, cb, 10, 1), run(ez, cb, 1, 1), run(ey, cb, 0, 4), run(ey, cr, 0, 5),
    run(ez, cb, 2, 1), run(ez, cr, 0, 5), run(ez, cb, 3, 1),
    // mode 4 (00110): 11-bit endpoints, deltas 4/5/4
    run(ew, cr, 0, 10), run(ew, cg, 0, 10), run(ew, cb, 0, 10), run(ex, cr, 0, 4), run(ew, cr, 10, 1),
    run(ez, cg, 4, 1), run(ey, cg, 0, 4), run(ex, cg, 0, 5), run(ew, cg, 10, 1), run(ez, cg, 0, 4),
    run(ex, cb, 0, 4), run(ew, cb, 10, 1), run(ez, cb, 1, 1), run(ey, cb, 0, 4), run(ey, cr, 0, 4),
    run(ez, cb, 0, 1), run(ez, cb, 2, 1), run(ez, cr, 0, 4), run(ey, cg, 4, 1), run(ez, cb, 3, 1),
    // mode 5 (01010): 11-bit endpoints, deltas 4/4/5
    run(ew, cr, 0, 10), run(ew, cg, 0, 10), run(ew, cb, 0, 10), run(ex, cr, 0, 4), run(ew, cr, 10, 1),
    run(ey, cb, 4, 1), run(ey, cg, 0, 4), run(ex, cg, 0, 4), run(ew, cg, 10, 1), run(ez, cb, 0, 1),
    run(ez, cg, 0, 4), run(ex, cb, 0, 5), run(ew, cb, 10, 1), run(ey, cb, 0, 4), run(ey, cr, 0, 4),
    run(ez, cb, 1, 1), run(ez, cb, 2, 1), run(ez, cr, 0, 4), run(ez, cb, 4, 1), run(ez, cb, 3, 1),
    // mode 6 (01110): 9-bit endpoints, deltas 5/5/5
    run(ew, cr, 0, 9), run(ey, cb, 4, 1), run(ew, cg, 0, 9), run(ey, cg, 4, 1), run(ew, cb, 0, 9),
    run(ez, cb, 4, 1), run(ex, cr, 0, 5), run(ez, cg, 4, 1), run(ey, cg, 0, 4), run(ex, cg, 0, 5),
    run(ez, cb, 0, 1), run(ez, cg, 0, 4), run(ex, cb, 0, 5), run(ez, cb, 1, 1), run(ey, cb, 0, 4),
    run(ey, cr, 0, 5), run(ez, cb, 2, 1), run(ez, cr, 0, 5), run(ez, cb, 3, 1),
    // mode 7 (10010): 8-bit endpoints, deltas 6/5/5
    run(ew, cr, 0, 8), run(ez, cg, 4, 1), run(ey, cb, 4, 1), run(ew, cg, 0, 8), run(ez, cb, 2, 1),
    run(ey, cg, 4, 1), run(ew, cb, 0, 8), run(ez, cb, 3, 1), run(ez, cb, 4, 1), run(ex, cr, 0, 6),
    run(ey, cg, 0, 4), run(ex, cg, 0, 5), run(ez, cb, 0, 1), run(ez, cg, 0, 4), run(ex, cb, 0, 5),
    run(ez, cb, 1, 1), run(ey, cb, 0, 4), run(ey, cr, 0, 6), run(ez, cr, 0, 6),
    // mode 8 (10110): 8-bit endpoints, deltas 5/6/5
    run(ew, cr, 0, 8), run(ez, cb, 0, 1), run(ey, cb, 4, 1), run(ew, cg, 0, 8), run(ey, cg, 5, 1),
    run(ey, cg, 4, 1), run(ew, cb, 0, 8), run(ez, cg, 5, 1), run(ez, cb, 4, 1), run(ex, cr, 0, 5),
    run(ez, cg, 4, 1), run(ey, cg, 0, 4), run(ex, cg, 0, 6), run(ez, cg, 0, 4), run(ex, cb, 0, 5),
    run(ez, cb, 1, 1), run(ey, cb, 0, 4), run(ey, cr, 0, 5), run(ez, cb, 2, 1), run(ez, cr, 0, 5),
    run(ez, cb, 3, 1),
    // mode 9 (11010): 8-bit endpoints, deltas 5/5/6
    run(ew, cr, 0, 8), run(ez, cb, 1, 1), run(ey, cb, 4, 1), run(ew, cg, 0, 8), run(ey, cb, 5, 1),
    run(ey, cg, 4, 1), run(ew, cb, 0, 8), run(ez, cb, 5, 1), run(ez, cb, 4, 1), run(ex, cr, 0, 5),
    run(ez, cg, 4, 1), run(ey, cg, 0, 4), run(ex, cg, 0, 5), run(ez, cb, 0, 1), run(ez, cg, 0, 4),
    run(ex, cb, 0, 6), run(ey, cb, 0, 4), run(ey, cr, 0, 5), run(ez, cb, 2, 1), run(ez, cr, 0, 5),
    run(ez, cb, 3, 1),
    // mode 10 (11110): four explicit 6-bit endpoints
    run(ew, cr, 0, 6), run(ez, cg, 4, 1), run(ez, cb, 0, 1), run(ez, cb, 1, 1), run(ey, cb, 4, 1),
    run(ew, cg, 0, 6), run(ey, cg, 5, 1), run(ey, cb, 5, 1), run(ez, cb, 2, 1), run(ey, cg, 4, 1),
    run(ew, cb, 0, 6), run(ez, cg, 5, 1), run(ez, cb, 3, 1), run(ez, cb, 5, 1), run(ez, cb, 4, 1),
    run(ex, cr, 0, 6), run(ey, cg, 0, 4), run(ex, cg, 0, 6), run(ez, cg, 0, 4), run(ex, cb, 0, 6),
    run(ey, cb, 0, 4), run(ey, cr, 0, 6), run(ez, cr, 0, 6),
    // mode 11 (00011): one subset, two explicit 10-bit endpoints
    run(ew, cr, 0, 10), run(ew, cg, 0, 10), run(ew, cb, 0, 10), run(ex, cr, 0, 10), run(ex, cg, 0, 10),
    run(ex, cb, 0, 10),
    // mode 12 (00111): one subset, 11-bit endpoint, deltas 9
    run(ew, cr, 0, 10), run(ew, cg, 0, 10), run(ew, cb, 0, 10), run(ex, cr, 0, 9), run(ew, cr, 10, 1),
    run(ex, cg, 0, 9), run(ew, cg, 10, 1), run(ex, cb, 0, 9), run(ew, cb, 10, 1),
    // mode 13 (01011): one subset, 12-bit endpoint, deltas 8
    run(ew, cr, 0, 10), run(ew, cg, 0, 10), run(ew, cb, 0, 10), run(ex, cr, 0, 8), rev(ew, cr, 10, 2),
    run(ex, cg, 0, 8), rev(ew, cg, 10, 2), run(ex, cb, 0, 8), rev(ew, cb, 10, 2),
    // mode 14 (01111): one subset, 16-bit endpoint, deltas 4
    run(ew, cr, 0, 10), run(ew, cg, 0, 10), run(ew, cb, 0, 10), run(ex, cr, 0, 4), rev(ew, cr, 10, 6),
    run(ex, cg, 0, 4), rev(ew, cg, 10, 6), run(ex, cb, 0, 4), rev(ew, cb, 10, 6),
};

struct Mode {
  uint8_t two_subsets, transformed, epb;  // endpoint precision
  uint8_t delta[3];                       // delta precision per channel (transformed modes)
  uint8_t first, count;                   // runs in kRuns
};
__constant__ const Mode kModes[14] = {
    {1, 1, 10, {5, 5, 5}, 0, 19},   {1, 1, 7, {6, 6, 6}, 19, 23},    {1, 1, 11, {5, 4, 4}, 42, 18},
    {1, 1, 11, {4, 5, 4}, 60, 20},  {1, 1, 11, {4, 4, 5}, 80, 20},   {1, 1, 9, {5, 5, 5}, 100, 19},
    {1, 1, 8, {6, 5, 5}, 119, 19},  {1, 1, 8, {5, 6, 5}, 138, 21},   {1, 1, 8, {5, 5, 6}, 159, 21},
    {1, 0, 6, {6, 6, 6}, 180, 23},  {0, 0, 10, {10, 10, 10}, 203, 6}, {0, 1, 11, {9, 9, 9}, 209, 9},
    {0, 1, 12, {8, 8, 8}, 218, 9},  {0, 1, 16, {4, 4, 4}, 227, 9},
};
// Mode index of a 5-bit mode value (low two bits 10 or 11); 0xFF = reserved.
__constant__ const uint8_t kMode5[32] = {
    0xFF, 0xFF, 2, 10, 0xFF, 0xFF, 3, 11, 0xFF, 0xFF, 4, 12, 0xFF, 0xFF, 5, 13,
    0xFF, 0xFF, 6, 0xFF, 0xFF, 0xFF, 7, 0xFF, 0xFF, 0xFF, 8, 0xFF, 0xFF, 0xFF, 9, 0xFF};
// Two-subset partitions (the specification's shape table): bit i set = texel i in subset 1.
__constant__ const uint16_t kPartition[32] = {
    0xCCCC, 0x8888, 0xEEEE, 0xECC8, 0xC880, 0xFEEC, 0xFEC8, 0xEC80, 0xC800, 0xFFEC, 0xFE80,
    0xE800, 0xFFE8, 0xFF00, 0xFFF0, 0xF000, 0xF710, 0x008E, 0x7100, 0x08CE, 0x008C, 0x7310,
    0x3100, 0x8CCE, 0x088C, 0x3110, 0x6666, 0x366C, 0x17E8, 0x0FF0, 0x718E, 0x399C};
// Anchor texel of subset 1 per partition (subset 0's anchor is texel 0).
__constant__ const uint8_t kAnchor[32] = {15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15,
                                          15, 2,  8,  2,  2,  8,  8,  15, 2,  8,  2,  2,  8,  8,  2,  2};
__constant__ const uint8_t kWeights3[8] = {0, 9, 18, 27, 37, 46, 55, 64};
__constant__ const uint8_t kWeights4[16] = {0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64};

constexpr int kTexelsPerThread = 16;

__device__ __forceinline__ uint32_t block_bits(uint64_t lo, uint64_t hi, uint32_t pos, uint32_t n) {
  uint64_t v;
  if (pos >= 64) v = hi >> (pos - 64);
  else if (pos + n <= 64) v = lo >> pos;
  else v = (lo >> pos) | (hi << (64 - pos));
  return (uint32_t)(v & ((1ull << n) - 1));
}

__device__ __forceinline__ int32_t sign_extend(int32_t v, uint32_t bits) {
  const uint32_t s = 32 - bits;
  return (int32_t)((uint32_t)v << s) >> s;
}

__device__ __forceinline__ int32_t unquantize(int32_t c, uint32_t epb, bool is_signed) {
  if (!is_signed) {
    if (epb >= 15 || c == 0) return c;
    if (c == (1 << epb) - 1) return 0xFFFF;
    return ((c << 16) + 0x8000) >> epb;
  }
  if (epb >= 16) return c;
  const bool neg = c < 0;
  int32_t m = neg ? -c : c, u;
  if (m == 0) u = 0;
  else if (m >= (1 << (epb - 1)) - 1) u = 0x7FFF;
  else u = ((m << 15) + 0x4000) >> (epb - 1);
  return neg ? -u : u;
}

__device__ __forceinline__ float finish(int32_t v, bool is_signed) {
  uint16_t h;
  if (!is_signed) h = (uint16_t)((v * 31) >> 6);
  else h = v < 0 ? (uint16_t)(0x8000 | ((-v * 31) >> 5)) : (uint16_t)((v * 31) >> 5);
  return __half2float(__ushort_as_half(h));
}

// One thread decodes one 4x4 block of one layer into RGBA32F texels (alpha 1); texels past
// width / height (a partial edge block) are not written.
__global__ void k_decode_bc6h(const uint4* __restrict__ blocks, uint32_t width, uint32_t height, uint32_t layers,
                              uint32_t is_signed_u, float4* __restrict__ out) {
  const uint32_t bw = (width + 3) / 4, bh = (height + 3) / 4;
  const uint64_t n_blocks = (uint64_t)bw * bh * layers;
  const bool is_signed = is_signed_u != 0;
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < n_blocks;
       b += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 q = blocks[b];
    const uint64_t lo = (uint64_t)q.x | (uint64_t)q.y << 32, hi = (uint64_t)q.z | (uint64_t)q.w << 32;
    const uint32_t layer = (uint32_t)(b / ((uint64_t)bw * bh)), rem = (uint32_t)(b % ((uint64_t)bw * bh));
    const uint32_t x0 = (rem % bw) * 4, y0 = (rem / bw) * 4;
    float4* dst = out + (size_t)layer * width * height;
    const uint32_t m2 = (uint32_t)(lo & 3);
    const uint32_t mi = m2 < 2 ? m2 : kMode5[lo & 31];
    if (mi == 0xFF) {
      for (int i = 0; i < kTexelsPerThread; ++i) {
        const uint32_t x = x0 + (i & 3), y = y0 + (i >> 2);
        if (x < width && y < height) dst[(size_t)y * width + x] = make_float4(0.f, 0.f, 0.f, 1.f);
      }
      continue;
    }
    const Mode md = kModes[mi];
    int32_t ep[4][3] = {};
    uint32_t pos = m2 < 2 ? 2 : 5;
    for (uint32_t r = md.first; r < (uint32_t)md.first + md.count; ++r) {
      const uint32_t code = kRuns[r], n = code & 31, lo_bit = (code >> 5) & 31;
      uint32_t v = block_bits(lo, hi, pos, n);
      pos += n;
      if (code >> 14) v = __brev(v) >> (32 - n);
      ep[(code >> 12) & 3][(code >> 10) & 3] |= (int32_t)(v << lo_bit);
    }
    uint32_t part = 0;
    if (md.two_subsets) {
      part = block_bits(lo, hi, pos, 5);
      pos += 5;
    }
    const int n_ep = md.two_subsets ? 4 : 2;
    const int32_t mask = (int32_t)((1u << md.epb) - 1);
    int32_t unq[4][3];
    for (int c = 0; c < 3; ++c) {
      if (is_signed) ep[0][c] = sign_extend(ep[0][c], md.epb);
      for (int e = 1; e < n_ep; ++e) {
        if (md.transformed) {
          ep[e][c] = (ep[0][c] + sign_extend(ep[e][c], md.delta[c])) & mask;
          if (is_signed) ep[e][c] = sign_extend(ep[e][c], md.epb);
        } else if (is_signed) {
          ep[e][c] = sign_extend(ep[e][c], md.epb);
        }
      }
      for (int e = 0; e < n_ep; ++e) unq[e][c] = unquantize(ep[e][c], md.epb, is_signed);
    }
    const uint32_t ib = md.two_subsets ? 3 : 4;
    const uint32_t anchor = md.two_subsets ? kAnchor[part] : 0;
    const uint32_t shape = md.two_subsets ? kPartition[part] : 0;
    for (uint32_t i = 0; i < (uint32_t)kTexelsPerThread; ++i) {
      const uint32_t nb = ib - ((i == 0 || (md.two_subsets && i == anchor)) ? 1 : 0);
      const uint32_t idx = block_bits(lo, hi, pos, nb);
      pos += nb;
      const int32_t w = md.two_subsets ? kWeights3[idx] : kWeights4[idx];
      const uint32_t s = (shape >> i) & 1;
      float rgb[3];
      for (int c = 0; c < 3; ++c) {
        const int32_t v = (unq[2 * s][c] * (64 - w) + unq[2 * s + 1][c] * w + 32) >> 6;
        rgb[c] = finish(v, is_signed);
      }
      const uint32_t x = x0 + (i & 3), y = y0 + (i >> 2);
      if (x < width && y < height) dst[(size_t)y * width + x] = make_float4(rgb[0], rgb[1], rgb[2], 1.f);
    }
  }
}

}  // namespace

int decode_bc6h_device(const void* d_blocks, uint32_t width, uint32_t height, uint32_t layers, bool is_signed,
                       float4* d_out, cudaStream_t stream) {
  const uint64_t n_blocks = (uint64_t)((width + 3) / 4) * ((height + 3) / 4) * layers;
  if (n_blocks == 0) return NB_OK;
  const int threads = 256;
  const uint64_t want = (n_blocks + threads - 1) / threads;
  const int grid = (int)std::min<uint64_t>(want, (uint64_t)sm_count() * 16);
  k_decode_bc6h<<<grid, threads, 0, stream>>>((const uint4*)d_blocks, width, height, layers, is_signed ? 1u : 0u,
                                               d_out);
  NB_CUDA(cudaGetLastError(), "k_decode_bc6h");
  return NB_OK;
}


// ---- DDS cube maps -------------------------------------------------------------------------
// Microsoft's DDS layout: "DDS " magic; a 124-byte DDS_HEADER (size, flags, height, width,
// pitch, depth, mip count, 11 reserved words, the 32-byte DDS_PIXELFORMAT at byte 76 with its
// flags at 80 and FourCC at 84, caps 1-4 at 108-120); for FourCC "DX10" a 20-byte
// DDS_HEADER_DXT10 at byte 128 (DXGI format, resource dimension, misc flags - 0x4 for a cube -,
// array size, misc flags 2); then each array layer's mip chain in turn.
namespace {
constexpr uint32_t kDxgiRgba32f = 2, kDxgiRgba16f = 10, kDxgiBc6hUf16 = 95, kDxgiBc6hSf16 = 96;
constexpr uint32_t kD3dfmtRgba16f = 113, kD3dfmtRgba32f = 116;
constexpr uint32_t kDdpfFourcc = 0x4, kDdsCaps2Cubemap = 0x200;
constexpr uint32_t kMaxFace = 32768;

uint32_t le32(const uint8_t* p) { return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; }
}  // namespace

int parse_dds_cube(const uint8_t* p, size_t n, DdsCube* out) {
  if (n < 128 || std::memcmp(p, "DDS ", 4) != 0) return fail(NB_ERR_INVALID_ARG, "not a DDS file");
  if (le32(p + 4) != 124) return fail(NB_ERR_INVALID_ARG, "DDS header size %u != 124", le32(p + 4));
  const uint32_t height = le32(p + 12), width = le32(p + 16);
  const uint32_t mips = std::max(1u, le32(p + 28));
  const uint32_t pf_flags = le32(p + 80), fourcc = le32(p + 84), caps2 = le32(p + 112);
  size_t offset = 128;
  if ((pf_flags & kDdpfFourcc) && std::memcmp(p + 84, "DX10", 4) == 0) {
    if (n < 148) return fail(NB_ERR_INVALID_ARG, "DDS file truncated in its DX10 header");
    const uint32_t dxgi = le32(p + 128);
    offset = 148;
    // Six array layers whatever the header says, as texture.rs:95-96 forces them.
    if (dxgi == kDxgiBc6hUf16) out->format = kDdsBc6hUf16;
    else if (dxgi == kDxgiBc6hSf16) out->format = kDdsBc6hSf16;
    else if (dxgi == kDxgiRgba16f) out->format = kDdsRgba16f;
    else if (dxgi == kDxgiRgba32f) out->format = kDdsRgba32f;
    else return fail(NB_ERR_INVALID_ARG, "DDS DXGI format %u is not supported (BC6H_UF16, BC6H_SF16, "
                     "R16G16B16A16_FLOAT or R32G32B32A32_FLOAT)", dxgi);
  } else if (pf_flags & kDdpfFourcc) {
    if (fourcc == kD3dfmtRgba16f) out->format = kDdsRgba16f;
    else if (fourcc == kD3dfmtRgba32f) out->format = kDdsRgba32f;
    else return fail(NB_ERR_INVALID_ARG, "DDS FourCC 0x%08x is not supported", fourcc);
    if (!(caps2 & kDdsCaps2Cubemap)) return fail(NB_ERR_INVALID_ARG, "DDS file is not a cube map");
  } else {
    return fail(NB_ERR_INVALID_ARG, "DDS file without a FourCC pixel format is not supported");
  }
  if (width == 0 || width != height || width > kMaxFace)
    return fail(NB_ERR_INVALID_ARG, "cube faces must be square, 1 to %u texels (%u x %u)", kMaxFace, width, height);
  if (mips > 32) return fail(NB_ERR_INVALID_ARG, "DDS mip count %u", mips);
  const bool bc = out->format == kDdsBc6hUf16 || out->format == kDdsBc6hSf16;
  const uint64_t texel = out->format == kDdsRgba32f ? 16 : 8;
  uint64_t chain = 0, level0 = 0;
  for (uint32_t m = 0; m < mips; ++m) {
    const uint64_t w = std::max(1u, width >> m), h = std::max(1u, height >> m);
    const uint64_t bytes = bc ? ((w + 3) / 4) * ((h + 3) / 4) * 16 : w * h * texel;
    if (m == 0) level0 = bytes;
    chain += bytes;
  }
  if ((uint64_t)n < offset + 6 * chain)
    return fail(NB_ERR_INVALID_ARG, "DDS file truncated: %zu bytes, %llu expected", n,
                (unsigned long long)(offset + 6 * chain));
  out->size = width;
  out->face_bytes = (size_t)level0;
  for (int f = 0; f < 6; ++f) out->face[f] = p + offset + (size_t)f * chain;
  return NB_OK;
}

}  // namespace nb

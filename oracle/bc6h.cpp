// CPU oracle of BC6H block decoding (TEST INFRASTRUCTURE ONLY: loaded by tests/ to check the
// library's device decoder against; the product never links or calls it).
//
// The reference samples its environment from a BC6H_UF16 cube texture (texture.rs:89-94,
// pathtracing.wgsl:168) and leaves the decoding to the graphics hardware, so the reference
// decoder is the texture unit's.  This file restates the published format (Direct3D 11 "BC6H
// format"; Khronos Data Format Specification, "BC6H") and is pinned against the GB300 texture
// unit's own BC6H decode by the fixtures under tests/golden/ (bc6h_texunit.npz) and by a GPU
// test that decodes fresh random blocks both ways.
//
// Written independently of the device decoder: the endpoint layouts are kept here as the
// specification writes them (e.g. "gy4 by4 bz4 rw9:0 ..."; a token "cAB" names channel c of
// endpoint A (w, x: subset 0; y, z: subset 1) and B is a bit or a range hi:lo whose right-hand
// bit sits at the lower block position, so "rw10:11" stores bit 11 first), and the block is
// read one bit at a time.  Output is half-float bits per texel and channel.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct ModeSpec {
  int mode_bits;      // 2 or 5
  unsigned value;     // mode value
  int subsets;        // 1 or 2
  bool transformed;   // endpoints 1.. are deltas of endpoint 0
  int precision;      // endpoint bits
  int delta[3];       // delta bits (r, g, b)
  const char* layout;
};

const ModeSpec kSpecs[14] = {
    {2, 0x00, 2, true, 10, {5, 5, 5},
     "gy4 by4 bz4 rw9:0 gw9:0 bw9:0 rx4:0 gz4 gy3:0 gx4:0 bz0 gz3:0 bx4:0 bz1 by3:0 ry4:0 bz2 rz4:0 bz3"},
    {2, 0x01, 2, true, 7, {6, 6, 6},
     "gy5 gz4 gz5 rw6:0 bz0 bz1 by4 gw6:0 by5 bz2 gy4 bw6:0 bz3 bz5 bz4 rx5:0 gy3:0 gx5:0 gz3:0 bx5:0 by3:0 "
     "ry5:0 rz5:0"},
    {5, 0x02, 2, true, 11, {5, 4, 4},
     "rw9:0 gw9:0 bw9:0 rx4:0 rw10 gy3:0 gx3:0 gw10 bz0 gz3:0 bx3:0 bw10 bz1 by3:0 ry4:0 bz2 rz4:0 bz3"},
    {5, 0x06, 2, true, 11, {4, 5, 4},
     "rw9:0 gw9:0 bw9:0 rx3:0 rw10 gz4 gy3:0 gx4:0 gw10 gz3:0 bx3:0 bw10 bz1 by3:0 ry3:0 bz0 bz2 rz3:0 gy4 bz3"},
    {5, 0x0A, 2, true, 11, {4, 4, 5},
     "rw9:0 gw9:0 bw9:0 rx3:0 rw10 by4 gy3:0 gx3:0 gw10 bz0 gz3:0 bx4:0 bw10 by3:0 ry3:0 bz1 bz2 rz3:0 bz4 bz3"},
    {5, 0x0E, 2, true, 9, {5, 5, 5},
     "rw8:0 by4 gw8:0 gy4 bw8:0 bz4 rx4:0 gz4 gy3:0 gx4:0 bz0 gz3:0 bx4:0 bz1 by3:0 ry4:0 bz2 rz4:0 bz3"},
    {5, 0x12, 2, true, 8, {6, 5, 5},
     "rw7:0 gz4 by4 gw7:0 bz2 gy4 bw7:0 bz3 bz4 rx5:0 gy3:0 gx4:0 bz0 gz3:0 bx4:0 bz1 by3:0 ry5:0 rz5:0"},
    {5, 0x16, 2, true, 8, {5, 6, 5},
     "rw7:0 bz0 by4 gw7:0 gy5 gy4 bw7:0 gz5 bz4 rx4:0 gz4 gy3:0 gx5:0 gz3:0 bx4:0 bz1 by3:0 ry4:0 bz2 rz4:0 "
     "bz3"},
    {5, 0x1A, 2, true, 8, {5, 5, 6},
     "rw7:0 bz1 by4 gw7:0 by5 gy4 bw7:0 bz5 bz4 rx4:0 gz4 gy3:0 gx4:0 bz0 gz3:0 bx5:0 by3:0 ry4:0 bz2 rz4:0 "
     "bz3"},
    {5, 0x1E, 2, false, 6, {6, 6, 6},
     "rw5:0 gz4 bz0 bz1 by4 gw5:0 gy5 by5 bz2 gy4 bw5:0 gz5 bz3 bz5 bz4 rx5:0 gy3:0 gx5:0 gz3:0 bx5:0 by3:0 "
     "ry5:0 rz5:0"},
    {5, 0x03, 1, false, 10, {10, 10, 10}, "rw9:0 gw9:0 bw9:0 rx9:0 gx9:0 bx9:0"},
    {5, 0x07, 1, true, 11, {9, 9, 9}, "rw9:0 gw9:0 bw9:0 rx8:0 rw10 gx8:0 gw10 bx8:0 bw10"},
    {5, 0x0B, 1, true, 12, {8, 8, 8}, "rw9:0 gw9:0 bw9:0 rx7:0 rw10:11 gx7:0 gw10:11 bx7:0 bw10:11"},
    {5, 0x0F, 1, true, 16, {4, 4, 4}, "rw9:0 gw9:0 bw9:0 rx3:0 rw10:15 gx3:0 gw10:15 bx3:0 bw10:15"},
};

// One block bit as (endpoint, channel, bit of that endpoint channel).
struct BitDest {
  int endpoint, channel, bit;
};

std::vector<BitDest> expand(const char* layout) {
  std::vector<BitDest> out;
  const char* p = layout;
  while (*p) {
    while (*p == ' ') ++p;
    if (!*p) break;
    const int channel = *p == 'r' ? 0 : *p == 'g' ? 1 : 2;
    ++p;
    const int endpoint = *p - 'w';  // w x y z -> 0 1 2 3
    ++p;
    int hi = 0, lo;
    while (*p >= '0' && *p <= '9') hi = hi * 10 + (*p++ - '0');
    lo = hi;
    if (*p == ':') {
      ++p;
      lo = 0;
      while (*p >= '0' && *p <= '9') lo = lo * 10 + (*p++ - '0');
    }
    // the right-hand bit sits at the lowest block position
    const int step = hi >= lo ? 1 : -1;
    for (int b = lo;; b += step) {
      out.push_back({endpoint, channel, b});
      if (b == hi) break;
    }
  }
  return out;
}

const int kPartitions[32][16] = {
    {0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1}, {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1},
    {0, 1, 1, 1, 0, 1, 1, 1, 0, 1, 1, 1, 0, 1, 1, 1}, {0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 1, 1, 0, 1, 1, 1},
    {0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 1, 1}, {0, 0, 1, 1, 0, 1, 1, 1, 0, 1, 1, 1, 1, 1, 1, 1},
    {0, 0, 0, 1, 0, 0, 1, 1, 0, 1, 1, 1, 1, 1, 1, 1}, {0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 1, 1, 0, 1, 1, 1},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 1, 1}, {0, 0, 1, 1, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
    {0, 0, 0, 0, 0, 0, 0, 1, 0, 1, 1, 1, 1, 1, 1, 1}, {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 1, 1, 1},
    {0, 0, 0, 1, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1}, {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1},
    {0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1}, {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1},
    {0, 0, 0, 0, 1, 0, 0, 0, 1, 1, 1, 0, 1, 1, 1, 1}, {0, 1, 1, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 1, 1, 1, 0}, {0, 1, 1, 1, 0, 0, 1, 1, 0, 0, 0, 1, 0, 0, 0, 0},
    {0, 0, 1, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 1, 0, 0, 0, 1, 1, 0, 0, 1, 1, 1, 0},
    {0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 1, 1, 0, 0}, {0, 1, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 0, 1},
    {0, 0, 1, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 0}, {0, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 1, 0, 0},
    {0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1, 0}, {0, 0, 1, 1, 0, 1, 1, 0, 0, 1, 1, 0, 1, 1, 0, 0},
    {0, 0, 0, 1, 0, 1, 1, 1, 1, 1, 1, 0, 1, 0, 0, 0}, {0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0},
    {0, 1, 1, 1, 0, 0, 0, 1, 1, 0, 0, 0, 1, 1, 1, 0}, {0, 0, 1, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1, 1, 0, 0},
};
const int kFixup[32] = {15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15,
                        15, 2,  8,  2,  2,  8,  8,  15, 2,  8,  2,  2,  8,  8,  2,  2};
const int kW3[8] = {0, 9, 18, 27, 37, 46, 55, 64};
const int kW4[16] = {0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64};

struct BitReader {
  const uint8_t* b;
  int pos = 0;
  int bit() {
    const int v = (b[pos >> 3] >> (pos & 7)) & 1;
    ++pos;
    return v;
  }
  int bits(int n) {
    int v = 0;
    for (int i = 0; i < n; ++i) v |= bit() << i;
    return v;
  }
};

int sext(int v, int n) { return (v & (1 << (n - 1))) ? v - (1 << n) : v; }

int unquant(int c, int prec, bool sgn) {
  if (!sgn) {
    if (prec >= 15) return c;
    if (c == 0) return 0;
    if (c == (1 << prec) - 1) return 0xFFFF;
    return ((c << 16) + 0x8000) >> prec;
  }
  if (prec >= 16) return c;
  int s = 0;
  if (c < 0) {
    s = 1;
    c = -c;
  }
  int u;
  if (c == 0) u = 0;
  else if (c >= (1 << (prec - 1)) - 1) u = 0x7FFF;
  else u = ((c << 15) + 0x4000) >> (prec - 1);
  return s ? -u : u;
}

uint16_t to_half_bits(int v, bool sgn) {
  if (!sgn) return (uint16_t)((v * 31) >> 6);
  if (v < 0) return (uint16_t)(0x8000 | (((-v) * 31) >> 5));
  return (uint16_t)((v * 31) >> 5);
}

void decode_block(const uint8_t* block, bool sgn, uint16_t* out /* 16 x 3 */) {
  static const std::vector<std::vector<BitDest>> layouts = [] {
    std::vector<std::vector<BitDest>> v;
    for (int m = 0; m < 14; ++m) v.push_back(expand(kSpecs[m].layout));
    return v;
  }();
  BitReader r{block};
  int mode = -1;
  const int two = r.bits(2);
  if (two < 2) {
    mode = two;
  } else {
    const unsigned v = (unsigned)two | (unsigned)r.bits(3) << 2;
    for (int m = 2; m < 14; ++m)
      if (kSpecs[m].value == v) mode = m;
  }
  if (mode < 0) {
    std::memset(out, 0, 16 * 3 * sizeof(uint16_t));
    return;
  }
  const ModeSpec& M = kSpecs[mode];
  int e[4][3] = {};
  for (const BitDest& d : layouts[mode]) e[d.endpoint][d.channel] |= r.bit() << d.bit;
  const int part = M.subsets == 2 ? r.bits(5) : 0;
  const int n_end = 2 * M.subsets;
  for (int c = 0; c < 3; ++c) {
    if (sgn) e[0][c] = sext(e[0][c], M.precision);
    for (int k = 1; k < n_end; ++k) {
      if (M.transformed) {
        e[k][c] = (e[0][c] + sext(e[k][c], M.delta[c])) & ((1 << M.precision) - 1);
        if (sgn) e[k][c] = sext(e[k][c], M.precision);
      } else if (sgn) {
        e[k][c] = sext(e[k][c], M.precision);
      }
    }
  }
  int u[4][3];
  for (int k = 0; k < n_end; ++k)
    for (int c = 0; c < 3; ++c) u[k][c] = unquant(e[k][c], M.precision, sgn);
  const int index_bits = M.subsets == 2 ? 3 : 4;
  for (int t = 0; t < 16; ++t) {
    const bool anchor = t == 0 || (M.subsets == 2 && t == kFixup[part]);
    const int idx = r.bits(index_bits - (anchor ? 1 : 0));
    const int w = M.subsets == 2 ? kW3[idx] : kW4[idx];
    const int s = M.subsets == 2 ? kPartitions[part][t] : 0;
    for (int c = 0; c < 3; ++c) {
      const int v = (u[2 * s][c] * (64 - w) + u[2 * s + 1][c] * w + 32) >> 6;
      out[t * 3 + c] = to_half_bits(v, sgn);
    }
  }
}

float half_to_float(uint16_t h) {
  const int s = h >> 15, ex = (h >> 10) & 31, m = h & 1023;
  float v;
  if (ex == 0) v = std::ldexp((float)m, -24);
  else if (ex == 31) v = m ? NAN : INFINITY;
  else v = std::ldexp((float)(1024 + m), ex - 25);
  return s ? -v : v;
}

}  // namespace

extern "C" {

// Half-float bits of the 16 texels (row-major in the block) x RGB of n blocks.
void or_bc6h_decode_blocks(const uint8_t* blocks, size_t n, int is_signed, uint16_t* out) {
  for (size_t i = 0; i < n; ++i) decode_block(blocks + 16 * i, is_signed != 0, out + 48 * i);
}

// layers x height x width RGBA32F texels (alpha 1) from layers x ceil(h/4) x ceil(w/4) blocks.
void or_bc6h_decode(const uint8_t* blocks, uint32_t width, uint32_t height, uint32_t layers, int is_signed,
                    float* out) {
  const uint32_t bw = (width + 3) / 4, bh = (height + 3) / 4;
  uint16_t h[48];
  for (uint32_t l = 0; l < layers; ++l)
    for (uint32_t by = 0; by < bh; ++by)
      for (uint32_t bx = 0; bx < bw; ++bx) {
        decode_block(blocks + 16 * (((size_t)l * bh + by) * bw + bx), is_signed != 0, h);
        for (int t = 0; t < 16; ++t) {
          const uint32_t x = bx * 4 + (t & 3), y = by * 4 + (t >> 2);
          if (x >= width || y >= height) continue;
          float* o = out + (((size_t)l * height + y) * width + x) * 4;
          for (int c = 0; c < 3; ++c) o[c] = half_to_float(h[t * 3 + c]);
          o[3] = 1.0f;
        }
      }
}

}  // extern "C"

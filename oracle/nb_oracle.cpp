// CPU oracle for the nBounce path-tracing pass.
//
// TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg load this library as the reference for parity checks.  The product (nbounce_gb300)
// never links, loads or calls it.
//
// This file restates, operation for operation, the reference algorithm of julcst/nbounce:
//   src/pathtracing/common.wgsl         PCG4D hash, map4f, luminance, build_tbn
//   src/pathtracing/raytracing_sw.wgsl  Moller-Trumbore, slab test, TLAS/BLAS stack traversal,
//                                       hit attribute interpolation
//   src/pathtracing/pathtracing.wgsl    generate_ray, VNDF / cosine sampling, Fresnel, Lambda,
//                                       lobe choice, Russian roulette, running-mean accumulate
//   src/pathtracing/bvh.rs              binned / brute-force SAH builder, node layout
//   src/pathtracing/scene.rs:220-305    instance records, 8-corner bounds, BLAS/TLAS assembly
// plus a Sobol-Burley sample table after Burley 2020 ("Practical Hash-based Owen
// Scrambling", JCGT 9(4)) for the sobol_burley 0.5.0 crate the reference calls at
// src/pathtracing/pathtracer.rs:62-64 (the crate itself is not part of the reference tree).
//
// Arithmetic contract (shared with the CUDA kernels by specification, not by code):
// every WGSL expression is evaluated left to right in IEEE binary32, round to nearest,
// with no contraction (this file is compiled with -ffp-contract=off).  WGSL builtins whose
// precision the WGSL spec leaves open are pinned as follows:
//   dot(a,b)      = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a,b)    = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
//   normalize(v)  = v / sqrt(dot(v,v))    (correctly rounded sqrt and division)
//   M * v         = ((M[0]*v.x + M[1]*v.y) + M[2]*v.z) (+ M[3]*v.w)
//   mix(a,b,t)    = a*(1-t) + b*t
//   min/max       = IEEE 754-2019 minimumNumber/maximumNumber (NaN ignored, -0 < +0)
//   pow(x, n)     = repeated multiplication for the integral exponents the pass uses (2, 5, 8)
//   sin/cos       = Cody-Waite reduction by pi/2 (three-part split) + Taylor polynomials of
//                   degree 9 / 10 on [-pi/4, pi/4], Horner form, no fusion
//   out-of-range Sobol table reads return 0 (robust buffer access).
// The FP64 "truth" render evaluates the same algorithm in binary64 with libm sin/cos.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <thread>
#include <type_traits>
#include <vector>

#include "joe_kuo_68.inc"

namespace {

// ---------------------------------------------------------------------------------------
// scalar helpers
// ---------------------------------------------------------------------------------------
template <class R> static inline R wmin(R a, R b) {
  if (a != a) return b;
  if (b != b) return a;
  if (a < b) return a;
  if (b < a) return b;
  return std::signbit(a) ? a : b;
}
template <class R> static inline R wmax(R a, R b) {
  if (a != a) return b;
  if (b != b) return a;
  if (a > b) return a;
  if (b > a) return b;
  return std::signbit(a) ? b : a;
}
// Rust `f32 as u32`: saturating, NaN -> 0
static inline uint32_t sat_u32(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
}
static inline float bits_f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

constexpr float kMaxFloat = 3.40282346638528859812e+38f;  // 0x1.fffffep+127f
constexpr float kNoHit = kMaxFloat;
constexpr float kEps = 0.00000001f;
constexpr float kBias = 0.1f;
constexpr float kPi = 3.14159265359f;
constexpr float kTwoPi = 2.0f * kPi;
constexpr uint32_t kLdsPerBounce = 2u;
constexpr uint32_t kLdsStride = 8u * kLdsPerBounce + 1u;  // pathtracing.wgsl:4, fixed at 17
constexpr int kStackSize = 64;  // reference uses 32 (raytracing_sw.wgsl:5-6); overflow is flagged

// ---------------------------------------------------------------------------------------
// deterministic sin/cos (binary32), see header comment
// ---------------------------------------------------------------------------------------
// pi/2 split into three binary32 parts whose leading parts have short significands so that
// k*A and k*B are exact for the small k reached here (|x| < 64).
constexpr float kPio2A = 1.5703125f;                   // 201/128
constexpr float kPio2B = 0x1.fb6p-12f;                 // 12 significant bits
constexpr float kPio2C = -0x1.777a5cp-25f;              // pi/2 - A - B, rounded
constexpr float kTwoOverPi = 0.636619772367581343f;   // rounds to 0x1.45f306p-1
// Taylor coefficients 1/n! rounded to binary32
constexpr float kS3 = -1.0f / 6.0f, kS5 = 1.0f / 120.0f, kS7 = -1.0f / 5040.0f, kS9 = 1.0f / 362880.0f;
constexpr float kC2 = -0.5f, kC4 = 1.0f / 24.0f, kC6 = -1.0f / 720.0f, kC8 = 1.0f / 40320.0f,
                kC10 = -1.0f / 3628800.0f;

static inline void sincos_f32(float x, float* s, float* c) {
  float kf = std::floor(x * kTwoOverPi + 0.5f);
  int k = (int)kf;
  float r = ((x - kf * kPio2A) - kf * kPio2B) - kf * kPio2C;
  float r2 = r * r;
  float ps = r + r * r2 * (kS3 + r2 * (kS5 + r2 * (kS7 + r2 * kS9)));
  float pc = 1.0f + r2 * (kC2 + r2 * (kC4 + r2 * (kC6 + r2 * (kC8 + r2 * kC10))));
  switch (k & 3) {
    case 0: *s = ps; *c = pc; break;
    case 1: *s = pc; *c = -ps; break;
    case 2: *s = -ps; *c = -pc; break;
    default: *s = -pc; *c = ps; break;
  }
}
static inline void sincos_r(float x, float* s, float* c) { sincos_f32(x, s, c); }
static inline void sincos_r(double x, double* s, double* c) { *s = std::sin(x); *c = std::cos(x); }

// ---------------------------------------------------------------------------------------
// vectors
// ---------------------------------------------------------------------------------------
template <class R> struct V3 { R x, y, z; };
template <class R> static inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> static inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> static inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> static inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> static inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> static inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> static inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> static inline V3<R> operator/(V3<R> a, V3<R> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class R> static inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> static inline V3<R> cross(V3<R> a, V3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> static inline V3<R> normalize(V3<R> v) {
  R l = std::sqrt(dot(v, v));
  return {v.x / l, v.y / l, v.z / l};
}
template <class R> static inline V3<R> vmin(V3<R> a, V3<R> b) { return {wmin(a.x, b.x), wmin(a.y, b.y), wmin(a.z, b.z)}; }
template <class R> static inline V3<R> vmax(V3<R> a, V3<R> b) { return {wmax(a.x, b.x), wmax(a.y, b.y), wmax(a.z, b.z)}; }
template <class R> static inline R luminance(V3<R> c) { return R(0.2126f) * c.x + R(0.7152f) * c.y + R(0.0722f) * c.z; }
template <class R> static inline R pow2(R x) { return x * x; }
template <class R> static inline R pow5(R x) { R x2 = x * x; return x2 * x2 * x; }
template <class R> static inline R pow8(R x) { R x2 = x * x; R x4 = x2 * x2; return x4 * x4; }
template <class R> static inline V3<R> cvt3(const float* p) { return {R(p[0]), R(p[1]), R(p[2])}; }
template <class R> static inline V3<R> reflect(V3<R> i, V3<R> n) { return i - (R(2) * dot(n, i)) * n; }

// column-major mat4 as 16 floats: column c = m[4c..4c+3]
template <class R> static inline V3<R> col3(const float* m, int c) { return {R(m[4 * c]), R(m[4 * c + 1]), R(m[4 * c + 2])}; }
// mat3(M) * v
template <class R> static inline V3<R> mat3_mul(const float* m, V3<R> v) {
  return col3<R>(m, 0) * v.x + col3<R>(m, 1) * v.y + col3<R>(m, 2) * v.z;
}
// transpose(mat3(M)) * v
template <class R> static inline V3<R> mat3t_mul(const float* m, V3<R> v) {
  return {dot(col3<R>(m, 0), v), dot(col3<R>(m, 1), v), dot(col3<R>(m, 2), v)};
}

// ---------------------------------------------------------------------------------------
// common.wgsl
// ---------------------------------------------------------------------------------------
static inline void hash4u(const uint32_t s[4], uint32_t v[4]) {  // common.wgsl:27-33
  for (int i = 0; i < 4; ++i) v[i] = s[i] * 1664525u + 1013904223u;
  v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2];
  for (int i = 0; i < 4; ++i) v[i] ^= v[i] >> 16u;
  v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2];
}
static inline void hash4f(const uint32_t s[4], float out[4]) {  // common.wgsl:7-9,39-41
  uint32_t h[4];
  hash4u(s, h);
  for (int i = 0; i < 4; ++i) out[i] = bits_f((h[i] >> 9u) | 0x3F800000u) - 1.0f;
}

// ---------------------------------------------------------------------------------------
// Sobol-Burley (Burley 2020): Joe-Kuo Sobol + nested uniform (Owen) scrambling through a
// Laine-Karras style hash on reversed bits + index shuffling.
// ---------------------------------------------------------------------------------------
struct SobolDirs {
  uint32_t v[68][32];
  SobolDirs() {
    for (int k = 0; k < 32; ++k) v[0][k] = 1u << (31 - k);
    for (int j = 1; j < 68; ++j) {
      uint32_t p = kJoeKuoPoly[j];
      int s = 31 - __builtin_clz(p);
      uint32_t a = (p >> 1) & ((1u << (s - 1)) - 1u);
      uint64_t m[33];
      for (int k = 1; k <= s; ++k) m[k] = kJoeKuoM[j][k - 1];
      for (int k = s + 1; k <= 32; ++k) {
        uint64_t x = m[k - s] ^ (m[k - s] << s);
        for (int i = 1; i < s; ++i)
          if ((a >> (s - 1 - i)) & 1u) x ^= m[k - i] << i;
        m[k] = x;
      }
      for (int k = 1; k <= 32; ++k) v[j][k - 1] = (uint32_t)((m[k] << (32 - k)) & 0xFFFFFFFFull);
    }
  }
};
static const SobolDirs& sobol_dirs() { static SobolDirs d; return d; }

static inline uint32_t reverse_bits(uint32_t x) {
  x = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
  x = ((x >> 2) & 0x33333333u) | ((x & 0x33333333u) << 2);
  x = ((x >> 4) & 0x0F0F0F0Fu) | ((x & 0x0F0F0F0Fu) << 4);
  x = ((x >> 8) & 0x00FF00FFu) | ((x & 0x00FF00FFu) << 8);
  return (x >> 16) | (x << 16);
}
// Laine-Karras permutation with the multipliers published in Burley 2020, listing 2
static inline uint32_t lk_permute(uint32_t x, uint32_t seed) {
  x += seed;
  x ^= x * 0x6c50b47cu;
  x ^= x * 0xb82f1e52u;
  x ^= x * 0xc7afe638u;
  x ^= x * 0x8d22f6e6u;
  return x;
}
static inline uint32_t nested_uniform_scramble(uint32_t x, uint32_t seed) {
  return reverse_bits(lk_permute(reverse_bits(x), seed));
}
// "lowbias32" integer hash (C. Wellons, hash-prospector, public domain) for seed derivation
static inline uint32_t hash_u32(uint32_t x) {
  x ^= x >> 16; x *= 0x7feb352du;
  x ^= x >> 15; x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
static inline uint32_t sobol_u32(uint32_t index, int dim) {
  const SobolDirs& d = sobol_dirs();
  uint32_t x = 0;
  for (int k = 0; index; ++k, index >>= 1)
    if (index & 1u) x ^= d.v[dim][k];
  return x;
}
static void sobol_burley_4d(uint32_t index, uint32_t dimset, uint32_t seed, float out[4]) {
  uint32_t sidx = nested_uniform_scramble(index, hash_u32(dimset ^ hash_u32(seed)));
  for (int k = 0; k < 4; ++k) {
    uint32_t dim = 4u * dimset + (uint32_t)k;
    uint32_t x = sobol_u32(sidx, (int)dim);
    x = nested_uniform_scramble(x, hash_u32(dim ^ 0x9e3779b9u ^ hash_u32(seed ^ 0x85ebca6bu)));
    out[k] = (float)(x >> 8) * (1.0f / 16777216.0f);
  }
}

// ---------------------------------------------------------------------------------------
// bvh.rs
// ---------------------------------------------------------------------------------------
struct Node { float mn[3]; uint32_t start; float mx[3]; uint32_t end; };  // bvh.rs:15-24
static_assert(sizeof(Node) == 32, "node layout");
struct Prim { float c[3]; float mn[3]; float mx[3]; uint32_t payload; };

static inline bool finite3(const float e[3]) {
  return std::isfinite(e[0]) && std::isfinite(e[1]) && std::isfinite(e[2]);
}
static inline float sah_area_cost(const float mn[3], const float mx[3], uint32_t count) {
  float e[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
  if (!finite3(e)) return std::numeric_limits<float>::infinity();
  float area = e[0] * e[1] + e[0] * e[2] + e[1] * e[2];
  return (float)count * area;
}
struct Bin {  // bvh.rs:112-151
  float mn[3] = {INFINITY, INFINITY, INFINITY};
  float mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  uint32_t count = 0;
  void include(const Prim& p) {
    for (int k = 0; k < 3; ++k) { mn[k] = wmin(mn[k], p.mn[k]); mx[k] = wmax(mx[k], p.mx[k]); }
    count += 1;
  }
  void include_bin(const Bin& o) {
    for (int k = 0; k < 3; ++k) { mn[k] = wmin(mn[k], o.mn[k]); mx[k] = wmax(mx[k], o.mx[k]); }
    count += o.count;
  }
  float cost() const { return sah_area_cost(mn, mx, count); }
};
static inline float node_cost(const Node& n) { return sah_area_cost(n.mn, n.mx, n.end - n.start); }
static Node new_leaf(const Prim* p, uint32_t s, uint32_t e) {  // bvh.rs:27-39
  Node n;
  for (int k = 0; k < 3; ++k) { n.mn[k] = p[s].mn[k]; n.mx[k] = p[s].mx[k]; }
  for (uint32_t i = s + 1; i < e; ++i)
    for (int k = 0; k < 3; ++k) { n.mn[k] = wmin(n.mn[k], p[i].mn[k]); n.mx[k] = wmax(n.mx[k], p[i].mx[k]); }
  n.start = s; n.end = e;
  return n;
}
static Node from_bin(const Bin& b, uint32_t start) {
  Node n;
  for (int k = 0; k < 3; ++k) { n.mn[k] = b.mn[k]; n.mx[k] = b.mx[k]; }
  n.start = start; n.end = start + b.count;
  return n;
}
struct Split { int axis; float mid; };

static bool find_best_split(const Prim* p, const Node& parent, Split* out) {  // bvh.rs:232-258
  float best = node_cost(parent);
  bool found = false;
  for (int axis = 0; axis < 3; ++axis) {
    for (uint32_t i = parent.start; i < parent.end; ++i) {
      float mid = p[i].c[axis];
      Bin l, r;
      for (uint32_t j = parent.start; j < parent.end; ++j) {
        if (p[j].c[axis] < mid) l.include(p[j]); else r.include(p[j]);
      }
      float cost = l.cost() + r.cost();
      if (cost < best) { best = cost; *out = {axis, mid}; found = true; }
    }
  }
  return found;
}
static bool approximate_best_split(const Prim* p, const Node& parent, Split* out) {  // bvh.rs:260-296
  const int NB = 16;
  Bin bins[NB * 3];
  float step[3];
  for (int k = 0; k < 3; ++k) step[k] = (parent.mx[k] - parent.mn[k]) / (float)NB;
  for (uint32_t i = parent.start; i < parent.end; ++i) {
    uint32_t b[3];
    for (int k = 0; k < 3; ++k) {
      b[k] = sat_u32(std::floor((p[i].c[k] - parent.mn[k]) / step[k]));
      if (b[k] > (uint32_t)(NB - 1)) b[k] = NB - 1;
    }
    bins[b[0]].include(p[i]);
    bins[NB + b[1]].include(p[i]);
    bins[NB * 2 + b[2]].include(p[i]);
  }
  float best = node_cost(parent);
  bool found = false;
  for (int axis = 0; axis < 3; ++axis) {
    Bin l;
    for (int i = 0; i < NB - 1; ++i) {
      l.include_bin(bins[axis * NB + i]);
      Bin r;
      for (int j = i + 1; j < NB; ++j) r.include_bin(bins[axis * NB + j]);
      float cost = l.cost() + r.cost();
      if (cost < best) {
        best = cost;
        *out = {axis, parent.mn[axis] + step[axis] * (float)(i + 1)};
        found = true;
      }
    }
  }
  return found;
}
static bool do_split(Prim* p, const Node& parent, Split s, Node* lo, Node* hi) {  // bvh.rs:307-330
  Bin l, r;
  for (uint32_t i = parent.start; i < parent.end; ++i) {
    float c = p[i].c[s.axis];
    if (c < s.mid) {
      l.include(p[i]);
      std::swap(p[i], p[parent.start + l.count - 1]);
    } else {
      r.include(p[i]);
    }
  }
  if (l.count == 0 || r.count == 0) return false;
  *lo = from_bin(l, parent.start);
  *hi = from_bin(r, parent.start + l.count);
  return true;
}
static bool split_node(Prim* p, const Node& parent, Node* lo, Node* hi) {  // bvh.rs:208-230
  uint32_t count = parent.end - parent.start;
  if (count <= 1) return false;
  if (count == 2) {
    Node l = new_leaf(p, parent.start, parent.start + 1);
    Node r = new_leaf(p, parent.start + 1, parent.start + 2);
    if (node_cost(l) + node_cost(r) < node_cost(parent)) { *lo = l; *hi = r; return true; }
    return false;
  }
  Split s;
  if (count <= 11) {
    if (!find_best_split(p, parent, &s)) return false;
  } else {
    if (!approximate_best_split(p, parent, &s)) return false;
  }
  return do_split(p, parent, s, lo, hi);
}
// BVHTree::append (bvh.rs:162-190); returns the index of the new root
static uint32_t bvh_append(std::vector<Node>& nodes, Prim* p, uint32_t s, uint32_t e) {
  const uint32_t kMaxDepth = 32;
  uint32_t parent = (uint32_t)nodes.size();
  nodes.push_back(new_leaf(p, s, e));
  std::vector<std::pair<uint32_t, uint32_t>> stack;
  stack.push_back({0u, parent});
  while (!stack.empty()) {
    auto [depth, idx] = stack.back();
    stack.pop_back();
    if (depth >= kMaxDepth) continue;
    Node node = nodes[idx];
    Node lo, hi;
    if (split_node(p, node, &lo, &hi)) {
      uint32_t li = (uint32_t)nodes.size();
      nodes[idx].end = 0;
      nodes[idx].start = li;
      nodes.push_back(lo);
      nodes.push_back(hi);
      stack.push_back({depth + 1, li});
      stack.push_back({depth + 1, li + 1});
    }
  }
  return parent;
}

// ---------------------------------------------------------------------------------------
// scene.rs:220-305
// ---------------------------------------------------------------------------------------
struct Instance {  // scene.rs:220-230, 160 bytes
  float w2l[16];
  float l2w[16];
  float color[4];
  float roughness, metallic, emissive;
  uint32_t node;
};
static_assert(sizeof(Instance) == 160, "instance layout");
struct Vertex { float pos[3]; float u; float nrm[3]; float v; float tan[4]; };
static_assert(sizeof(Vertex) == 48, "vertex layout");

}  // namespace

extern "C" {

// Primitive as produced by Scene::parse_gltf (scene.rs:59-67,199-206): a transform, a
// material and a range of the (rebased) index buffer.  w2l is the caller's inverse of l2w.
typedef struct or_primitive {
  float l2w[16];
  float w2l[16];
  float color[4];
  float roughness, metallic, emissive;
  uint32_t index_start, index_end;
} or_primitive;

typedef struct or_env {
  uint32_t kind;      // 0 = constant, 1 = equirect RGBA32F, 2 = cube RGBA32F (6 square faces
                      // +X, -X, +Y, -Y, +Z, -Z of height rows of width texels)
  float color[4];
  const float* texels;
  uint32_t width, height;
} or_env;

}  // extern "C"

namespace {

struct Scene {
  std::vector<Vertex> verts;
  std::vector<uint32_t> indices;  // permuted (flatten_triangle_list)
  std::vector<Node> blas, tlas;
  std::vector<Instance> inst;      // TLAS-permuted
};

// Mat4::transform_point3: ((x_axis*p.x + y_axis*p.y) + z_axis*p.z) + w_axis
static inline void transform_point3(const float* m, const float p[3], float out[3]) {
  for (int r = 0; r < 3; ++r) out[r] = m[r] * p[0] + m[4 + r] * p[1] + m[8 + r] * p[2] + m[12 + r];
}

// dedup != 0 builds one BLAS per distinct index range and reuses it for later primitives with
// the same range; dedup == 0 appends one BLAS per primitive exactly as scene.rs:285-299 does.
static Scene* build_scene(const float* vdata, uint32_t nv, const uint32_t* idx, uint32_t ni,
                          const or_primitive* prims, uint32_t np, int dedup) {
  Scene* sc = new Scene();
  sc->verts.resize(nv);
  std::memcpy(sc->verts.data(), vdata, (size_t)nv * sizeof(Vertex));
  // build_triangle_cache (bvh.rs:90-104)
  uint32_t nt = ni / 3;
  std::vector<Prim> tris(nt);
  for (uint32_t t = 0; t < nt; ++t) {
    const float* a = sc->verts[idx[3 * t]].pos;
    const float* b = sc->verts[idx[3 * t + 1]].pos;
    const float* c = sc->verts[idx[3 * t + 2]].pos;
    for (int k = 0; k < 3; ++k) {
      tris[t].c[k] = (a[k] + b[k] + c[k]) / 3.0f;
      tris[t].mn[k] = wmin(wmin(a[k], b[k]), c[k]);
      tris[t].mx[k] = wmax(wmax(a[k], b[k]), c[k]);
    }
    tris[t].payload = t;
  }
  std::vector<Prim> ib(np);
  std::vector<Instance> raw(np);
  std::map<std::pair<uint32_t, uint32_t>, uint32_t> built;
  for (uint32_t i = 0; i < np; ++i) {
    const or_primitive& pr = prims[i];
    std::pair<uint32_t, uint32_t> range{pr.index_start / 3, pr.index_end / 3};
    uint32_t root;
    auto it = dedup ? built.find(range) : built.end();
    if (it != built.end()) {
      root = it->second;
    } else {
      root = bvh_append(sc->blas, tris.data(), range.first, range.second);
      built[range] = root;
    }
    Instance& in = raw[i];
    std::memcpy(in.w2l, pr.w2l, 64);
    std::memcpy(in.l2w, pr.l2w, 64);
    std::memcpy(in.color, pr.color, 16);
    in.roughness = pr.roughness; in.metallic = pr.metallic; in.emissive = pr.emissive;
    in.node = root;
    const Node& r = sc->blas[root];
    // InstanceWithBounds::approximate_from_instance (scene.rs:239-259)
    float wmn[3] = {INFINITY, INFINITY, INFINITY}, wmx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
      float l[3] = {(c & 1) ? r.mx[0] : r.mn[0], (c & 2) ? r.mx[1] : r.mn[1], (c & 4) ? r.mx[2] : r.mn[2]};
      float w[3];
      transform_point3(in.l2w, l, w);
      for (int k = 0; k < 3; ++k) { wmn[k] = wmin(wmn[k], w[k]); wmx[k] = wmax(wmx[k], w[k]); }
    }
    for (int k = 0; k < 3; ++k) {
      ib[i].mn[k] = wmn[k];
      ib[i].mx[k] = wmx[k];
      ib[i].c[k] = (wmn[k] + wmx[k]) * 0.5f;  // BVHPrimitive::center default (bvh.rs:10-12)
    }
    ib[i].payload = i;
  }
  if (np) bvh_append(sc->tlas, ib.data(), 0, np);
  sc->inst.resize(np);
  for (uint32_t i = 0; i < np; ++i) sc->inst[i] = raw[ib[i].payload];
  sc->indices.resize(ni);
  for (uint32_t t = 0; t < nt; ++t)
    for (int k = 0; k < 3; ++k) sc->indices[3 * t + k] = idx[3 * tris[t].payload + k];
  for (uint32_t i = 3 * nt; i < ni; ++i) sc->indices[i] = idx[i];
  return sc;
}

// ---------------------------------------------------------------------------------------
// raytracing_sw.wgsl
// ---------------------------------------------------------------------------------------
template <class R> struct Ray { V3<R> o, d, inv; };

template <class R> struct HitT {
  uint32_t instance = 0, i0 = 0, i1 = 0, i2 = 0;
  R b0 = 0, b1 = 0, b2 = 0;
  R dist;
  uint32_t n_aabb = 0, n_tri = 0, n_inst = 0;
  bool overflow = false;
};

template <class R> static inline R no_hit() { return R(kNoHit); }

// Moller-Trumbore, backface culled (raytracing_sw.wgsl:51-78); returns false on a miss
template <class R>
static inline bool intersect_triangle(const Ray<R>& ray, V3<R> v0, V3<R> v1, V3<R> v2, R* t, R* u, R* v) {
  V3<R> e1 = v1 - v0;
  V3<R> e2 = v2 - v0;
  V3<R> h = cross(ray.d, e2);
  R det = dot(e1, h);
  if (det < R(kEps)) return false;
  R inv_det = R(1) / det;
  V3<R> s = ray.o - v0;
  R uu = inv_det * dot(s, h);
  if (uu < R(0) || uu > R(1)) return false;
  V3<R> q = cross(s, e1);
  R vv = inv_det * dot(ray.d, q);
  if (vv < R(0) || uu + vv > R(1)) return false;
  R tt = inv_det * dot(e2, q);
  if (tt < R(kBias)) return false;
  *t = tt; *u = uu; *v = vv;
  return true;
}

// slab test (raytracing_sw.wgsl:81-89)
template <class R> static inline R intersect_aabb(const Ray<R>& ray, const float mn[3], const float mx[3]) {
  V3<R> tmin = (cvt3<R>(mn) - ray.o) * ray.inv;
  V3<R> tmax = (cvt3<R>(mx) - ray.o) * ray.inv;
  V3<R> t1 = vmin(tmin, tmax);
  V3<R> t2 = vmax(tmin, tmax);
  R tn = wmax(t1.x, wmax(t1.y, t1.z));
  R tf = wmin(t2.x, wmin(t2.y, t2.z));
  return (tn <= tf && tf >= R(0)) ? tn : no_hit<R>();
}

// intersect_BLAS (raytracing_sw.wgsl:252-319); any_hit stops at the first accepted triangle
template <class R>
static HitT<R> intersect_blas(const Scene& sc, const Ray<R>& ray, uint32_t top, bool any_hit) {
  HitT<R> hit;
  hit.dist = no_hit<R>();
  R stack_d[kStackSize];
  uint32_t stack_i[kStackSize];
  int i = 0;
  const Node& tn = sc.blas[top];
  R d_top = intersect_aabb(ray, tn.mn, tn.mx);
  hit.n_aabb += 1;
  if (d_top < hit.dist) { stack_i[i] = top; stack_d[i] = d_top; ++i; }
  while (i > 0) {
    --i;
    if (stack_d[i] >= hit.dist) continue;
    const Node& node = sc.blas[stack_i[i]];
    if (node.end > 0u) {
      for (uint32_t j = node.start * 3u; j < node.end * 3u; j += 3u) {
        uint32_t i0 = sc.indices[j], i1 = sc.indices[j + 1], i2 = sc.indices[j + 2];
        R t, u, v;
        bool ok = intersect_triangle(ray, cvt3<R>(sc.verts[i0].pos), cvt3<R>(sc.verts[i1].pos),
                                     cvt3<R>(sc.verts[i2].pos), &t, &u, &v);
        hit.n_tri += 1;
        if (ok && t < hit.dist) {
          hit.dist = t;
          hit.b0 = R(1) - u - v; hit.b1 = u; hit.b2 = v;
          hit.i0 = i0; hit.i1 = i1; hit.i2 = i2;
          if (any_hit) return hit;
        }
      }
    } else {
      uint32_t il = node.start, ir = il + 1;
      const Node& ln = sc.blas[il];
      const Node& rn = sc.blas[ir];
      R dl = intersect_aabb(ray, ln.mn, ln.mx);
      R dr = intersect_aabb(ray, rn.mn, rn.mx);
      hit.n_aabb += 2;
      uint32_t fi = il, ni = ir; R fd = dl, nd = dr;
      if (dl < dr) { fi = ir; fd = dr; ni = il; nd = dl; }
      if (fd < hit.dist) {
        if (i >= kStackSize) { hit.overflow = true; return hit; }
        stack_i[i] = fi; stack_d[i] = fd; ++i;
      }
      if (nd < hit.dist) {
        if (i >= kStackSize) { hit.overflow = true; return hit; }
        stack_i[i] = ni; stack_d[i] = nd; ++i;
      }
    }
  }
  return hit;
}

// intersect_TLAS (raytracing_sw.wgsl:176-250)
template <class R> static HitT<R> intersect_tlas(const Scene& sc, const Ray<R>& ray, bool any_hit) {
  HitT<R> hit;
  hit.dist = no_hit<R>();
  if (sc.tlas.empty()) return hit;
  R stack_d[kStackSize];
  uint32_t stack_i[kStackSize];
  int i = 0;
  const Node& top = sc.tlas[0];
  R d_top = intersect_aabb(ray, top.mn, top.mx);
  hit.n_aabb += 1;
  if (d_top < hit.dist) { stack_i[i] = 0; stack_d[i] = d_top; ++i; }
  while (i > 0) {
    --i;
    if (stack_d[i] >= hit.dist) continue;
    const Node& node = sc.tlas[stack_i[i]];
    if (node.end > 0u) {
      for (uint32_t j = node.start; j < node.end; ++j) {
        const Instance& in = sc.inst[j];
        // local_origin = W2L * vec4(o, 1)
        V3<R> lo = col3<R>(in.w2l, 0) * ray.o.x + col3<R>(in.w2l, 1) * ray.o.y +
                   col3<R>(in.w2l, 2) * ray.o.z + col3<R>(in.w2l, 3) * R(1);
        V3<R> ld = mat3_mul<R>(in.w2l, ray.d);
        Ray<R> lr{lo, ld, V3<R>{R(1), R(1), R(1)} / ld};
        HitT<R> hl = intersect_blas(sc, lr, in.node, any_hit);
        hit.n_aabb += hl.n_aabb;
        hit.n_tri += hl.n_tri;
        hit.n_inst += 1;
        hit.overflow |= hl.overflow;
        if (hl.dist < hit.dist) {
          hit.dist = hl.dist;
          hit.instance = j;
          hit.i0 = hl.i0; hit.i1 = hl.i1; hit.i2 = hl.i2;
          hit.b0 = hl.b0; hit.b1 = hl.b1; hit.b2 = hl.b2;
          if (any_hit) return hit;
        }
      }
    } else {
      uint32_t il = node.start, ir = il + 1;
      R dl = intersect_aabb(ray, sc.tlas[il].mn, sc.tlas[il].mx);
      R dr = intersect_aabb(ray, sc.tlas[ir].mn, sc.tlas[ir].mx);
      hit.n_aabb += 2;
      uint32_t fi = il, ni = ir; R fd = dl, nd = dr;
      if (dl < dr) { fi = ir; fd = dr; ni = il; nd = dl; }
      if (fd < hit.dist) {
        if (i >= kStackSize) { hit.overflow = true; return hit; }
        stack_i[i] = fi; stack_d[i] = fd; ++i;
      }
      if (nd < hit.dist) {
        if (i >= kStackSize) { hit.overflow = true; return hit; }
        stack_i[i] = ni; stack_d[i] = nd; ++i;
      }
    }
  }
  return hit;
}

template <class R> struct HitInfo {
  V3<R> position, normal, tangent;
  R tangent_w;
  R dist;
  const Instance* inst;
  uint32_t n_aabb, n_tri, n_inst;
};

// per-render sums of the reference's per-ray work counters (raytracing_sw.wgsl:99-101,121-122)
struct WorkCounters {
  uint64_t rays = 0, n_aabb = 0, n_tri = 0, n_inst = 0;
};

// intersect_scene (raytracing_sw.wgsl:138-173); texcoords are not used by shading
template <class R> static HitInfo<R> intersect_scene(const Scene& sc, const Ray<R>& ray, bool* overflow) {
  HitT<R> h = intersect_tlas(sc, ray, false);
  HitInfo<R> info;
  info.dist = h.dist;
  info.n_aabb = h.n_aabb;
  info.n_tri = h.n_tri;
  info.n_inst = h.n_inst;
  info.inst = nullptr;
  if (h.overflow) *overflow = true;
  if (h.dist == no_hit<R>()) return info;
  const Instance& in = sc.inst[h.instance];
  info.inst = &in;
  info.position = ray.o + h.dist * ray.d;
  const Vertex& a = sc.verts[h.i0];
  const Vertex& b = sc.verts[h.i1];
  const Vertex& c = sc.verts[h.i2];
  V3<R> ln = cvt3<R>(a.nrm) * h.b0 + cvt3<R>(b.nrm) * h.b1 + cvt3<R>(c.nrm) * h.b2;
  V3<R> lt = cvt3<R>(a.tan) * h.b0 + cvt3<R>(b.tan) * h.b1 + cvt3<R>(c.tan) * h.b2;
  R ltw = R(a.tan[3]) * h.b0 + R(b.tan[3]) * h.b1 + R(c.tan[3]) * h.b2;
  info.normal = mat3t_mul<R>(in.w2l, ln);
  info.tangent = mat3_mul<R>(in.l2w, lt);
  info.tangent_w = ltw;
  return info;
}

// ---------------------------------------------------------------------------------------
// environment lookup (pathtracing.wgsl:168 samples a cube texture at mip 0 with a linear
// clamp-to-edge sampler, texture.rs:89-144).  The oracle defines a constant, an equirect
// RGBA32F map (bilinear, clamp in v and wrap in u) and a cube map of RGBA32F faces: face and
// (s, t) by the standard cube-map table (faces +X, -X, +Y, -Y, +Z, -Z; ties to X, then Y),
// texel coordinates ((s + 1) / 2) N - 1/2, bilinear with clamp at the face's edges.
// ---------------------------------------------------------------------------------------
template <class R> static V3<R> env_lookup(const or_env& env, V3<R> dir);

// ---------------------------------------------------------------------------------------
// pathtracing.wgsl
// ---------------------------------------------------------------------------------------
template <class R> static inline V3<R> fract3(V3<R> v) { return {v.x - std::floor(v.x), v.y - std::floor(v.y), v.z - std::floor(v.z)}; }

struct Vec4f { float x, y, z, w; };
static inline Vec4f sobol_read(const float* table, uint64_t n_vec4, uint64_t idx) {
  if (idx >= n_vec4) return {0, 0, 0, 0};
  return {table[4 * idx], table[4 * idx + 1], table[4 * idx + 2], table[4 * idx + 3]};
}
template <class R> struct Rand4 { R x, y, z, w; };
template <class R> static inline Rand4<R> cp_rotate(Vec4f s, const float shift[4]) {
  // fract(sample + shift), evaluated in binary32 like the reference for both modes
  float a = s.x + shift[0], b = s.y + shift[1], c = s.z + shift[2], d = s.w + shift[3];
  return {R(a - std::floor(a)), R(b - std::floor(b)), R(c - std::floor(c)), R(d - std::floor(d))};
}

// generate_ray (pathtracing.wgsl:27-41)
template <class R>
static Ray<R> generate_ray(uint32_t x, uint32_t y, uint32_t W, uint32_t H, R rx, R ry, const float* c2w) {
  R uvx = R(2) * (R(x) + rx) / R(W) - R(1);
  R uvy = R(2) * (R(y) + ry) / R(H) - R(1);
  R pw = R(c2w[15]);
  V3<R> pos = V3<R>{R(c2w[12]), R(c2w[13]), R(c2w[14])} / pw;
  // clip_to_world * vec4(-uv, -1, 1)
  R cx = -uvx, cy = -uvy, cz = R(-1), cw = R(1);
  R wd[4];
  for (int r = 0; r < 4; ++r)
    wd[r] = R(c2w[r]) * cx + R(c2w[4 + r]) * cy + R(c2w[8 + r]) * cz + R(c2w[12 + r]) * cw;
  V3<R> dir = pos - V3<R>{wd[0], wd[1], wd[2]} / wd[3];
  return {pos, dir, V3<R>{R(1), R(1), R(1)} / dir};
}

// sample_vndf_iso (pathtracing.wgsl:68-98)
template <class R> static V3<R> sample_vndf_iso(R r0, R r1, V3<R> wi, R alpha, V3<R> n) {
  if (alpha == R(0)) return n;
  V3<R> wi_z = n * dot(wi, n);
  V3<R> wi_xy = wi - wi_z;
  V3<R> wiStd = normalize(wi_z - alpha * wi_xy);
  R wiStd_z = dot(wiStd, n);
  R phi = (R(2) * r0 - R(1)) * R(kPi);
  R z = (R(1) - r1) * (R(1) + wiStd_z) - wiStd_z;
  R sinTheta = std::sqrt(wmin(wmax(R(1) - z * z, R(0)), R(1)));
  R sp, cp;
  sincos_r(phi, &sp, &cp);
  R x = sinTheta * cp;
  R y = sinTheta * sp;
  V3<R> cStd{x, y, z};
  V3<R> wr = n + V3<R>{R(0), R(0), R(1)};
  R safe_wrz = wmax(wr.z, R(1e-6f));
  V3<R> c = dot(wr, cStd) * wr / safe_wrz - cStd;
  V3<R> wmStd = c + wiStd;
  V3<R> wmStd_z = n * dot(n, wmStd);
  V3<R> wmStd_xy = wmStd_z - wmStd;
  return normalize(wmStd_z + alpha * wmStd_xy);
}

// sample_cosine_hemisphere (pathtracing.wgsl:100-105)
template <class R> static V3<R> sample_cosine_hemisphere(R r0, R r1) {
  R phi = R(kTwoPi) * r0;
  R sinT = std::sqrt(R(1) - r1);
  R cosT = std::sqrt(r1);
  R sp, cp;
  sincos_r(phi, &sp, &cp);
  return {cp * sinT, sp * sinT, cosT};
}
template <class R> static inline V3<R> F_schlick(R hdotv, V3<R> r0) {  // pathtracing.wgsl:113-115
  R p = pow5(R(1) - hdotv);
  return r0 + (V3<R>{R(1), R(1), R(1)} - r0) * p;
}
template <class R> static inline R lambda_tr(R ndotv, R alpha2) {  // pathtracing.wgsl:119-125
  R cos2 = ndotv * ndotv;
  R sin2 = R(1) - cos2;
  R tan2 = sin2 / cos2;
  return (R(-1) + std::sqrt(R(1) + alpha2 * tan2)) / R(2);
}

struct RenderArgs {
  const Scene* sc;
  const float* c2w;
  uint32_t W, H;
  const float* sobol;
  uint64_t sobol_n;  // number of vec4 entries
  uint32_t bounces;
  float cf;
  const or_env* env;
  uint32_t rr_start;  // Russian roulette from this bounce on (0: the reference schedule)
};

// sample_rendering_eq (pathtracing.wgsl:161-241); counts traversal queries into *rays
template <class R>
static V3<R> sample_rendering_eq(const RenderArgs& a, uint32_t sample, const float shift[4], Ray<R> ray,
                                 WorkCounters* wc, bool* overflow) {
  V3<R> T{R(1), R(1), R(1)};
  for (uint32_t bounce = 0; bounce <= a.bounces; ++bounce) {
    HitInfo<R> hit = intersect_scene(*a.sc, ray, overflow);
    wc->rays += 1;
    wc->n_aabb += hit.n_aabb;
    wc->n_tri += hit.n_tri;
    wc->n_inst += hit.n_inst;
    if (hit.dist == no_hit<R>()) return T * env_lookup<R>(*a.env, ray.d);
    const Instance& in = *hit.inst;
    V3<R> color{R(in.color[0]), R(in.color[1]), R(in.color[2])};
    if (in.emissive > 0.0f) return T * color;
    R alpha = R(in.roughness) * R(in.roughness);
    R alpha2 = alpha * alpha;
    V3<R> n = normalize(hit.normal);
    uint64_t base = (uint64_t)sample * kLdsStride + 1u + (uint64_t)bounce * kLdsPerBounce;
    Rand4<R> s0 = cp_rotate<R>(sobol_read(a.sobol, a.sobol_n, base + 0), shift);
    Rand4<R> s1 = cp_rotate<R>(sobol_read(a.sobol, a.sobol_n, base + 1), shift);
    V3<R> wo = normalize(-ray.d);
    R cosThetaO = dot(wo, n);
    V3<R> wi;
    R metallic = R(in.metallic);
    V3<R> albedo = color;
    V3<R> F0 = V3<R>{R(0.04f), R(0.04f), R(0.04f)} * (R(1) - metallic) + albedo * metallic;
    R specular_weight = luminance(F_schlick(dot(wo, n), F0));
    R diffuse_weight = (R(1) - metallic) * luminance(albedo);
    R p_specular = specular_weight / (specular_weight + diffuse_weight);
    R p_diffuse = R(1) - p_specular;
    if (s0.x < p_specular) {
      V3<R> wm = sample_vndf_iso(s0.y, s0.z, wo, alpha, n);
      wi = reflect(-wo, wm);
      R cosThetaD = dot(wo, wm);
      R cosThetaI = dot(wi, n);
      V3<R> F = F_schlick(cosThetaD, F0);
      R LambdaL = lambda_tr(cosThetaI, alpha2);
      R LambdaV = lambda_tr(cosThetaO, alpha2);
      V3<R> spec = F * (R(1) + LambdaV) / (R(1) + LambdaL + LambdaV);
      T = T * (spec / p_specular);
    } else {
      V3<R> nt = normalize(hit.tangent - dot(hit.tangent, n) * n);  // build_tbn (common.wgsl:55-59)
      V3<R> bt = cross(n, nt);
      V3<R> ls = sample_cosine_hemisphere(s1.y, s1.z);
      wi = nt * ls.x + bt * ls.y + n * ls.z;
      V3<R> wm = normalize(wi + wo);
      R cosThetaD = dot(wi, wm);
      R cosThetaI = dot(wi, n);
      R FD90 = R(0.5f) + R(2) * alpha * pow2(cosThetaD);
      R response = (R(1) + (FD90 - R(1)) * pow5(R(1) - cosThetaI)) * (R(1) + (FD90 - R(1)) * pow5(R(1) - cosThetaO));
      V3<R> diffuse = (R(1) - metallic) * albedo * response;
      T = T * (diffuse / p_diffuse);
    }
    R p_continue = wmin(R(1) - pow8(R(bounce) / R(a.bounces)), R(1));
    p_continue = p_continue * wmin(luminance(T) * R(a.cf), R(1));
    // start-bounce variant (BASELINE's "RR from bounce 3"): no roulette before rr_start
    if (bounce < a.rr_start) p_continue = R(1);
    if (s0.z < p_continue) {
      T = T / p_continue;
    } else {
      return {R(0), R(0), R(0)};
    }
    ray = Ray<R>{hit.position, wi, V3<R>{R(1), R(1), R(1)} / wi};
  }
  return {R(0), R(0), R(0)};
}

// Equirect lookup (the build's definition; the reference samples a cube map): on the
// normalised direction d, u = atan2(d.x, -d.z) / (2 pi) + 0.5 and v = acos(d.y) / pi; bilinear
// filtering with wrap in u and clamp in v, texel centres at (i + 0.5) / size; a NaN direction
// sees black.  binary32: atan on [0,1] is x * P(x^2) with a least-squares fitted degree-7 P
// (max error 1.7e-7), atan2/acos by octant reduction, Horner without fusion.  binary64 (truth
// mode): libm atan2/acos.
constexpr float kAtanP[8] = {0x1.fffffcp-1f, -0x1.5551dp-2f, 0x1.98faep-3f, -0x1.1f1e82p-3f,
                             0x1.96172p-4f,  -0x1.e75096p-5f, 0x1.8d5abp-6f, -0x1.3394dap-8f};
static inline float atan2_f32(float y, float x) {
  float ax = std::fabs(x), ay = std::fabs(y);
  float mx = ax > ay ? ax : ay, mn = ax > ay ? ay : ax;
  float a = mx > 0.0f ? mn / mx : 0.0f;
  float a2 = a * a;
  float p = kAtanP[7];
  for (int k = 6; k >= 0; --k) p = p * a2 + kAtanP[k];
  float r = a * p;
  if (ay > ax) r = 1.57079637f - r;
  if (x < 0.0f) r = 3.14159274f - r;
  if (y < 0.0f) r = -r;
  return r;
}
static inline float acos_f32(float y) { return atan2_f32(std::sqrt((1.0f - y) * (1.0f + y)), y); }

template <class R> static uint32_t cube_face(R x, R y, R z, R* s, R* t) {
  const R ax = std::fabs(x), ay = std::fabs(y), az = std::fabs(z);
  R sc, tc, ma;
  uint32_t f;
  if (ax >= ay && ax >= az) {
    f = x >= R(0) ? 0u : 1u;
    ma = ax;
    sc = x >= R(0) ? -z : z;
    tc = -y;
  } else if (ay >= az) {
    f = y >= R(0) ? 2u : 3u;
    ma = ay;
    sc = x;
    tc = y >= R(0) ? z : -z;
  } else {
    f = z >= R(0) ? 4u : 5u;
    ma = az;
    sc = z >= R(0) ? x : -x;
    tc = -y;
  }
  *s = sc / ma;
  *t = tc / ma;
  return f;
}

template <class R> static V3<R> env_lookup_cube(const or_env& env, V3<R> dir) {
  R s, t;
  const uint32_t f = cube_face<R>(dir.x, dir.y, dir.z, &s, &t);
  const int N = (int)env.width;
  const R fx = (s + R(1)) * R(0.5) * (R)N - R(0.5), fy = (t + R(1)) * R(0.5) * (R)N - R(0.5);
  if (fx != fx || fy != fy) return {R(0), R(0), R(0)};
  const R x0 = std::floor(fx), y0 = std::floor(fy);
  const R tx = fx - x0, ty = fy - y0;
  const int xi = (int)x0, yi = (int)y0;
  const int xa = std::min(std::max(xi, 0), N - 1), xb = std::min(std::max(xi + 1, 0), N - 1);
  const int ya = (int)f * N + std::min(std::max(yi, 0), N - 1), yb = (int)f * N + std::min(std::max(yi + 1, 0), N - 1);
  const float* t00 = env.texels + 4 * ((size_t)ya * N + xa);
  const float* t10 = env.texels + 4 * ((size_t)ya * N + xb);
  const float* t01 = env.texels + 4 * ((size_t)yb * N + xa);
  const float* t11 = env.texels + 4 * ((size_t)yb * N + xb);
  R c[3];
  for (int ch = 0; ch < 3; ++ch)
    c[ch] = (R(t00[ch]) * (R(1) - tx) + R(t10[ch]) * tx) * (R(1) - ty) + (R(t01[ch]) * (R(1) - tx) + R(t11[ch]) * tx) * ty;
  return {c[0], c[1], c[2]};
}

static V3<float> env_lookup_f32(const or_env& env, V3<float> dir) {
  V3<float> d = normalize(dir);
  float u = atan2_f32(d.x, -d.z) * 0.159154943f + 0.5f;
  float v = acos_f32(wmin(wmax(d.y, -1.0f), 1.0f)) * 0.318309886f;
  float fx = u * (float)env.width - 0.5f, fy = v * (float)env.height - 0.5f;
  if (fx != fx || fy != fy) return {0.0f, 0.0f, 0.0f};
  float x0 = std::floor(fx), y0 = std::floor(fy);
  float tx = fx - x0, ty = fy - y0;
  int W = (int)env.width, H = (int)env.height;
  int xi = (int)x0, yi = (int)y0;
  int xa = ((xi % W) + W) % W, xb = (((xi + 1) % W) + W) % W;
  int ya = yi < 0 ? 0 : (yi > H - 1 ? H - 1 : yi), yb = yi + 1 < 0 ? 0 : (yi + 1 > H - 1 ? H - 1 : yi + 1);
  const float* t00 = env.texels + 4 * ((size_t)ya * W + xa);
  const float* t10 = env.texels + 4 * ((size_t)ya * W + xb);
  const float* t01 = env.texels + 4 * ((size_t)yb * W + xa);
  const float* t11 = env.texels + 4 * ((size_t)yb * W + xb);
  float c[3];
  for (int ch = 0; ch < 3; ++ch)
    c[ch] = (t00[ch] * (1.0f - tx) + t10[ch] * tx) * (1.0f - ty) + (t01[ch] * (1.0f - tx) + t11[ch] * tx) * ty;
  return {c[0], c[1], c[2]};
}

template <class R> static V3<R> env_lookup(const or_env& env, V3<R> dir) {
  if (env.kind == 0) return {R(env.color[0]), R(env.color[1]), R(env.color[2])};
  if (env.kind == 2) return env_lookup_cube<R>(env, dir);
  if constexpr (std::is_same<R, float>::value) return env_lookup_f32(env, dir);
  double dx = dir.x, dy = dir.y, dz = dir.z;
  double l = std::sqrt(dx * dx + dy * dy + dz * dz);
  dx /= l; dy /= l; dz /= l;
  double u = std::atan2(dx, -dz) / (2.0 * M_PI) + 0.5;
  double v = std::acos(std::max(-1.0, std::min(1.0, dy))) / M_PI;
  double fx = u * env.width - 0.5, fy = v * env.height - 0.5;
  double x0 = std::floor(fx), y0 = std::floor(fy);
  double tx = fx - x0, ty = fy - y0;
  auto tex = [&](long xi, long yi, int ch) {
    long W = env.width, H = env.height;
    xi = ((xi % W) + W) % W;
    yi = std::max(0L, std::min(H - 1, yi));
    return (double)env.texels[4 * ((size_t)yi * W + xi) + ch];
  };
  double c[3];
  for (int ch = 0; ch < 3; ++ch) {
    double a = tex((long)x0, (long)y0, ch) * (1 - tx) + tex((long)x0 + 1, (long)y0, ch) * tx;
    double b = tex((long)x0, (long)y0 + 1, ch) * (1 - tx) + tex((long)x0 + 1, (long)y0 + 1, ch) * tx;
    c[ch] = a * (1 - ty) + b * ty;
  }
  return {R(c[0]), R(c[1]), R(c[2])};
}

template <class F> static void parallel_for(uint32_t n, int threads, F&& fn) {
  if (threads <= 1 || n <= 1) { for (uint32_t i = 0; i < n; ++i) fn(i); return; }
  std::atomic<uint32_t> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&] { for (uint32_t i; (i = next.fetch_add(1)) < n;) fn(i); });
  for (auto& th : pool) th.join();
}

template <class R>
static uint64_t render_region(const RenderArgs& a, uint32_t first_sample, uint32_t spp, uint32_t x0, uint32_t y0,
                              uint32_t w, uint32_t h, float* out_rgba, float* per_sample, int threads,
                              uint32_t* overflow_flag, uint64_t* counters) {
  std::atomic<uint64_t> total_rays{0}, total_aabb{0}, total_tri{0}, total_inst{0};
  std::atomic<uint32_t> ovf{0};
  // one work item per pixel (regions can be a few pixels wide; samples stay in order per pixel)
  parallel_for(w * h, threads, [&](uint32_t item) {
    WorkCounters wc;
    bool overflow = false;
    const uint32_t xx = item % w, yy = item / w;
    const uint32_t px = x0 + xx, py = y0 + yy;
    const size_t o = (size_t)yy * w + xx;
    uint32_t hin[4] = {px, py, px, py};
    float shift[4];
    hash4f(hin, shift);
    // the running mean is kept in R: binary32 is the reference's own mix (pathtracing.wgsl:258);
    // the binary64 truth mode averages its binary64 samples in binary64
    R cr = out_rgba[4 * o], cg = out_rgba[4 * o + 1], cb = out_rgba[4 * o + 2];
    for (uint32_t k = 0; k < spp; ++k) {
      uint32_t sample = first_sample + k;
      R weight = R(1) / (R)sample;  // pathtracer.rs:235
      Rand4<R> j = cp_rotate<R>(sobol_read(a.sobol, a.sobol_n, (uint64_t)sample * kLdsStride), shift);
      Ray<R> ray = generate_ray<R>(px, py, a.W, a.H, j.x, j.y, a.c2w);
      V3<R> L = sample_rendering_eq<R>(a, sample, shift, ray, &wc, &overflow);
      if (per_sample) {
        float* q = per_sample + 4 * (o * spp + k);
        q[0] = (float)L.x; q[1] = (float)L.y; q[2] = (float)L.z; q[3] = 1.0f;
      }
      // mix(color, L, weight) (pathtracing.wgsl:258)
      cr = cr * (R(1) - weight) + L.x * weight;
      cg = cg * (R(1) - weight) + L.y * weight;
      cb = cb * (R(1) - weight) + L.z * weight;
    }
    out_rgba[4 * o] = (float)cr; out_rgba[4 * o + 1] = (float)cg; out_rgba[4 * o + 2] = (float)cb;
    out_rgba[4 * o + 3] = 1.0f;
    total_rays += wc.rays;
    total_aabb += wc.n_aabb;
    total_tri += wc.n_tri;
    total_inst += wc.n_inst;
    if (overflow) ovf = 1;
  });
  if (overflow_flag) *overflow_flag = ovf.load();
  if (counters) {
    counters[0] = total_rays.load();
    counters[1] = total_aabb.load();
    counters[2] = total_tri.load();
    counters[3] = total_inst.load();
  }
  return total_rays.load();
}

}  // namespace

extern "C" {

// ---- common.wgsl ----
void or_hash4u(const uint32_t* in4, uint32_t* out4) { hash4u(in4, out4); }
void or_hash4f(const uint32_t* in4, float* out4) { hash4f(in4, out4); }
void or_sincos(const float* x, uint64_t n, float* s, float* c) {
  for (uint64_t i = 0; i < n; ++i) sincos_f32(x[i], &s[i], &c[i]);
}

// ---- environment lookup (pathtracing.wgsl:168) on caller directions: n x 3 floats in,
// n x 3 out; precision 32 (binary32, the kernels' contract) or 64 ----
void or_env_lookup(const or_env* env, const float* dirs, uint64_t n, int precision, float* out) {
  for (uint64_t i = 0; i < n; ++i) {
    const float* d = dirs + 3 * i;
    if (precision == 64) {
      const V3<double> c = env_lookup<double>(*env, V3<double>{d[0], d[1], d[2]});
      out[3 * i] = (float)c.x; out[3 * i + 1] = (float)c.y; out[3 * i + 2] = (float)c.z;
    } else {
      const V3<float> c = env_lookup<float>(*env, V3<float>{d[0], d[1], d[2]});
      out[3 * i] = c.x; out[3 * i + 1] = c.y; out[3 * i + 2] = c.z;
    }
  }
}

// ---- Sobol ----
uint32_t or_sobol_u32(uint32_t index, uint32_t dim) { return dim < 68 ? sobol_u32(index, (int)dim) : 0u; }
// Table in the reference's layout: row-major [sample][dimension set] of vec4 (pathtracer.rs:62-64)
void or_sobol_table(uint32_t n_samples, uint32_t n_dimsets, uint32_t seed, float* out) {
  for (uint32_t i = 0; i < n_samples; ++i)
    for (uint32_t d = 0; d < n_dimsets; ++d) sobol_burley_4d(i, d, seed, out + 4 * ((size_t)i * n_dimsets + d));
}

// ---- bvh.rs over a bare triangle list (one BLAS): nodes (8 words each) + permuted indices ----
uint32_t or_bvh_build_triangles(const float* positions /* nv*3 */, const uint32_t* idx, uint32_t ni,
                                float* nodes_out /* capacity 2*nt words*8 */, uint32_t* idx_out) {
  uint32_t nt = ni / 3;
  std::vector<Prim> tris(nt);
  for (uint32_t t = 0; t < nt; ++t) {
    const float* a = positions + 3 * (size_t)idx[3 * t];
    const float* b = positions + 3 * (size_t)idx[3 * t + 1];
    const float* c = positions + 3 * (size_t)idx[3 * t + 2];
    for (int k = 0; k < 3; ++k) {
      tris[t].c[k] = (a[k] + b[k] + c[k]) / 3.0f;
      tris[t].mn[k] = wmin(wmin(a[k], b[k]), c[k]);
      tris[t].mx[k] = wmax(wmax(a[k], b[k]), c[k]);
    }
    tris[t].payload = t;
  }
  std::vector<Node> nodes;
  if (nt) bvh_append(nodes, tris.data(), 0, nt);
  std::memcpy(nodes_out, nodes.data(), nodes.size() * sizeof(Node));
  for (uint32_t t = 0; t < nt; ++t)
    for (int k = 0; k < 3; ++k) idx_out[3 * t + k] = idx[3 * tris[t].payload + k];
  return (uint32_t)nodes.size();
}

// ---- scene.rs:280-305 ----
void* or_scene_build(const float* vertices, uint32_t nv, const uint32_t* indices, uint32_t ni,
                     const or_primitive* prims, uint32_t np, int dedup) {
  return build_scene(vertices, nv, indices, ni, prims, np, dedup);
}
void or_scene_sizes(void* h, uint32_t* n_blas, uint32_t* n_tlas, uint32_t* n_inst, uint32_t* n_idx) {
  Scene* s = (Scene*)h;
  *n_blas = (uint32_t)s->blas.size(); *n_tlas = (uint32_t)s->tlas.size();
  *n_inst = (uint32_t)s->inst.size(); *n_idx = (uint32_t)s->indices.size();
}
void or_scene_export(void* h, void* blas, void* tlas, void* inst, uint32_t* indices) {
  Scene* s = (Scene*)h;
  if (blas) std::memcpy(blas, s->blas.data(), s->blas.size() * sizeof(Node));
  if (tlas) std::memcpy(tlas, s->tlas.data(), s->tlas.size() * sizeof(Node));
  if (inst) std::memcpy(inst, s->inst.data(), s->inst.size() * sizeof(Instance));
  if (indices) std::memcpy(indices, s->indices.data(), s->indices.size() * 4);
}
void or_scene_free(void* h) { delete (Scene*)h; }

// ---- traversal of ray batches: rays are 8 floats (o.xyz, tmin(unused), d.xyz, pad) ----
// hit_f: t, u, v, 0 (t = FLT_MAX on a miss); hit_u: instance, i0, i1, i2; counters: n_aabb, n_tri, n_inst, overflow
void or_trace(void* h, const float* rays, uint64_t n, int any_hit, float* hit_f, uint32_t* hit_u,
              uint32_t* counters, int threads) {
  const Scene& sc = *(Scene*)h;
  uint32_t chunks = (uint32_t)((n + 1023) / 1024);
  parallel_for(chunks, threads, [&](uint32_t c) {
    for (uint64_t r = (uint64_t)c * 1024; r < std::min<uint64_t>(n, (uint64_t)c * 1024 + 1024); ++r) {
      const float* q = rays + 8 * r;
      Ray<float> ray;
      ray.o = {q[0], q[1], q[2]};
      ray.d = {q[4], q[5], q[6]};
      ray.inv = V3<float>{1.0f, 1.0f, 1.0f} / ray.d;
      HitT<float> hit = intersect_tlas(sc, ray, any_hit != 0);
      hit_f[4 * r] = hit.dist; hit_f[4 * r + 1] = hit.b1; hit_f[4 * r + 2] = hit.b2; hit_f[4 * r + 3] = 0.0f;
      if (hit_u) {
        hit_u[4 * r] = hit.instance; hit_u[4 * r + 1] = hit.i0; hit_u[4 * r + 2] = hit.i1; hit_u[4 * r + 3] = hit.i2;
      }
      if (counters) {
        counters[4 * r] = hit.n_aabb; counters[4 * r + 1] = hit.n_tri;
        counters[4 * r + 2] = hit.n_inst; counters[4 * r + 3] = hit.overflow ? 1u : 0u;
      }
    }
  });
}

// ---- primary rays exactly as generate_ray builds them (pathtracing.wgsl:245-255) ----
void or_primary_rays(const float* c2w, uint32_t W, uint32_t H, const float* sobol, uint64_t sobol_n,
                     uint32_t sample, float* rays_out /* W*H*8 */) {
  for (uint32_t y = 0; y < H; ++y)
    for (uint32_t x = 0; x < W; ++x) {
      uint32_t hin[4] = {x, y, x, y};
      float shift[4];
      hash4f(hin, shift);
      Rand4<float> j = cp_rotate<float>(sobol_read(sobol, sobol_n, (uint64_t)sample * kLdsStride), shift);
      Ray<float> r = generate_ray<float>(x, y, W, H, j.x, j.y, c2w);
      float* q = rays_out + 8 * ((size_t)y * W + x);
      q[0] = r.o.x; q[1] = r.o.y; q[2] = r.o.z; q[3] = 0.0f;
      q[4] = r.d.x; q[5] = r.d.y; q[6] = r.d.z; q[7] = 0.0f;
    }
}

// ---- the pass: spp dispatches (samples first_sample .. first_sample+spp-1, 1-based) over a
// pixel region, accumulated as the running mean in out_rgba (w*h RGBA32F, in/out).
// precision 32 = faithful binary32, 64 = binary64 truth.  Returns traversal queries issued.
uint64_t or_render(void* h, const float* c2w, uint32_t W, uint32_t H, const float* sobol, uint64_t sobol_n,
                   uint32_t first_sample, uint32_t spp, uint32_t bounces, float cf, const or_env* env,
                   uint32_t x0, uint32_t y0, uint32_t w, uint32_t hh, float* out_rgba, float* per_sample,
                   int precision, int threads, uint32_t* overflow, uint64_t* counters, uint32_t rr_start) {
  RenderArgs a{(const Scene*)h, c2w, W, H, sobol, sobol_n, bounces, cf, env, rr_start};
  if (precision == 64)
    return render_region<double>(a, first_sample, spp, x0, y0, w, hh, out_rgba, per_sample, threads, overflow,
                                 counters);
  return render_region<float>(a, first_sample, spp, x0, y0, w, hh, out_rgba, per_sample, threads, overflow,
                              counters);
}

}  // extern "C"

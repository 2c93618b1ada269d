// Host side of the scene: the reference's SAH BVH builder (src/pathtracing/bvh.rs), the
// BLAS/TLAS assembly of SceneBuffers::from_scene (src/pathtracing/scene.rs:280-305), and the
// translation of those reference-layout trees into the device layout (nb_internal.h).
//
// The builder reproduces bvh.rs node for node: 16-bin binned SAH above 11 primitives,
// brute-force SAH for 3..11, the manual split for 2, cost = count * (xy + xz + yz) with no
// traversal constant, MAX_DEPTH 32, explicit DFS stack (children appended at len, len+1;
// right child processed first) and the unstable in-place swap partition.  Rust evaluates
// f32 arithmetic without contraction; this file is compiled with -ffp-contract=off to match.
// The one deliberate difference from the reference is parallelism: distinct BLASes (disjoint
// triangle ranges) are built on worker threads into private node lists that are then
// concatenated in primitive order with their indices offset, which yields the same array
// as the sequential appends.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <utility>

#include "nb_internal.h"

namespace nb {
namespace {

// glam Vec3::min/max with IEEE minimumNumber/maximumNumber semantics (NaN ignored, -0 < +0)
inline float min_num(float a, float b) {
  if (a != a) return b;
  if (b != b) return a;
  if (a < b) return a;
  if (b < a) return b;
  return std::signbit(a) ? a : b;
}
inline float max_num(float a, float b) {
  if (a != a) return b;
  if (b != b) return a;
  if (a > b) return a;
  if (b > a) return b;
  return std::signbit(a) ? b : a;
}
// Rust `f32 as u32` (saturating; NaN -> 0)
inline uint32_t as_u32(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
}

struct Prim {
  float c[3];
  float mn[3];
  float mx[3];
  uint32_t payload;
};

inline float area_cost(const float mn[3], const float mx[3], uint32_t count) {
  float ex = mx[0] - mn[0], ey = mx[1] - mn[1], ez = mx[2] - mn[2];
  if (!(std::isfinite(ex) && std::isfinite(ey) && std::isfinite(ez))) return INFINITY;
  float area = ex * ey + ex * ez + ey * ez;
  return (float)count * area;
}

struct Box {
  float mn[3] = {INFINITY, INFINITY, INFINITY};
  float mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  uint32_t count = 0;
  void add(const Prim& p) {
    mn[0] = min_num(mn[0], p.mn[0]); mn[1] = min_num(mn[1], p.mn[1]); mn[2] = min_num(mn[2], p.mn[2]);
    mx[0] = max_num(mx[0], p.mx[0]); mx[1] = max_num(mx[1], p.mx[1]); mx[2] = max_num(mx[2], p.mx[2]);
    count += 1;
  }
  void merge(const Box& o) {
    for (int k = 0; k < 3; ++k) { mn[k] = min_num(mn[k], o.mn[k]); mx[k] = max_num(mx[k], o.mx[k]); }
    count += o.count;
  }
  float cost() const { return area_cost(mn, mx, count); }
};

inline float node_cost(const nb_bvh_node& n) { return area_cost(n.min, n.max, n.end - n.start); }

nb_bvh_node leaf_over(const Prim* p, uint32_t s, uint32_t e) {
  nb_bvh_node n;
  for (int k = 0; k < 3; ++k) { n.min[k] = p[s].mn[k]; n.max[k] = p[s].mx[k]; }
  for (uint32_t i = s + 1; i < e; ++i)
    for (int k = 0; k < 3; ++k) { n.min[k] = min_num(n.min[k], p[i].mn[k]); n.max[k] = max_num(n.max[k], p[i].mx[k]); }
  n.start = s;
  n.end = e;
  return n;
}

nb_bvh_node node_of(const Box& b, uint32_t start) {
  nb_bvh_node n;
  for (int k = 0; k < 3; ++k) { n.min[k] = b.mn[k]; n.max[k] = b.mx[k]; }
  n.start = start;
  n.end = start + b.count;
  return n;
}

// bvh.rs:232-258 (3..11 primitives)
bool brute_force_split(const Prim* p, const nb_bvh_node& parent, int* axis_out, float* mid_out) {
  float best = node_cost(parent);
  bool found = false;
  for (int axis = 0; axis < 3; ++axis) {
    for (uint32_t i = parent.start; i < parent.end; ++i) {
      float mid = p[i].c[axis];
      Box l, r;
      for (uint32_t j = parent.start; j < parent.end; ++j) (p[j].c[axis] < mid ? l : r).add(p[j]);
      float cost = l.cost() + r.cost();
      if (cost < best) { best = cost; *axis_out = axis; *mid_out = mid; found = true; }
    }
  }
  return found;
}

// bvh.rs:260-296 (12+ primitives, 16 bins per axis)
bool binned_split(const Prim* p, const nb_bvh_node& parent, int* axis_out, float* mid_out) {
  constexpr int kBins = 16;
  Box bins[3][kBins];
  float step[3];
  for (int k = 0; k < 3; ++k) step[k] = (parent.max[k] - parent.min[k]) / (float)kBins;
  for (uint32_t i = parent.start; i < parent.end; ++i) {
    const Prim& q = p[i];
    for (int k = 0; k < 3; ++k) {
      uint32_t b = as_u32(std::floor((q.c[k] - parent.min[k]) / step[k]));
      bins[k][b < (uint32_t)(kBins - 1) ? b : (uint32_t)(kBins - 1)].add(q);
    }
  }
  float best = node_cost(parent);
  bool found = false;
  for (int axis = 0; axis < 3; ++axis) {
    // suffix unions: min/max/count merges are associative and commutative, so right[i + 1]
    // equals the right-hand bin the reference accumulates from bins i+1..15
    Box right[kBins + 1];
    for (int j = kBins - 1; j >= 1; --j) {
      right[j] = right[j + 1];
      right[j].merge(bins[axis][j]);
    }
    Box left;
    for (int i = 0; i < kBins - 1; ++i) {
      left.merge(bins[axis][i]);
      float cost = left.cost() + right[i + 1].cost();
      if (cost < best) {
        best = cost;
        *axis_out = axis;
        *mid_out = parent.min[axis] + step[axis] * (float)(i + 1);
        found = true;
      }
    }
  }
  return found;
}

// bvh.rs:307-330
bool partition(Prim* p, const nb_bvh_node& parent, int axis, float mid, nb_bvh_node* lo, nb_bvh_node* hi) {
  Box l, r;
  for (uint32_t i = parent.start; i < parent.end; ++i) {
    if (p[i].c[axis] < mid) {
      l.add(p[i]);
      std::swap(p[i], p[parent.start + l.count - 1]);
    } else {
      r.add(p[i]);
    }
  }
  if (l.count == 0 || r.count == 0) return false;
  *lo = node_of(l, parent.start);
  *hi = node_of(r, parent.start + l.count);
  return true;
}

// bvh.rs:208-230
bool split_node(Prim* p, const nb_bvh_node& parent, nb_bvh_node* lo, nb_bvh_node* hi) {
  uint32_t count = parent.end - parent.start;
  if (count <= 1) return false;
  if (count == 2) {
    nb_bvh_node l = leaf_over(p, parent.start, parent.start + 1);
    nb_bvh_node r = leaf_over(p, parent.start + 1, parent.start + 2);
    if (node_cost(l) + node_cost(r) < node_cost(parent)) { *lo = l; *hi = r; return true; }
    return false;
  }
  int axis = 0;
  float mid = 0.0f;
  bool ok = count <= 11 ? brute_force_split(p, parent, &axis, &mid) : binned_split(p, parent, &axis, &mid);
  return ok && partition(p, parent, axis, mid, lo, hi);
}

// BVHTree::append (bvh.rs:162-190) into `nodes`; returns the root index
uint32_t append_tree(std::vector<nb_bvh_node>& nodes, Prim* p, uint32_t s, uint32_t e) {
  constexpr uint32_t kMaxDepth = 32;
  uint32_t root = (uint32_t)nodes.size();
  nodes.push_back(leaf_over(p, s, e));
  std::vector<std::pair<uint32_t, uint32_t>> stack;
  stack.emplace_back(0u, root);
  while (!stack.empty()) {
    auto [depth, idx] = stack.back();
    stack.pop_back();
    if (depth >= kMaxDepth) continue;
    nb_bvh_node node = nodes[idx];
    nb_bvh_node lo, hi;
    if (split_node(p, node, &lo, &hi)) {
      uint32_t li = (uint32_t)nodes.size();
      nodes[idx].end = 0;
      nodes[idx].start = li;
      nodes.push_back(lo);
      nodes.push_back(hi);
      stack.emplace_back(depth + 1, li);
      stack.emplace_back(depth + 1, li + 1);
    }
  }
  return root;
}

void triangle_cache(const float* pos, size_t pos_stride, const uint32_t* idx, size_t nt, Prim* out) {
  for (size_t t = 0; t < nt; ++t) {
    const float* a = pos + pos_stride * idx[3 * t];
    const float* b = pos + pos_stride * idx[3 * t + 1];
    const float* c = pos + pos_stride * idx[3 * t + 2];
    Prim& q = out[t];
    for (int k = 0; k < 3; ++k) {
      q.c[k] = (a[k] + b[k] + c[k]) / 3.0f;  // bvh.rs:97
      q.mn[k] = min_num(min_num(a[k], b[k]), c[k]);
      q.mx[k] = max_num(max_num(a[k], b[k]), c[k]);
    }
    q.payload = (uint32_t)t;
  }
}

template <class F> void run_parallel(size_t n, F&& fn) {
  unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  size_t workers = std::min<size_t>(hw, n);
  if (workers <= 1) { for (size_t i = 0; i < n; ++i) fn(i); return; }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (size_t w = 0; w < workers; ++w)
    pool.emplace_back([&] { for (size_t i; (i = next.fetch_add(1)) < n;) fn(i); });
  for (auto& t : pool) t.join();
}

bool invert4(const float* m, float* out) {  // column-major, double precision, rounded
  double a[4][8];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) { a[r][c] = m[4 * c + r]; a[r][4 + c] = (r == c) ? 1.0 : 0.0; }
  for (int c = 0; c < 4; ++c) {
    int piv = c;
    for (int r = c + 1; r < 4; ++r) if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
    if (a[piv][c] == 0.0) return false;
    if (piv != c) for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
    double inv = 1.0 / a[c][c];
    for (int k = 0; k < 8; ++k) a[c][k] *= inv;
    for (int r = 0; r < 4; ++r) {
      if (r == c) continue;
      double f = a[r][c];
      for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[4 * c + r] = (float)a[r][4 + c];
  return true;
}

// Mat4::transform_point3: ((x_axis*p.x + y_axis*p.y) + z_axis*p.z) + w_axis
inline void transform_point3(const float* m, const float p[3], float out[3]) {
  for (int r = 0; r < 3; ++r) out[r] = m[r] * p[0] + m[4 + r] * p[1] + m[8 + r] * p[2] + m[12 + r];
}

}  // namespace

int build_bvh_triangles(const float* positions, size_t n_vertices, const uint32_t* indices, size_t n_indices,
                        std::vector<nb_bvh_node>* nodes, std::vector<uint32_t>* permuted) {
  size_t nt = n_indices / 3;
  for (size_t i = 0; i < 3 * nt; ++i)
    if (indices[i] >= n_vertices) return fail(NB_ERR_INVALID_ARG, "index %zu out of range (%u >= %zu)", i, indices[i], n_vertices);
  std::vector<Prim> tris(nt);
  triangle_cache(positions, 3, indices, nt, tris.data());
  nodes->clear();
  if (nt) append_tree(*nodes, tris.data(), 0, (uint32_t)nt);
  permuted->assign(indices, indices + n_indices);
  for (size_t t = 0; t < nt; ++t)
    for (int k = 0; k < 3; ++k) (*permuted)[3 * t + k] = indices[3 * tris[t].payload + k];
  return NB_OK;
}

int build_scene_reference(const nb_vertex* vertices, size_t nv, const uint32_t* indices, size_t ni,
                          const nb_primitive* prims, size_t np, uint32_t flags, HostScene* out) {
  auto t0 = std::chrono::steady_clock::now();
  if (nv > 0xFFFFFFFFull || ni > 0xFFFFFFFFull || np >= (size_t)kLeafBit)
    return fail(NB_ERR_INVALID_ARG, "scene too large");
  size_t nt = ni / 3;
  if (nt >= kLeafBit) return fail(NB_ERR_INVALID_ARG, "too many triangles");
  for (size_t i = 0; i < 3 * nt; ++i)
    if (indices[i] >= nv) return fail(NB_ERR_INVALID_ARG, "index %zu out of range (%u >= %zu)", i, indices[i], nv);
  for (size_t k = 0; k < np; ++k) {
    uint32_t s = prims[k].index_start / 3, e = prims[k].index_end / 3;
    if (e <= s || e > nt)
      return fail(NB_ERR_INVALID_ARG, "primitive %zu has an empty or out-of-range index range [%u, %u)", k,
                  prims[k].index_start, prims[k].index_end);
  }
  out->vertices.assign(vertices, vertices + nv);
  std::vector<Prim> tris(nt);
  triangle_cache(&vertices[0].position[0], sizeof(nb_vertex) / sizeof(float), indices, nt, tris.data());

  // group primitives by triangle range; distinct ranges must be disjoint for parallel builds
  std::map<std::pair<uint32_t, uint32_t>, std::vector<size_t>> groups;
  for (size_t k = 0; k < np; ++k) groups[{prims[k].index_start / 3, prims[k].index_end / 3}].push_back(k);
  std::vector<std::pair<std::pair<uint32_t, uint32_t>, std::vector<size_t>>> ranges(groups.begin(), groups.end());
  bool disjoint = true;
  for (size_t r = 1; r < ranges.size(); ++r)
    if (ranges[r].first.first < ranges[r - 1].first.second) disjoint = false;
  bool dedup = (flags & NB_SCENE_DEDUP_MESHES) != 0;

  // per primitive: private node list (root at local index 0) or a reference to the first occurrence
  std::vector<std::vector<nb_bvh_node>> local(np);
  std::vector<size_t> first_of(np);
  for (auto& g : ranges)
    for (size_t k : g.second) first_of[k] = g.second.front();
  auto build_group = [&](size_t gi) {
    auto& g = ranges[gi];
    const std::vector<size_t>& members = g.second;
    size_t reps = dedup ? 1 : members.size();
    for (size_t r = 0; r < reps; ++r)
      append_tree(local[members[r]], tris.data(), g.first.first, g.first.second);
  };
  if (disjoint) {
    // largest ranges first so the pool stays busy
    std::vector<size_t> order(ranges.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
      return (ranges[a].first.second - ranges[a].first.first) > (ranges[b].first.second - ranges[b].first.first);
    });
    run_parallel(order.size(), [&](size_t i) { build_group(order[i]); });
  } else {
    // overlapping distinct ranges: reproduce the reference's sequential appends exactly
    dedup = false;
    for (size_t k = 0; k < np; ++k) {
      first_of[k] = k;
      append_tree(local[k], tris.data(), prims[k].index_start / 3, prims[k].index_end / 3);
    }
  }

  // concatenate in primitive order (BVHTree::append numbering) and assemble instances
  out->blas.clear();
  std::vector<uint32_t> root_of(np);
  std::vector<Prim> bounds(np);
  std::vector<nb_instance> raw(np);
  for (size_t k = 0; k < np; ++k) {
    uint32_t root;
    if (dedup && first_of[k] != k) {
      root = root_of[first_of[k]];
    } else {
      uint32_t off = (uint32_t)out->blas.size();
      for (nb_bvh_node n : local[k]) {
        if (n.end == 0) n.start += off;
        out->blas.push_back(n);
      }
      root = off;
      std::vector<nb_bvh_node>().swap(local[k]);
    }
    root_of[k] = root;
    const nb_primitive& pr = prims[k];
    nb_instance& in = raw[k];
    std::memcpy(in.local_to_world, pr.local_to_world, 64);
    bool zero = true;
    for (float f : pr.world_to_local) zero &= (f == 0.0f);
    if (zero) {
      if (!invert4(pr.local_to_world, in.world_to_local))
        return fail(NB_ERR_INVALID_ARG, "primitive %zu: local_to_world is singular", k);
    } else {
      std::memcpy(in.world_to_local, pr.world_to_local, 64);
    }
    std::memcpy(in.color, pr.color, 16);
    in.roughness = pr.roughness;
    in.metallic = pr.metallic;
    in.emissive = pr.emissive;
    in.node = root;
    // InstanceWithBounds::approximate_from_instance (scene.rs:239-259)
    const nb_bvh_node& r = out->blas[root];
    float wmn[3] = {INFINITY, INFINITY, INFINITY}, wmx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
      float l[3] = {(c & 1) ? r.max[0] : r.min[0], (c & 2) ? r.max[1] : r.min[1], (c & 4) ? r.max[2] : r.min[2]};
      float w[3];
      transform_point3(in.local_to_world, l, w);
      for (int q = 0; q < 3; ++q) { wmn[q] = min_num(wmn[q], w[q]); wmx[q] = max_num(wmx[q], w[q]); }
    }
    for (int q = 0; q < 3; ++q) {
      bounds[k].mn[q] = wmn[q];
      bounds[k].mx[q] = wmx[q];
      bounds[k].c[q] = (wmn[q] + wmx[q]) * 0.5f;  // BVHPrimitive::center (bvh.rs:10-12)
    }
    bounds[k].payload = (uint32_t)k;
  }
  out->tlas.clear();
  if (np) append_tree(out->tlas, bounds.data(), 0, (uint32_t)np);
  out->instances.resize(np);
  for (size_t k = 0; k < np; ++k) out->instances[k] = raw[bounds[k].payload];
  out->indices.assign(indices, indices + ni);
  for (size_t t = 0; t < nt; ++t)
    for (int k = 0; k < 3; ++k) out->indices[3 * t + k] = indices[3 * tris[t].payload + k];
  out->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return NB_OK;
}

int adopt_reference_buffers(const nb_bvh_node* blas, size_t n_blas, const nb_bvh_node* tlas, size_t n_tlas,
                            const nb_instance* inst, size_t n_inst, const nb_vertex* v, size_t nv,
                            const uint32_t* idx, size_t ni, HostScene* out) {
  size_t nt = ni / 3;
  for (size_t i = 0; i < 3 * nt; ++i)
    if (idx[i] >= nv) return fail(NB_ERR_INVALID_ARG, "index %zu out of range", i);
  for (size_t i = 0; i < n_inst; ++i)
    if (inst[i].node >= n_blas) return fail(NB_ERR_INVALID_ARG, "instance %zu: BLAS root %u out of range", i, inst[i].node);
  if (n_inst && !n_tlas) return fail(NB_ERR_INVALID_ARG, "instances without a TLAS");
  out->vertices.assign(v, v + nv);
  out->indices.assign(idx, idx + ni);
  out->blas.assign(blas, blas + n_blas);
  out->tlas.assign(tlas, tlas + n_tlas);
  out->instances.assign(inst, inst + n_inst);
  out->build_ms = 0.0;
  return NB_OK;
}

namespace {

// Translates one reference tree into GpuNodes (preorder, left subtree first).  Returns the
// root reference; sets leaf lengths through `mark_leaf`.
template <class MarkLeaf>
int translate_tree(const std::vector<nb_bvh_node>& ref, uint32_t root, size_t n_prims, std::vector<GpuNode>* gpu,
                   std::vector<int64_t>* gpu_index, MarkLeaf&& mark_leaf, uint32_t* root_ref, uint32_t* depth_out) {
  auto ref_of = [&](uint32_t n, uint32_t* word) -> int {
    const nb_bvh_node& node = ref[n];
    if (node.end > 0) {
      if (node.start >= node.end || node.end > n_prims || node.start >= kLeafBit)
        return fail(NB_ERR_INVALID_ARG, "leaf node %u covers an invalid range [%u, %u)", n, node.start, node.end);
      int st = mark_leaf(node.start, node.end - node.start);
      if (st) return st;
      *word = kLeafBit | node.start;
      return NB_OK;
    }
    if ((*gpu_index)[n] < 0) return fail(NB_ERR_INVALID_ARG, "internal: unassigned node %u", n);
    *word = (uint32_t)(*gpu_index)[n];
    return NB_OK;
  };
  if (root >= ref.size()) return fail(NB_ERR_INVALID_ARG, "root %u out of range", root);
  uint32_t max_depth = 0;
  // assign indices in preorder, then fill records
  std::vector<std::pair<uint32_t, uint32_t>> stack{{root, 0u}};
  std::vector<uint32_t> order;
  while (!stack.empty()) {
    auto [n, d] = stack.back();
    stack.pop_back();
    max_depth = std::max(max_depth, d);
    const nb_bvh_node& node = ref[n];
    if (node.end > 0) continue;
    if ((*gpu_index)[n] >= 0) continue;  // shared subtree already translated
    if (d > 64) return fail(NB_ERR_INVALID_ARG, "BVH deeper than 64 levels");
    if ((size_t)node.start + 1 >= ref.size()) return fail(NB_ERR_INVALID_ARG, "inner node %u: child out of range", n);
    (*gpu_index)[n] = (int64_t)(gpu->size() + order.size());
    order.push_back(n);
    stack.emplace_back(node.start + 1, d + 1);
    stack.emplace_back(node.start, d + 1);
  }
  size_t base = gpu->size();
  gpu->resize(base + order.size());
  for (size_t i = 0; i < order.size(); ++i) {
    const nb_bvh_node& node = ref[order[i]];
    const nb_bvh_node& c0 = ref[node.start];
    const nb_bvh_node& c1 = ref[node.start + 1];
    GpuNode& g = (*gpu)[base + i];
    g.q0[0] = c0.min[0]; g.q0[1] = c0.max[0]; g.q0[2] = c0.min[1]; g.q0[3] = c0.max[1];
    g.q1[0] = c1.min[0]; g.q1[1] = c1.max[0]; g.q1[2] = c1.min[1]; g.q1[3] = c1.max[1];
    g.q2[0] = c0.min[2]; g.q2[1] = c0.max[2]; g.q2[2] = c1.min[2]; g.q2[3] = c1.max[2];
    int st = ref_of(node.start, &g.ref[0]);
    if (!st) st = ref_of(node.start + 1, &g.ref[1]);
    if (st) return st;
    g.pad[0] = g.pad[1] = 0;
  }
  int st = ref_of(root, root_ref);
  if (depth_out) *depth_out = max_depth;
  return st;
}

}  // namespace

int to_device_layout(HostScene* s) {
  size_t nt = s->indices.size() / 3;
  size_t nv = s->vertices.size();
  s->tris.assign(nt, GpuTri{});
  for (size_t t = 0; t < nt; ++t) {
    const float* a = s->vertices[s->indices[3 * t]].position;
    const float* b = s->vertices[s->indices[3 * t + 1]].position;
    const float* c = s->vertices[s->indices[3 * t + 2]].position;
    GpuTri& g = s->tris[t];
    for (int k = 0; k < 3; ++k) { g.v0[k] = a[k]; g.e1[k] = b[k] - a[k]; g.e2[k] = c[k] - a[k]; }
  }
  s->vattr.resize(nv);
  for (size_t i = 0; i < nv; ++i) {
    const nb_vertex& v = s->vertices[i];
    GpuVAttr& g = s->vattr[i];
    for (int k = 0; k < 3; ++k) { g.n[k] = v.normal[k]; g.t[k] = v.tangent[k]; }
    g.tw = v.tangent[3];
    g.pad = 0.0f;
  }
  // BLAS trees, one root table entry per distinct root node
  s->gblas.clear();
  s->blas_roots.clear();
  std::vector<int64_t> gidx(s->blas.size(), -1);
  std::map<uint32_t, uint32_t> root_id;
  auto mark_tri = [&](uint32_t start, uint32_t count) -> int {
    uint32_t& lc = s->tris[start].leaf_count;
    if (lc != 0 && lc != count)
      return fail(NB_ERR_INVALID_ARG, "triangle %u starts two leaves of different length", start);
    lc = count;
    return NB_OK;
  };
  size_t n_inst = s->instances.size();
  s->itrace.assign(n_inst, GpuInstTrace{});
  s->ishade.assign(n_inst, GpuInstShade{});
  for (size_t i = 0; i < n_inst; ++i) {
    const nb_instance& in = s->instances[i];
    auto it = root_id.find(in.node);
    uint32_t id;
    if (it == root_id.end()) {
      GpuRoot r{};
      const nb_bvh_node& rn = s->blas[in.node];
      for (int k = 0; k < 3; ++k) { r.mn[k] = rn.min[k]; r.mx[k] = rn.max[k]; }
      int st = translate_tree(s->blas, in.node, nt, &s->gblas, &gidx, mark_tri, &r.ref, nullptr);
      if (st) return st;
      id = (uint32_t)s->blas_roots.size();
      s->blas_roots.push_back(r);
      root_id[in.node] = id;
    } else {
      id = it->second;
    }
    GpuInstTrace& tr = s->itrace[i];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c) tr.row[r][c] = in.world_to_local[4 * c + r];
    tr.blas_root = id;
    GpuInstShade& sh = s->ishade[i];
    for (int c = 0; c < 3; ++c) {
      for (int k = 0; k < 3; ++k) sh.w2l_col[c][k] = in.world_to_local[4 * c + k];
      sh.w2l_col[c][3] = in.color[c];
    }
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 3; ++k) sh.l2w_row[r][k] = in.local_to_world[4 * k + r];
    sh.l2w_row[0][3] = in.roughness;
    sh.l2w_row[1][3] = in.metallic;
    sh.l2w_row[2][3] = in.emissive;
  }
  // TLAS
  s->gtlas.clear();
  s->has_tlas = !s->tlas.empty() && n_inst > 0;
  if (s->has_tlas) {
    std::vector<int64_t> tidx(s->tlas.size(), -1);
    auto mark_inst = [&](uint32_t start, uint32_t count) -> int {
      uint32_t& lc = s->itrace[start].leaf_count;
      if (lc != 0 && lc != count) return fail(NB_ERR_INVALID_ARG, "instance %u starts two TLAS leaves", start);
      lc = count;
      return NB_OK;
    };
    GpuRoot r{};
    const nb_bvh_node& rn = s->tlas[0];  // raytracing_sw.wgsl:183-186: the TLAS root is node 0
    for (int k = 0; k < 3; ++k) { r.mn[k] = rn.min[k]; r.mx[k] = rn.max[k]; }
    int st = translate_tree(s->tlas, 0, n_inst, &s->gtlas, &tidx, mark_inst, &r.ref, nullptr);
    if (st) return st;
    s->tlas_root = r;
  }
  return NB_OK;
}

}  // namespace nb

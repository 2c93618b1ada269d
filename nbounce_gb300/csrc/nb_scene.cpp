// Host side of the scene: the reference's SAH BVH builder (src/pathtracing/bvh.rs), the
// BLAS/TLAS assembly of SceneBuffers::from_scene (src/pathtracing/scene.rs:280-305), and the
// translation of those reference-layout trees into the device layout (nb_internal.h).
//
// The builder reproduces bvh.rs node for node: 16-bin binned SAH above 11 primitives,
// brute-force SAH for 3..11, the manual split for 2, cost = count * (xy + xz + yz) with no
// traversal constant, MAX_DEPTH 32, explicit DFS stack (children appended at len, len+1;
// right child processed first) and the unstable in-place swap partition.  Rust evaluates
// f32 arithmetic without contraction; this file is compiled with -ffp-contract=off to match.
// The one deliberate difference from the reference is parallelism, at two levels, both with
// an identical result: distinct BLASes (disjoint triangle ranges) are built on worker threads
// into private node lists that are concatenated in primitive order with their indices
// offset, and large subtrees inside one BLAS are split on separate threads, after which the
// reference's node numbering is replayed (append_tree_parallel).
//
// The device trees (to_device_layout) are the reference BLAS trees collapsed to 8-wide nodes,
// and a device TLAS of our own over tight world boxes of instances and of the parts of large
// instances (tlas_entries, entry_boxes); the reference TLAS itself is kept for export.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
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

// f(i) for i in [0, n) over up to 16 threads in chunks (f writes only its own elements)
template <class F>
void parallel_for(size_t n, F f) {
  const size_t chunk = 1 << 16;
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const size_t n_chunks = (n + chunk - 1) / chunk;
  if (hw == 1 || n_chunks < 2) {
    for (size_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (unsigned w = 0; w < std::min<size_t>(hw, n_chunks); ++w)
    pool.emplace_back([&] {
      for (size_t c; (c = next.fetch_add(1)) < n_chunks;)
        for (size_t i = c * chunk, e = std::min(n, i + chunk); i < e; ++i) f(i);
    });
  for (std::thread& th : pool) th.join();
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

// Parallel form of append_tree with an identical result.  A node's split depends only on the
// primitives of its own range, and sibling ranges are disjoint, so subtrees above a size
// threshold are split on separate threads.  The reference numbers nodes in the order its
// right-first DFS splits them (children at len, len + 1); replaying that DFS over the finished
// structure reproduces the numbering, and the in-place partitions leave the same permutation.
// Ranges too small to spawn anywhere below them (under 2 kParallelMin primitives, or no spawn
// depth left) are built by the sequential DFS into a flat array, spliced into the numbering by
// the replay, instead of one heap node per split.
struct TreeNode {
  nb_bvh_node n;
  std::unique_ptr<TreeNode> lo, hi;
  std::vector<nb_bvh_node> flat;  // sequential subtree: flat[0] is n, children at local indices
};

// append_tree's DFS from an already bounded root at depth0, into a fresh array (root at 0)
void append_subtree(std::vector<nb_bvh_node>& nodes, Prim* p, const nb_bvh_node& root, uint32_t depth0) {
  constexpr uint32_t kMaxDepth = 32;
  nodes.push_back(root);
  std::vector<std::pair<uint32_t, uint32_t>> stack;
  stack.emplace_back(depth0, 0u);
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
}

void split_recursive(Prim* p, TreeNode* t, uint32_t depth, int spawn_depth) {
  constexpr uint32_t kMaxDepth = 32;
  constexpr uint32_t kParallelMin = 1u << 15;
  if (depth >= kMaxDepth) return;
  if (spawn_depth <= 0 || t->n.end - t->n.start < 2 * kParallelMin) {
    append_subtree(t->flat, p, t->n, depth);
    return;
  }
  nb_bvh_node lo, hi;
  if (!split_node(p, t->n, &lo, &hi)) return;
  t->lo.reset(new TreeNode{lo, nullptr, nullptr});
  t->hi.reset(new TreeNode{hi, nullptr, nullptr});
  if (spawn_depth > 0 && lo.end - lo.start >= kParallelMin && hi.end - hi.start >= kParallelMin) {
    std::thread th(split_recursive, p, t->lo.get(), depth + 1, spawn_depth - 1);
    split_recursive(p, t->hi.get(), depth + 1, spawn_depth - 1);
    th.join();
  } else {
    split_recursive(p, t->lo.get(), depth + 1, spawn_depth);
    split_recursive(p, t->hi.get(), depth + 1, spawn_depth);
  }
}

uint32_t append_tree_parallel(std::vector<nb_bvh_node>& nodes, Prim* p, uint32_t s, uint32_t e, int spawn_depth) {
  TreeNode root{leaf_over(p, s, e), nullptr, nullptr};
  split_recursive(p, &root, 0, spawn_depth);
  uint32_t root_index = (uint32_t)nodes.size();
  nodes.push_back(root.n);
  std::vector<std::pair<const TreeNode*, uint32_t>> stack{{&root, root_index}};
  while (!stack.empty()) {
    auto [t, idx] = stack.back();
    stack.pop_back();
    if (!t->flat.empty()) {
      // the subtree's DFS numbers its nodes after the current end, in its own order: local
      // node j (j >= 1) becomes base + j - 1
      const std::vector<nb_bvh_node>& f = t->flat;
      if (f.size() > 1) {
        const uint32_t base = (uint32_t)nodes.size() - 1;
        nodes[idx].end = 0;
        nodes[idx].start = base + f[0].start;
        for (size_t j = 1; j < f.size(); ++j) {
          nb_bvh_node n = f[j];
          if (n.end == 0) n.start += base;
          nodes.push_back(n);
        }
      }
      continue;
    }
    if (!t->lo) continue;
    uint32_t li = (uint32_t)nodes.size();
    nodes[idx].end = 0;
    nodes[idx].start = li;
    nodes.push_back(t->lo->n);
    nodes.push_back(t->hi->n);
    stack.emplace_back(t->lo.get(), li);
    stack.emplace_back(t->hi.get(), li + 1);
  }
  return root_index;
}

int spawn_depth_for(uint32_t n) {
  unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  int d = 0;
  while ((1u << d) < hw && d < 6) ++d;
  return n >= (1u << 16) ? d : 0;
}

void triangle_cache(const float* pos, size_t pos_stride, const uint32_t* idx, size_t nt, Prim* out) {
  parallel_for(nt, [&](size_t t) {
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
  });
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
  if (nt) append_tree_parallel(*nodes, tris.data(), 0, (uint32_t)nt, spawn_depth_for((uint32_t)nt));
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
      append_tree_parallel(local[members[r]], tris.data(), g.first.first, g.first.second,
                           spawn_depth_for(g.first.second - g.first.first));
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

  // concatenate in primitive order (BVHTree::append numbering): the offsets first, then the
  // trees copied into place in parallel; then assemble the instances
  std::vector<uint32_t> root_of(np);
  std::vector<Prim> bounds(np);
  std::vector<nb_instance> raw(np);
  size_t total = 0;
  for (size_t k = 0; k < np; ++k) {
    if (dedup && first_of[k] != k) {
      root_of[k] = root_of[first_of[k]];
    } else {
      root_of[k] = (uint32_t)total;
      total += local[k].size();
    }
  }
  out->blas.assign(total, nb_bvh_node{});
  run_parallel(np, [&](size_t k) {
    if (dedup && first_of[k] != k) return;
    const uint32_t off = root_of[k];
    nb_bvh_node* dst = out->blas.data() + off;
    for (size_t j = 0; j < local[k].size(); ++j) {
      nb_bvh_node n = local[k][j];
      if (n.end == 0) n.start += off;
      dst[j] = n;
    }
    std::vector<nb_bvh_node>().swap(local[k]);
  });
  for (size_t k = 0; k < np; ++k) {
    const uint32_t root = root_of[k];
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
  parallel_for(nt, [&](size_t t) {
    for (int k = 0; k < 3; ++k) out->indices[3 * t + k] = indices[3 * tris[t].payload + k];
  });
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

// ---------------------------------------------------------------------------------------
// 8-wide device trees
//
// Each reference tree is collapsed into a tree of 8-wide nodes.  Leaf slots are the maximal
// subtrees of at most max_leaf contiguous primitives (a reference leaf with more counts as an
// inner node over its two contiguous halves): 2 triangles in a BLAS, 1 instance in the TLAS
// (the slot metadata holds at most 3).  Which binary nodes become wide nodes is chosen by the
// SAH-optimal dynamic programme of Ylitie, Karras and Laine 2017 ("Efficient incoherent ray
// traversal on GPUs through compressed wide BVHs", section 3): C(x, i) is the least cost of
// covering the subtree of x with at most i child slots, where a leaf slot costs nothing (every
// cover tests the same leaves) and a child wide node costs its box area plus the best cover of
// its own subtree with 8 slots - i.e. the expected number of wide-node visits of a random ray.
// Measured on the benchmark frame against the greedy collapse that opens the largest-area item
// first: 35% fewer BLAS nodes and 3% more rays/s; letting the programme also choose leaf sizes
// (1 to 3 triangles, with a triangle-test weight) was 0.3-1.5% slower than fixed 2-triangle
// leaves.  Nodes are emitted breadth-first so the inner children of a node are contiguous,
// and the primitives of a node's leaf slots are written contiguously, in slot order, into a
// new primitive order.  Traversal finds the same closest hit: the wide BLAS trees cover the
// same triangles with boxes that contain the reference boxes, and the device TLAS covers every
// instance's geometry; only the visiting order (exact-t ties) can differ.
// ---------------------------------------------------------------------------------------
struct Item {
  bool inner;       // inner binary node (else: primitive range)
  uint32_t node;    // binary node index (inner)
  uint32_t start, count;  // primitive range (range items)
  float mn[3], mx[3];  // the reference node's box, or the union of a range's primitive boxes
  double area() const {
    double e0 = (double)mx[0] - mn[0], e1 = (double)mx[1] - mn[1], e2 = (double)mx[2] - mn[2];
    return e0 * e1 + e0 * e2 + e1 * e2;
  }
};

struct Collapser {
  const std::vector<nb_bvh_node>& ref;
  // primitive boxes (float), indexed by reference primitive index
  const std::vector<float>& prim_box;  // 6 floats per primitive: min xyz, max xyz
  std::vector<WideNode>* out;
  std::vector<uint32_t>* prim_order;   // new order -> reference primitive index
  uint32_t max_leaf;                   // primitives per leaf slot (2 triangles, 1 instance; <= 3)

  struct Span {
    uint32_t first = 0xFFFFFFFFu, end = 0, count = 0;
  };
  // memo: primitive range and leaf count of a subtree, one entry per binary node, sized by the
  // caller; collapsers of disjoint trees share it (each writes only its own nodes' entries)
  std::vector<Span>* span = nullptr;

  // [first, end) of the primitives below binary node n.  bvh.rs partitions in place, so a
  // subtree covers a contiguous range (count == end - first); trees handed in through
  // nb_scene_create_from_bvh are only trusted where that holds.
  Span subtree_span(uint32_t n) const {
    std::vector<Span>& memo = *span;
    if (memo[n].first != 0xFFFFFFFFu) return memo[n];
    const nb_bvh_node& b = ref[n];
    Span r;
    if (b.end > 0) {
      r = Span{b.start, b.end, b.end - b.start};
    } else {
      Span l = subtree_span(b.start), h = subtree_span(b.start + 1);
      r = Span{std::min(l.first, h.first), std::max(l.end, h.end), l.count + h.count};
    }
    memo[n] = r;
    return r;
  }

  // a binary node becomes an item; subtrees of at most max_leaf primitives become one leaf
  Item item_of(uint32_t n) const {
    const nb_bvh_node& b = ref[n];
    Item it{};
    it.inner = b.end == 0;
    it.node = n;
    it.start = b.start;
    it.count = b.end > 0 ? b.end - b.start : 0;
    if (it.inner) {
      const Span r = subtree_span(n);
      if (r.count <= max_leaf && r.end - r.first == r.count) {
        it.inner = false;
        it.start = r.first;
        it.count = r.count;
      }
    }
    for (int k = 0; k < 3; ++k) { it.mn[k] = b.min[k]; it.mx[k] = b.max[k]; }
    return it;
  }
  Item range_item(uint32_t start, uint32_t count) const {
    Item it{};
    it.inner = false;
    it.start = start;
    it.count = count;
    for (int k = 0; k < 3; ++k) { it.mn[k] = INFINITY; it.mx[k] = -INFINITY; }
    for (uint32_t i = start; i < start + count; ++i)
      for (int k = 0; k < 3; ++k) {
        it.mn[k] = std::min(it.mn[k], prim_box[6 * (size_t)i + k]);
        it.mx[k] = std::max(it.mx[k], prim_box[6 * (size_t)i + 3 + k]);
      }
    return it;
  }
  // inner nodes split into their children, oversized leaves into two contiguous halves
  bool expandable(const Item& it) const { return it.inner || it.count > max_leaf; }
  void expand(const Item& it, std::vector<Item>* v) const {
    if (it.inner) {
      v->push_back(item_of(ref[it.node].start));
      v->push_back(item_of(ref[it.node].start + 1));
    } else {
      uint32_t h = it.count / 2;
      v->push_back(range_item(it.start, h));
      v->push_back(range_item(it.start + h, it.count - h));
    }
  }

  // quantise child boxes of one wide node on a per-axis power-of-two grid
  static void quantise(WideNode* w, const std::vector<Item>& slots) {
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (const Item& c : slots)
      for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], (double)c.mn[k]); hi[k] = std::max(hi[k], (double)c.mx[k]); }
    uint8_t* qlo[3] = {w->qlo_x, w->qlo_y, w->qlo_z};
    uint8_t* qhi[3] = {w->qhi_x, w->qhi_y, w->qhi_z};
    for (int k = 0; k < 3; ++k) {
      // p rounded down so that p <= every child's min
      float p = (float)lo[k];
      if ((double)p > lo[k]) p = std::nextafter(p, -INFINITY);
      double ext = hi[k] - (double)p;
      int e = ext > 0.0 ? (int)std::ceil(std::log2(ext / 255.0)) : -100;
      e = std::max(e, -126);
      for (;; ++e) {
        double scale = std::ldexp(1.0, e);
        bool ok = true;
        for (size_t i = 0; i < slots.size() && ok; ++i) {
          double ql = std::floor(((double)slots[i].mn[k] - p) / scale);
          double qh = std::ceil(((double)slots[i].mx[k] - p) / scale);
          while (ql > 0 && p + ql * scale > slots[i].mn[k]) ql -= 1;
          while (p + qh * scale < slots[i].mx[k]) qh += 1;
          if (ql < 0 || qh > 255) { ok = false; break; }
          qlo[k][i] = (uint8_t)ql;
          qhi[k][i] = (uint8_t)qh;
        }
        if (ok) break;
      }
      w->p[k] = p;
      w->e[k] = (uint8_t)(e + 127);
    }
  }

  // binary tree below a root (children stored after their parent) with its cost tables;
  // nodes without children are the leaf slots
  struct DpNode {
    Item it;
    int32_t l = -1, r = -1;
    float cost[8] = {};     // C(x, i + 1)
    uint8_t split[8] = {};  // best slots for the left child when covering with i + 1 slots
    uint8_t fewer = 0; // bit i: C(x, i + 1) = C(x, i)
  };
  std::vector<DpNode> dp;

  void dp_prepare(const Item& root) {
    dp.clear();
    dp.push_back(DpNode{root});
    std::vector<Item> two;
    for (size_t x = 0; x < dp.size(); ++x) {
      if (!expandable(dp[x].it)) continue;
      two.clear();
      expand(dp[x].it, &two);
      dp[x].l = (int32_t)dp.size();
      dp[x].r = (int32_t)dp.size() + 1;
      dp.push_back(DpNode{two[0]});
      dp.push_back(DpNode{two[1]});
    }
    for (size_t x = dp.size(); x-- > 0;) {
      DpNode& n = dp[x];
      if (n.l < 0) {
        for (int i = 0; i < 8; ++i) n.cost[i] = 0.0f;
        continue;
      }
      const DpNode& lo = dp[n.l];
      const DpNode& hi = dp[n.r];
      float d[9];
      for (int j = 2; j <= 8; ++j) {
        d[j] = INFINITY;
        for (int k = 1; k < j; ++k) {
          const float c = lo.cost[k - 1] + hi.cost[j - k - 1];
          if (c < d[j]) {
            d[j] = c;
            n.split[j - 1] = (uint8_t)k;
          }
        }
      }
      n.cost[0] = (float)n.it.area() + d[8];
      n.fewer = 0;
      for (int i = 2; i <= 8; ++i) {
        if (n.cost[i - 2] <= d[i]) {
          n.cost[i - 1] = n.cost[i - 2];
          n.fewer |= (uint8_t)(1u << (i - 1));
        } else {
          n.cost[i - 1] = d[i];
        }
      }
    }
  }

  // the slot roots of the best cover of x with at most i slots
  void dp_collect(int32_t x, int i, std::vector<int32_t>* out) const {
    const DpNode& n = dp[x];
    while (i > 1 && n.l >= 0 && ((n.fewer >> (i - 1)) & 1u)) --i;
    if (i == 1 || n.l < 0) {
      out->push_back(x);
      return;
    }
    const int k = n.split[i - 1];
    dp_collect(n.l, k, out);
    dp_collect(n.r, i - k, out);
  }

  // builds the wide tree rooted at binary node `root`; returns the index of its root
  uint32_t build(uint32_t root) {
    dp_prepare(item_of(root));
    std::vector<int32_t> queue{0};
    size_t head = 0;
    const uint32_t base = (uint32_t)out->size();
    out->push_back(WideNode{});
    std::vector<int32_t> items;
    while (head < queue.size()) {
      const int32_t cur = queue[head];
      const uint32_t self = base + (uint32_t)head;
      ++head;
      items.clear();
      if (dp[cur].l >= 0) {
        const int k = dp[cur].split[7];
        dp_collect(dp[cur].l, k, &items);
        dp_collect(dp[cur].r, 8 - k, &items);
      } else {
        items.push_back(cur);
      }
      WideNode w{};
      std::vector<Item> slots;
      w.child_base = (uint32_t)out->size();
      w.prim_base = (uint32_t)prim_order->size();
      uint32_t n_inner = 0, offset = 0;
      for (const int32_t x : items) {
        const Item& it = dp[x].it;
        uint8_t meta;
        if (dp[x].l >= 0) {
          meta = (uint8_t)(0x80u | n_inner);
          ++n_inner;
          queue.push_back(x);
          out->push_back(WideNode{});
        } else {
          meta = (uint8_t)((it.count << 5) | offset);
          for (uint32_t i = it.start; i < it.start + it.count; ++i) prim_order->push_back(i);
          offset += it.count;
        }
        w.meta[slots.size()] = meta;
        slots.push_back(it);
      }
      w.n_children = (uint8_t)slots.size();
      quantise(&w, slots);
      (*out)[self] = w;
    }
    std::vector<DpNode>().swap(dp);
    return base;
  }
};

void tri_boxes(const HostScene& s, std::vector<float>* box) {
  size_t nt = s.indices.size() / 3;
  box->resize(6 * nt);
  parallel_for(nt, [&](size_t t) {
    const float* a = s.vertices[s.indices[3 * t]].position;
    const float* b = s.vertices[s.indices[3 * t + 1]].position;
    const float* c = s.vertices[s.indices[3 * t + 2]].position;
    for (int k = 0; k < 3; ++k) {
      (*box)[6 * t + k] = std::min(std::min(a[k], b[k]), c[k]);
      (*box)[6 * t + 3 + k] = std::max(std::max(a[k], b[k]), c[k]);
    }
  });
}

int check_tree(const std::vector<nb_bvh_node>& ref, uint32_t root, size_t n_prims) {
  if (root >= ref.size()) return fail(NB_ERR_INVALID_ARG, "root %u out of range", root);
  std::vector<std::pair<uint32_t, uint32_t>> stack{{root, 0u}};
  size_t visited = 0;
  while (!stack.empty()) {
    auto [n, d] = stack.back();
    stack.pop_back();
    if (++visited > 2 * ref.size() + 2) return fail(NB_ERR_INVALID_ARG, "BVH contains a cycle");
    const nb_bvh_node& node = ref[n];
    if (node.end > 0) {
      if (node.start >= node.end || node.end > n_prims || node.start >= kLeafBit)
        return fail(NB_ERR_INVALID_ARG, "leaf node %u covers an invalid range [%u, %u)", n, node.start, node.end);
      continue;
    }
    if (d > 64) return fail(NB_ERR_INVALID_ARG, "BVH deeper than 64 levels");
    if ((size_t)node.start + 1 >= ref.size()) return fail(NB_ERR_INVALID_ARG, "inner node %u: child out of range", n);
    stack.emplace_back(node.start, d + 1);
    stack.emplace_back(node.start + 1, d + 1);
  }
  return NB_OK;
}

// true if no binary node lies below two of the roots (trees from the reference builder never
// share nodes; trees handed in through nb_scene_create_from_bvh may)
bool disjoint_trees(const std::vector<nb_bvh_node>& ref, const std::vector<uint32_t>& roots) {
  std::vector<uint8_t> seen(ref.size(), 0);
  std::vector<uint32_t> stack;
  for (uint32_t root : roots) {
    stack.assign(1, root);
    while (!stack.empty()) {
      const uint32_t n = stack.back();
      stack.pop_back();
      if (seen[n]) return false;
      seen[n] = 1;
      if (ref[n].end == 0) {
        stack.push_back(ref[n].start);
        stack.push_back(ref[n].start + 1);
      }
    }
  }
  return true;
}

// world box of an instance: the 8 corners of its BLAS root box through local_to_world
// (InstanceWithBounds::approximate_from_instance, scene.rs:239-259)
void instance_box(const nb_instance& in, const nb_bvh_node& r, float* box) {
  float wmn[3] = {INFINITY, INFINITY, INFINITY}, wmx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int c = 0; c < 8; ++c) {
    float l[3] = {(c & 1) ? r.max[0] : r.min[0], (c & 2) ? r.max[1] : r.min[1], (c & 4) ? r.max[2] : r.min[2]};
    float w[3];
    transform_point3(in.local_to_world, l, w);
    for (int q = 0; q < 3; ++q) { wmn[q] = min_num(wmn[q], w[q]); wmx[q] = max_num(wmx[q], w[q]); }
  }
  for (int q = 0; q < 3; ++q) { box[q] = wmn[q]; box[3 + q] = wmx[q]; }
}

// Entries of the device TLAS: an instance and the wide BLAS node its traversal starts at.
// An instance whose world box (the transformed BLAS root box the reference builds its TLAS
// over) has more than kRebraidArea of the scene's box area, and whose BLAS root has only
// inner children, enters once per child (partial re-braiding, Benthin et al. 2017, "Improved
// two-level BVHs using partial re-braiding"): the TLAS can then cull the parts of a large
// instance - the benchmark scene's terrain - that a ray misses, while small instances, for
// which a second entry would only repeat the ray transform, enter once.  Measured on the
// benchmark frame: 1452 -> 1518 Mrays/s; splitting every instance whose root has only inner
// children: 1409.
constexpr double kRebraidArea = 0.02;
struct TlasEntry {
  uint32_t inst, node;
};

std::vector<TlasEntry> tlas_entries(const HostScene& s, const std::vector<uint32_t>& inst_blas) {
  auto area = [](const float* lo, const float* hi) {
    const double x = (double)hi[0] - lo[0], y = (double)hi[1] - lo[1], z = (double)hi[2] - lo[2];
    return x * y + x * z + y * z;
  };
  const double scene = area(s.tlas[0].min, s.tlas[0].max);
  std::vector<TlasEntry> e;
  for (size_t i = 0; i < s.instances.size(); ++i) {
    const uint32_t root = s.wblas_root[inst_blas[i]];
    const WideNode& w = s.wblas[root];
    bool split = w.n_children > 1;
    for (int k = 0; k < w.n_children; ++k) split = split && (w.meta[k] & 0x80u);
    if (split) {
      float ib[6];
      instance_box(s.instances[i], s.blas[s.instances[i].node], ib);
      split = area(ib, ib + 3) > kRebraidArea * scene;
    }
    if (split) {
      for (int k = 0; k < w.n_children; ++k) e.push_back({(uint32_t)i, w.child_base + (w.meta[k] & 7u)});
    } else {
      e.push_back({(uint32_t)i, root});
    }
  }
  return e;
}

// World boxes of the TLAS entries: the bounds of the vertices below the entry's wide node
// under the instance's local_to_world, in double, widened by 1e-5 of the box's largest
// extent plus 1e-6 of its coordinates' magnitude (the binary32 transforms on either side
// round at ~1e-7 relative) and rounded outward to float.  For a rotated instance this is much
// tighter than the box of its transformed BLAS root box (a rotated box's corners reach up to
// sqrt(3) times further out per axis than a round mesh inside it: 1357 -> 1452 Mrays/s on the
// benchmark frame).  Traversal stays conservative: every box contains its entry's geometry.
void entry_boxes(const HostScene& s, const std::vector<uint32_t>& tri_order, const std::vector<TlasEntry>& e,
                 std::vector<Prim>* out) {
  // the distinct wide nodes the entries start at, and the vertices below each (unique, in
  // order of first use: only their bounds are taken), gathered in parallel
  std::map<uint32_t, size_t> node_idx;
  std::vector<uint32_t> nodes;
  for (const TlasEntry& en : e)
    if (node_idx.emplace(en.node, nodes.size()).second) nodes.push_back(en.node);
  std::vector<std::vector<uint32_t>> verts(nodes.size());
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  auto gather = [&](size_t k, std::vector<uint8_t>& mark) {
    std::vector<uint32_t>& v = verts[k];
    std::vector<uint32_t> st{nodes[k]};
    while (!st.empty()) {
      const WideNode& w = s.wblas[st.back()];
      st.pop_back();
      for (int c = 0; c < w.n_children; ++c) {
        const uint32_t meta = w.meta[c];
        if (meta & 0x80u) {
          st.push_back(w.child_base + (meta & 7u));
          continue;
        }
        const uint32_t first = w.prim_base + (meta & 31u), cnt = meta >> 5;
        for (uint32_t j = 0; j < cnt; ++j) {
          const uint32_t t = tri_order[first + j];
          for (int q = 0; q < 3; ++q) {
            const uint32_t vi = s.indices[3 * (size_t)t + q];
            if (!mark[vi]) {
              mark[vi] = 1;
              v.push_back(vi);
            }
          }
        }
      }
    }
    for (uint32_t vi : v) mark[vi] = 0;
  };
  {
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (unsigned w = 0; w < std::min<size_t>(hw, nodes.size()); ++w)
      pool.emplace_back([&] {
        std::vector<uint8_t> mark(s.vertices.size(), 0);
        for (size_t k; (k = next.fetch_add(1)) < nodes.size();) gather(k, mark);
      });
    for (std::thread& th : pool) th.join();
  }
  out->assign(e.size(), Prim{});
  auto one = [&](size_t j) {
    const nb_instance& in = s.instances[e[j].inst];
    const std::vector<uint32_t>& v = verts[node_idx.at(e[j].node)];
    Prim& p = (*out)[j];
    p.payload = (uint32_t)j;
    if (v.empty()) {  // no geometry: the transformed root box
      float ib[6];
      instance_box(in, s.blas[in.node], ib);
      for (int r = 0; r < 3; ++r) { p.mn[r] = ib[r]; p.mx[r] = ib[3 + r]; p.c[r] = (p.mn[r] + p.mx[r]) * 0.5f; }
      return;
    }
    const float* m = in.local_to_world;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t vi : v) {
      const float* q = s.vertices[vi].position;
      for (int r = 0; r < 3; ++r) {
        const double w = (double)m[r] * q[0] + (double)m[4 + r] * q[1] + (double)m[8 + r] * q[2] + (double)m[12 + r];
        lo[r] = std::min(lo[r], w);
        hi[r] = std::max(hi[r], w);
      }
    }
    const double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
    for (int r = 0; r < 3; ++r) {
      const double pad = 1e-5 * ext + 1e-6 * std::max(std::fabs(lo[r]), std::fabs(hi[r]));
      p.mn[r] = std::nextafter((float)(lo[r] - pad), -INFINITY);
      p.mx[r] = std::nextafter((float)(hi[r] + pad), INFINITY);
      p.c[r] = (p.mn[r] + p.mx[r]) * 0.5f;
    }
  };
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (unsigned w = 0; w < hw; ++w)
    pool.emplace_back([&] {
      for (size_t j; (j = next.fetch_add(1)) < e.size();) one(j);
    });
  for (std::thread& th : pool) th.join();
}

}  // namespace

int to_device_layout(HostScene* s) {
  const size_t nt = s->indices.size() / 3;
  const size_t nv = s->vertices.size();
  const size_t n_inst = s->instances.size();
  std::vector<float> tbox;
  tri_boxes(*s, &tbox);

  // BLAS: one wide tree per distinct root (in order of first use); triangles re-ordered per
  // wide tree.  Disjoint trees are collapsed in parallel into their own arrays and appended in
  // order, their node and triangle indices moved by the sizes before them: the same arrays as
  // collapsing them one after the other.
  s->wblas.clear();
  s->wblas_root.clear();
  std::vector<uint32_t> tri_order;
  std::map<uint32_t, uint32_t> root_id;
  std::vector<uint32_t> roots;
  std::vector<uint32_t> inst_blas(n_inst);
  for (size_t i = 0; i < n_inst; ++i) {
    const uint32_t root = s->instances[i].node;
    auto it = root_id.find(root);
    if (it == root_id.end()) {
      int st = check_tree(s->blas, root, nt);
      if (st) return st;
      it = root_id.emplace(root, (uint32_t)roots.size()).first;
      roots.push_back(root);
    }
    inst_blas[i] = it->second;
  }
  std::vector<Collapser::Span> memo(s->blas.size());
  std::vector<std::vector<WideNode>> wide(roots.size());
  std::vector<std::vector<uint32_t>> order(roots.size());
  auto collapse = [&](size_t k) {
    Collapser cb{s->blas, tbox, &wide[k], &order[k], 2, &memo};
    cb.build(roots[k]);  // the root is the first node of its array
  };
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (roots.size() > 1 && hw > 1 && disjoint_trees(s->blas, roots)) {
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (unsigned w = 0; w < std::min<size_t>(hw, roots.size()); ++w)
      pool.emplace_back([&] {
        for (size_t k; (k = next.fetch_add(1)) < roots.size();) collapse(k);
      });
    for (std::thread& th : pool) th.join();
  } else {
    for (size_t k = 0; k < roots.size(); ++k) collapse(k);
  }
  for (size_t k = 0; k < roots.size(); ++k) {
    const uint32_t node_off = (uint32_t)s->wblas.size(), prim_off = (uint32_t)tri_order.size();
    s->wblas_root.push_back(node_off);
    for (WideNode w : wide[k]) {
      w.child_base += node_off;
      w.prim_base += prim_off;
      s->wblas.push_back(w);
    }
    tri_order.insert(tri_order.end(), order[k].begin(), order[k].end());
    std::vector<WideNode>().swap(wide[k]);
    std::vector<uint32_t>().swap(order[k]);
  }
  s->tris.assign(tri_order.size(), GpuTri{});
  parallel_for(tri_order.size(), [&](size_t k) {
    const uint32_t t = tri_order[k];
    const float* a = s->vertices[s->indices[3 * t]].position;
    const float* b = s->vertices[s->indices[3 * t + 1]].position;
    const float* c = s->vertices[s->indices[3 * t + 2]].position;
    GpuTri& g = s->tris[k];
    for (int q = 0; q < 3; ++q) { g.v0[q] = a[q]; g.e1[q] = b[q] - a[q]; g.e2[q] = c[q] - a[q]; }
    g.pad0 = 0;
    g.ref_index = t;
    g.pad2 = 0;
  });
  s->vattr.resize(nv);
  parallel_for(nv, [&](size_t i) {
    const nb_vertex& v = s->vertices[i];
    GpuVAttr& g = s->vattr[i];
    for (int k = 0; k < 3; ++k) { g.n[k] = v.normal[k]; g.t[k] = v.tangent[k]; }
    g.tw = v.tangent[3];
    g.pad = 0.0f;
  });

  // TLAS over the entries (tlas_entries, entry_boxes): the reference's SAH build over their
  // boxes, collapsed like the BLAS; entries re-ordered by the wide TLAS
  s->wtlas.clear();
  s->itrace.clear();
  s->tlas_entries = 0;
  s->ishade.assign(n_inst, GpuInstShade{});
  s->has_tlas = !s->tlas.empty() && n_inst > 0;
  if (s->has_tlas) {
    int st = check_tree(s->tlas, 0, n_inst);
    if (st) return st;
    const std::vector<TlasEntry> entries = tlas_entries(*s, inst_blas);
    std::vector<Prim> eb;
    entry_boxes(*s, tri_order, entries, &eb);
    std::vector<nb_bvh_node> tlas;
    append_tree(tlas, eb.data(), 0, (uint32_t)eb.size());
    std::vector<float> ebox(6 * eb.size());
    for (size_t k = 0; k < eb.size(); ++k)
      for (int q = 0; q < 3; ++q) { ebox[6 * k + q] = eb[k].mn[q]; ebox[6 * k + 3 + q] = eb[k].mx[q]; }
    std::vector<uint32_t> order;
    std::vector<Collapser::Span> tmemo(tlas.size());
    Collapser ct{tlas, ebox, &s->wtlas, &order, 1, &tmemo};
    ct.build(0);  // raytracing_sw.wgsl:183-186: the TLAS root is node 0
    s->itrace.assign(order.size(), GpuInstTrace{});
    s->tlas_entries = order.size();
    for (size_t k = 0; k < order.size(); ++k) {
      const TlasEntry& en = entries[eb[order[k]].payload];
      const nb_instance& in = s->instances[en.inst];
      GpuInstTrace& tr = s->itrace[k];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) tr.row[r][c] = in.world_to_local[4 * c + r];
      tr.blas_root = en.node;
      tr.ref_index = en.inst;
    }
  }
  for (size_t i = 0; i < n_inst; ++i) {
    const nb_instance& in = s->instances[i];
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
  return NB_OK;
}

}  // namespace nb

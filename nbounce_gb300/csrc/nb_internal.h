// Internal declarations shared by the host builder (nb_scene.cpp), the Sobol generator
// (nb_sobol.cpp) and the CUDA side (nb_api.cu / nb_kernels.cu).
//
// Device layout.  The reference uploads 32-byte BVH nodes, 160-byte instances, 48-byte
// vertices and a u32 index list, and its traversal loads both children of an inner node as
// two separate 32-byte nodes and every triangle through three indexed 48-byte vertex loads
// (raytracing_sw.wgsl:218-225, 275-279).  The device layout keeps the same trees but packs
// what one traversal step touches into 16-byte-aligned records read with 128-bit loads:
//   GpuNode      64 B  both children's boxes + child references of one inner node
//   GpuRoot      32 B  a tree's root box + reference (the traversal tests the root box first)
//   GpuTri       48 B  v0, e1 = v1 - v0, e2 = v2 - v0 (the subtractions intersect_triangle
//                      performs), leaf length in v0.w of a leaf's first triangle
//   GpuInstTrace 64 B  the three rows of world_to_local used to transform rays, BLAS root id,
//                      TLAS leaf length in the first instance of each TLAS leaf
//   GpuInstShade 96 B  what intersect_scene/shading read from an instance
//   GpuVAttr     32 B  vertex normal + tangent (positions live in GpuTri)
// A child reference is either an inner-node index or kLeafBit | first primitive.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/nbounce.h"

namespace nb {

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kLdsStride = 17u;      // pathtracing.wgsl:4 (fixed, independent of bounces)
constexpr uint32_t kLdsPerBounce = 2u;    // pathtracing.wgsl:2
constexpr uint32_t kMaxSampleCount = 1024u;  // pathtracer.rs:56

struct alignas(16) GpuNode {
  float q0[4];    // c0.min.x, c0.max.x, c0.min.y, c0.max.y
  float q1[4];    // c1.min.x, c1.max.x, c1.min.y, c1.max.y
  float q2[4];    // c0.min.z, c0.max.z, c1.min.z, c1.max.z
  uint32_t ref[2];
  uint32_t pad[2];
};
struct alignas(16) GpuRoot {
  float mn[3];
  uint32_t ref;
  float mx[3];
  uint32_t pad;
};
struct alignas(16) GpuTri {
  float v0[3];
  uint32_t leaf_count;
  float e1[3];
  uint32_t pad1;
  float e2[3];
  uint32_t pad2;
};
struct alignas(16) GpuInstTrace {
  float row[3][4];     // row r = (W[0][r], W[1][r], W[2][r], W[3][r]) of world_to_local
  uint32_t blas_root;  // index into the BLAS root table
  uint32_t leaf_count; // TLAS leaf length if this instance starts a TLAS leaf
  uint32_t pad[2];
};
struct alignas(16) GpuInstShade {
  float w2l_col[3][4];  // column c .xyz of world_to_local, .w = color[c]
  float l2w_row[3][4];  // row r .xyz of mat3(local_to_world), .w = roughness / metallic / emissive
};
struct alignas(16) GpuVAttr {
  float n[3];
  float tw;
  float t[3];
  float pad;
};
static_assert(sizeof(GpuNode) == 64, "GpuNode");
static_assert(sizeof(GpuRoot) == 32, "GpuRoot");
static_assert(sizeof(GpuTri) == 48, "GpuTri");
static_assert(sizeof(GpuInstTrace) == 64, "GpuInstTrace");
static_assert(sizeof(GpuInstShade) == 96, "GpuInstShade");
static_assert(sizeof(GpuVAttr) == 32, "GpuVAttr");
static_assert(sizeof(nb_vertex) == 48 && sizeof(nb_bvh_node) == 32 && sizeof(nb_instance) == 160, "ref layout");

// Host copy of a scene: the reference-layout buffers and their device-layout translation.
struct HostScene {
  std::vector<nb_vertex> vertices;
  std::vector<uint32_t> indices;  // triangle-permuted (flatten_triangle_list)
  std::vector<nb_bvh_node> blas, tlas;
  std::vector<nb_instance> instances;  // TLAS-permuted

  std::vector<GpuNode> gblas, gtlas;
  GpuRoot tlas_root{};
  bool has_tlas = false;
  std::vector<GpuRoot> blas_roots;
  std::vector<GpuInstTrace> itrace;
  std::vector<GpuInstShade> ishade;
  std::vector<GpuTri> tris;
  std::vector<GpuVAttr> vattr;
  double build_ms = 0.0;
};

// error reporting (thread-local message, nb_api.cu)
int fail(int status, const char* fmt, ...);

// nb_scene.cpp
int build_bvh_triangles(const float* positions, size_t n_vertices, const uint32_t* indices, size_t n_indices,
                        std::vector<nb_bvh_node>* nodes, std::vector<uint32_t>* permuted);
int build_scene_reference(const nb_vertex* vertices, size_t nv, const uint32_t* indices, size_t ni,
                          const nb_primitive* prims, size_t np, uint32_t flags, HostScene* out);
int adopt_reference_buffers(const nb_bvh_node* blas, size_t n_blas, const nb_bvh_node* tlas, size_t n_tlas,
                            const nb_instance* inst, size_t n_inst, const nb_vertex* v, size_t nv,
                            const uint32_t* idx, size_t ni, HostScene* out);
int to_device_layout(HostScene* s);

// nb_sobol.cpp
void sobol_burley_table(uint32_t n_samples, uint32_t n_dimsets, uint32_t seed, float* out);

}  // namespace nb

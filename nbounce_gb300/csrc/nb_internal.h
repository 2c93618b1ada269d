// Internal declarations shared by the host builder (nb_scene.cpp), the Sobol generator
// (nb_sobol.cpp) and the CUDA side (nb_api.cu / nb_kernels.cu).
//
// Device layout.  The reference uploads 32-byte BVH nodes, 160-byte instances, 48-byte
// vertices and a u32 index list, and its traversal loads both children of an inner node as
// two separate 32-byte nodes and every triangle through three indexed 48-byte vertex loads
// (raytracing_sw.wgsl:218-225, 275-279).  The device layout keeps the same trees but packs
// what one traversal step touches into 16-byte-aligned records read with 128-bit loads:
//   WideNode     80 B  8 children of a collapsed node: 8-bit quantised boxes, slot metadata
//   GpuTri       48 B  v0, e1 = v1 - v0, e2 = v2 - v0 (the subtractions intersect_triangle
//                      performs) + the reference triangle index
//   GpuInstTrace 64 B  the three rows of world_to_local used to transform rays, BLAS root,
//                      reference instance index
//   GpuInstShade 96 B  what intersect_scene/shading read from an instance
//   GpuVAttr     32 B  vertex normal + tangent (positions live in GpuTri)
// Triangles and instances are stored in the order of the wide trees' leaves.
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

struct alignas(16) GpuTri {
  float v0[3];
  uint32_t pad0;
  float e1[3];
  uint32_t ref_index;  // index in the reference's permuted triangle list (reported by hits)
  float e2[3];
  uint32_t pad2;
};
struct alignas(16) GpuInstTrace {
  float row[3][4];     // row r = (W[0][r], W[1][r], W[2][r], W[3][r]) of world_to_local
  uint32_t blas_root;  // root of the instance's BLAS in the wide BLAS node array
  uint32_t ref_index;  // TLAS-permuted instance index of the reference (reported by hits)
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
// 8-wide node collapsed from the reference's binary tree (80 B = 5 x 16 B).  Child boxes are
// quantised to 8 bits per plane on a per-axis power-of-two grid anchored at p; the quantised
// boxes contain the exact ones.  meta[k]: 0 = empty slot; 0x80 | r = inner child at
// child_base + r; (n << 5) | o = leaf of n (1..3) primitives at prim_base + o.
struct alignas(16) WideNode {
  float p[3];
  uint8_t e[3];        // biased exponent of the grid step per axis (float bits e << 23)
  uint8_t n_children;
  uint32_t child_base;
  uint32_t prim_base;
  uint8_t meta[8];
  uint8_t qlo_x[8], qlo_y[8], qlo_z[8], qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(WideNode) == 80, "WideNode");
constexpr uint32_t kInstanceBit = 0x80000000u;  // TLAS stack entry that names an instance

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

  std::vector<WideNode> wblas, wtlas;  // 8-wide trees; the TLAS root is wtlas[0]
  std::vector<uint32_t> wblas_root;    // per distinct BLAS root: index of its root in wblas
  size_t wblas_nodes = 0, wtlas_nodes = 0;  // sizes kept after the host copies are dropped
  size_t tlas_entries = 0;                  // device TLAS leaves (itrace records)
  bool has_tlas = false;
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

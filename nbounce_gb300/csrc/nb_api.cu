// C ABI of the GB300-native nBounce pass (declared in include/nbounce.h).
//
// Mirrors the reference host driver: SceneBuffers::from_scene (src/pathtracing/scene.rs:280-453)
// becomes nb_scene_create, Pathtracer::{new, dispatch, invalidate, resize, output_texture,
// sample_count} (src/pathtracing/pathtracer.rs:51-239) become nb_pathtracer_*.  The library
// owns every device allocation; failures return a status and set a thread-local message.

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include <cuda_fp16.h>

#include "nb_internal.h"
#include "nb_mlp.cuh"
#include "nb_launch.h"
#include "nb_runtime.h"

namespace nb {

static thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

}  // namespace nb

using namespace nb;

struct nb_pathtracer {
  uint32_t width = 0, height = 0;
  nb_globals globals{0, 0.0f, 8, 4.0f};
  uint32_t max_sample_count = kMaxSampleCount;
  DeviceArena image;  // output image
  DeviceArena tables; // Sobol table + counters
  DeviceArena work;   // path queues (sized on demand)
  float* d_out = nullptr;
  float4* d_sobol = nullptr;
  uint32_t sobol_entries = 0;
  uint32_t* d_counts = nullptr;
  uint32_t* d_fetch = nullptr;
  uint32_t* d_status = nullptr;
  unsigned long long* d_rays = nullptr;
  PathBatch pb{};
  std::unique_ptr<WaveTables> wt{new WaveTables()};  // kernel parameter tables (host copy)
  uint32_t capacity = 0;  // paths the work buffers hold
  uint32_t batch_paths = 1u << 27;
  nb_cache* cache = nullptr;  // radiance-cache mode when set
  uint32_t sampling = 0;      // NB_SAMPLE_* flags
  uint32_t rr_start = 0;      // Russian roulette start bounce (0: the reference schedule)
  DeviceArena shadow;         // shadow-ray queue of environment next-event estimation
  uint32_t shadow_capacity = 0;
  ShadowQueue sq{};
  int sms = 1;
  // optional traversal work counters (instrumented trace kernel), 8 per bounce slot
  DeviceArena counter_mem;
  unsigned long long* d_trace_counts = nullptr;
  // optional per-kernel event timing: (kind, start, stop) of every recorded launch
  bool timing = false;
  std::vector<cudaEvent_t> event_pool;
  std::vector<std::tuple<int, cudaEvent_t, cudaEvent_t>> timed;
};

enum { kKindRaygen = 0, kKindTrace = 1, kKindShade = 2, kKindAccumulate = 3, kKindCacheInfer = 4, kKindCacheTrain = 5 };

// Launches `launch` on st, bracketed by two events when timing is on.
template <class F>
static cudaError_t timed_launch(nb_pathtracer* pt, int kind, cudaStream_t st, F&& launch) {
  if (!pt->timing) return launch();
  cudaEvent_t ev[2];
  for (int k = 0; k < 2; ++k) {
    if (!pt->event_pool.empty()) {
      ev[k] = pt->event_pool.back();
      pt->event_pool.pop_back();
    } else {
      cudaError_t e = cudaEventCreate(&ev[k]);
      if (e != cudaSuccess) return e;
    }
  }
  cudaEventRecord(ev[0], st);
  cudaError_t e = launch();
  cudaEventRecord(ev[1], st);
  pt->timed.emplace_back(kind, ev[0], ev[1]);
  return e;
}

static int upload_scene(nb_scene* s) {
  HostScene& h = s->host;
  int st = to_device_layout(&h);
  if (st) return st;
  nbd::DevScene& d = s->dev;
  const WideNode *wb = nullptr, *wt = nullptr;
  const GpuInstTrace* it = nullptr;
  const GpuInstShade* is = nullptr;
  const GpuTri* tr = nullptr;
  const GpuVAttr* va = nullptr;
  const uint32_t* ti = nullptr;
  if ((st = s->arena.upload(h.wblas, &wb)) || (st = s->arena.upload(h.wtlas, &wt)) ||
      (st = s->arena.upload(h.itrace, &it)) || (st = s->arena.upload(h.ishade, &is)) ||
      (st = s->arena.upload(h.tris, &tr)) || (st = s->arena.upload(h.vattr, &va)) ||
      (st = s->arena.upload(h.indices, &ti)))
    return st;
  d.blas_wide = (const float4*)wb;
  d.tlas_wide = (const float4*)wt;
  d.inst_trace = (const float4*)it;
  d.inst_shade = (const float4*)is;
  d.tris = (const float4*)tr;
  d.vattr = (const float4*)va;
  d.tri_idx = ti;
  d.has_tlas = h.has_tlas ? 1u : 0u;
  d.n_tris = (uint32_t)h.tris.size();
  d.n_inst = (uint32_t)h.itrace.size();
  d.n_vertices = (uint32_t)h.vertices.size();
  void* p = nullptr;
  if ((st = s->arena.alloc(2 * sizeof(uint32_t), &p))) return st;
  s->d_fetch = (uint32_t*)p;
  s->d_status = s->d_fetch + 1;
  NB_CUDA(cudaMemset(p, 0, 2 * sizeof(uint32_t)), "cudaMemset");
  // drop device-layout host copies; keep the reference-layout buffers for nb_scene_export
  h.wblas_nodes = h.wblas.size();
  h.wtlas_nodes = h.wtlas.size();
  std::vector<WideNode>().swap(h.wblas);
  std::vector<WideNode>().swap(h.wtlas);
  std::vector<GpuTri>().swap(h.tris);
  std::vector<GpuVAttr>().swap(h.vattr);
  s->sms = sm_count();
  return NB_OK;
}

static int check_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(NB_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  return NB_OK;
}

extern "C" {

int nb_version(void) { return NB_VERSION; }
const char* nb_last_error(void) { return g_last_error.c_str(); }
const char* nb_status_string(int status) {
  switch (status) {
    case NB_OK: return "NB_OK";
    case NB_ERR_INVALID_ARG: return "NB_ERR_INVALID_ARG";
    case NB_ERR_OOM: return "NB_ERR_OOM";
    case NB_ERR_CUDA: return "NB_ERR_CUDA";
    case NB_ERR_TIMEOUT: return "NB_ERR_TIMEOUT";
    case NB_ERR_STACK_OVERFLOW: return "NB_ERR_STACK_OVERFLOW";
    case NB_ERR_NO_DEVICE: return "NB_ERR_NO_DEVICE";
    case NB_ERR_EXHAUSTED: return "NB_ERR_EXHAUSTED";
    case NB_ERR_BUSY: return "NB_ERR_BUSY";
    case NB_ERR_CANCELLED: return "NB_ERR_CANCELLED";
    case NB_ERR_EXPIRED: return "NB_ERR_EXPIRED";
    default: return "unknown status";
  }
}

int nb_sobol_burley_table(uint32_t n_samples, uint32_t n_dimsets, uint32_t seed, float* out) {
  if (!out && n_samples && n_dimsets) return fail(NB_ERR_INVALID_ARG, "out is NULL");
  if (n_dimsets > 17) return fail(NB_ERR_INVALID_ARG, "at most 17 dimension sets (68 Sobol dimensions)");
  sobol_burley_table(n_samples, n_dimsets, seed, out);
  return NB_OK;
}

int nb_bvh_build(const float* positions, size_t n_vertices, const uint32_t* indices, size_t n_indices,
                 nb_bvh_node* nodes_out, size_t nodes_capacity, size_t* n_nodes_out, uint32_t* indices_out) {
  if ((!positions && n_vertices) || (!indices && n_indices) || !n_nodes_out || (!indices_out && n_indices))
    return fail(NB_ERR_INVALID_ARG, "NULL argument");
  std::vector<nb_bvh_node> nodes;
  std::vector<uint32_t> perm;
  try {
    int st = build_bvh_triangles(positions, n_vertices, indices, n_indices, &nodes, &perm);
    if (st) return st;
  } catch (const std::bad_alloc&) {
    return fail(NB_ERR_OOM, "host allocation failed");
  }
  *n_nodes_out = nodes.size();
  if (nodes.size() > nodes_capacity || (!nodes_out && !nodes.empty()))
    return fail(NB_ERR_INVALID_ARG, "nodes_capacity %zu < %zu nodes", nodes_capacity, nodes.size());
  if (!nodes.empty()) std::memcpy(nodes_out, nodes.data(), nodes.size() * sizeof(nb_bvh_node));
  if (n_indices) std::memcpy(indices_out, perm.data(), n_indices * sizeof(uint32_t));
  return NB_OK;
}

// ---- scenes ----------------------------------------------------------------------------
int nb_scene_create(const nb_vertex* vertices, size_t n_vertices, const uint32_t* indices, size_t n_indices,
                    const nb_primitive* primitives, size_t n_primitives, uint32_t flags, nb_scene** out) {
  if (!out) return fail(NB_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if ((!vertices && n_vertices) || (!indices && n_indices) || (!primitives && n_primitives))
    return fail(NB_ERR_INVALID_ARG, "NULL array with nonzero size");
  const bool host_only = (flags & NB_SCENE_HOST_ONLY) != 0;
  int st = host_only ? NB_OK : check_device();
  if (st) return st;
  nb_scene* s = new (std::nothrow) nb_scene();
  if (!s) return fail(NB_ERR_OOM, "host allocation failed");
  try {
    st = build_scene_reference(vertices, n_vertices, indices, n_indices, primitives, n_primitives, flags, &s->host);
    if (!st) st = host_only ? to_device_layout(&s->host) : upload_scene(s);
    s->uploaded = !st && !host_only;
  } catch (const std::bad_alloc&) {
    st = fail(NB_ERR_OOM, "host allocation failed");
  }
  if (st) {
    s->arena.release();
    delete s;
    return st;
  }
  *out = s;
  return NB_OK;
}

int nb_scene_create_from_bvh(const nb_bvh_node* blas, size_t n_blas, const nb_bvh_node* tlas, size_t n_tlas,
                             const nb_instance* instances, size_t n_instances, const nb_vertex* vertices,
                             size_t n_vertices, const uint32_t* indices, size_t n_indices, nb_scene** out) {
  if (!out) return fail(NB_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if ((!blas && n_blas) || (!tlas && n_tlas) || (!instances && n_instances) || (!vertices && n_vertices) ||
      (!indices && n_indices))
    return fail(NB_ERR_INVALID_ARG, "NULL array with nonzero size");
  int st = check_device();
  if (st) return st;
  nb_scene* s = new (std::nothrow) nb_scene();
  if (!s) return fail(NB_ERR_OOM, "host allocation failed");
  try {
    st = adopt_reference_buffers(blas, n_blas, tlas, n_tlas, instances, n_instances, vertices, n_vertices, indices,
                                 n_indices, &s->host);
    if (!st) st = upload_scene(s);
    s->uploaded = !st;
  } catch (const std::bad_alloc&) {
    st = fail(NB_ERR_OOM, "host allocation failed");
  }
  if (st) {
    s->arena.release();
    delete s;
    return st;
  }
  *out = s;
  return NB_OK;
}

int nb_scene_export(const nb_scene* s, nb_bvh_node* blas, nb_bvh_node* tlas, nb_instance* instances,
                    uint32_t* indices) {
  if (!s) return fail(NB_ERR_INVALID_ARG, "scene is NULL");
  const HostScene& h = s->host;
  if (blas && !h.blas.empty()) std::memcpy(blas, h.blas.data(), h.blas.size() * sizeof(nb_bvh_node));
  if (tlas && !h.tlas.empty()) std::memcpy(tlas, h.tlas.data(), h.tlas.size() * sizeof(nb_bvh_node));
  if (instances && !h.instances.empty())
    std::memcpy(instances, h.instances.data(), h.instances.size() * sizeof(nb_instance));
  if (indices && !h.indices.empty()) std::memcpy(indices, h.indices.data(), h.indices.size() * sizeof(uint32_t));
  return NB_OK;
}

int nb_scene_get_info(const nb_scene* s, nb_scene_info* info) {
  if (!s || !info) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  const HostScene& h = s->host;
  info->n_vertices = h.vertices.size();
  info->n_triangles = h.indices.size() / 3;
  info->n_instances = h.instances.size();
  info->n_blas_roots = h.wblas_root.size();
  info->n_blas_nodes_ref = h.blas.size();
  info->n_tlas_nodes_ref = h.tlas.size();
  info->n_blas_nodes_gpu = s->uploaded ? h.wblas_nodes : h.wblas.size();
  info->n_tlas_nodes_gpu = s->uploaded ? h.wtlas_nodes : h.wtlas.size();
  info->n_tlas_entries = h.tlas_entries;
  info->device_bytes = s->arena.bytes;
  info->build_ms = h.build_ms;
  return NB_OK;
}

void nb_scene_destroy(nb_scene* s) {
  if (!s) return;
  s->arena.release();
  delete s;
}

// ---- environment -----------------------------------------------------------------------
// Importance-sampling tables of an equirect or cube map over its texel table (a cube's six
// faces stacked, 6 N rows of N texels): texel weight w = luminance x the texel's solid angle
// at its centre - sin(theta) of the row for an equirect map, 1 / (1 + s^2 + t^2)^(3/2) for a
// cube face - with negative or non-finite luminance counted as 0 and a uniform luminance if
// the whole map is black.  Sums in double, tables in float: marginal CDF over rows, a CDF per
// row, and per texel the density over the table's (u, v) = w / sum(w) x width x height.
static int build_env_distribution(nb_env* e, const float* texels, uint32_t W, uint32_t H, bool cube) {
  std::vector<double> w((size_t)W * H), row_sum(H, 0.0);
  double total = 0.0;
  for (int pass = 0; pass < 2 && !(total > 0.0); ++pass) {
    total = 0.0;
    for (uint32_t y = 0; y < H; ++y) {
      const double sin_t = std::sin(3.14159265358979323846 * ((double)y + 0.5) / (double)H);
      const double tc = 2.0 * ((double)(y % W) + 0.5) / (double)W - 1.0;  // cube: t of the row
      double r = 0.0;
      for (uint32_t x = 0; x < W; ++x) {
        const float* t = texels + ((size_t)y * W + x) * 4;
        double lum = pass == 0 ? 0.2126 * t[0] + 0.7152 * t[1] + 0.0722 * t[2] : 1.0;
        if (!(lum > 0.0) || !std::isfinite(lum)) lum = 0.0;
        double omega = sin_t;
        if (cube) {
          const double sc = 2.0 * ((double)x + 0.5) / (double)W - 1.0, j = 1.0 + sc * sc + tc * tc;
          omega = 1.0 / (j * std::sqrt(j));
        }
        w[(size_t)y * W + x] = lum * omega;
        r += lum * omega;
      }
      row_sum[y] = r;
      total += r;
    }
  }
  std::vector<float> cdf_rows(H + 1), cdf_cols((size_t)H * (W + 1)), pdf_uv((size_t)W * H);
  double acc = 0.0;
  cdf_rows[0] = 0.0f;
  for (uint32_t y = 0; y < H; ++y) {
    acc += row_sum[y];
    cdf_rows[y + 1] = (float)(acc / total);
    float* c = cdf_cols.data() + (size_t)y * (W + 1);
    double a = 0.0;
    c[0] = 0.0f;
    for (uint32_t x = 0; x < W; ++x) {
      a += w[(size_t)y * W + x];
      c[x + 1] = row_sum[y] > 0.0 ? (float)(a / row_sum[y]) : (float)(x + 1) / (float)W;
      pdf_uv[(size_t)y * W + x] = (float)(w[(size_t)y * W + x] / total * (double)W * (double)H);
    }
    c[W] = 1.0f;
  }
  cdf_rows[H] = 1.0f;
  const float *cr = nullptr, *cc = nullptr, *pu = nullptr;
  int st;
  if ((st = e->arena.upload(cdf_rows, &cr)) || (st = e->arena.upload(cdf_cols, &cc)) ||
      (st = e->arena.upload(pdf_uv, &pu)))
    return st;
  e->dev.cdf_rows = cr;
  e->dev.cdf_cols = cc;
  e->dev.pdf_uv = pu;
  return NB_OK;
}

int nb_env_create(const nb_env_desc* desc, nb_env** out) {
  if (!desc || !out) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  *out = nullptr;
  if (desc->kind != NB_ENV_CONSTANT && desc->kind != NB_ENV_EQUIRECT && desc->kind != NB_ENV_CUBE)
    return fail(NB_ERR_INVALID_ARG, "unknown environment kind %u", desc->kind);
  if (desc->kind == NB_ENV_CUBE && desc->width != desc->height)
    return fail(NB_ERR_INVALID_ARG, "cube faces must be square (%u x %u)", desc->width, desc->height);
  if (desc->kind != NB_ENV_CONSTANT && (desc->width > 32768 || desc->height > 32768))
    return fail(NB_ERR_INVALID_ARG, "environment of %u x %u texels (32768 at most per side)", desc->width,
                desc->height);
  int st = check_device();
  if (st) return st;
  nb_env* e = new (std::nothrow) nb_env();
  if (!e) return fail(NB_ERR_OOM, "host allocation failed");
  e->dev.kind = desc->kind;
  e->dev.r = desc->color[0];
  e->dev.g = desc->color[1];
  e->dev.b = desc->color[2];
  if (desc->kind == NB_ENV_EQUIRECT || desc->kind == NB_ENV_CUBE) {
    if (!desc->texels || desc->width == 0 || desc->height == 0) {
      delete e;
      return fail(NB_ERR_INVALID_ARG, "texel environment needs texels and a size");
    }
    const uint32_t rows = desc->kind == NB_ENV_CUBE ? 6 * desc->height : desc->height;
    size_t n = (size_t)desc->width * rows * 4 * sizeof(float);
    void* p = nullptr;
    if ((st = e->arena.alloc(n, &p))) { delete e; return st; }
    cudaError_t ce = cudaMemcpy(p, desc->texels, n, cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) { e->arena.release(); delete e; return cuda_fail(ce, "cudaMemcpy(env)"); }
    e->dev.texels = (const float4*)p;
    e->dev.width = desc->width;
    e->dev.height = rows;
    if ((st = build_env_distribution(e, desc->texels, desc->width, rows, desc->kind == NB_ENV_CUBE))) {
      e->arena.release();
      delete e;
      return st;
    }
  }
  *out = e;
  return NB_OK;
}

int nb_env_create_dds(const void* bytes, size_t n, nb_env** out) {
  if (!bytes || !out) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  *out = nullptr;
  DdsCube dds;
  int st = parse_dds_cube((const uint8_t*)bytes, n, &dds);
  if (st) return st;
  if ((st = check_device())) return st;
  const uint32_t N = dds.size;
  const size_t n_texels = (size_t)6 * N * N;
  std::vector<float> host(n_texels * 4);
  nb_env* e = new (std::nothrow) nb_env();
  if (!e) return fail(NB_ERR_OOM, "host allocation failed");
  auto bail = [&](int status) {
    e->arena.release();
    delete e;
    return status;
  };
  void* texels = nullptr;
  if ((st = e->arena.alloc(n_texels * sizeof(float4), &texels))) return bail(st);
  if (dds.format == kDdsBc6hUf16 || dds.format == kDdsBc6hSf16) {
    DeviceArena blocks;
    void* d_blocks = nullptr;
    if ((st = blocks.alloc(6 * dds.face_bytes, &d_blocks))) return bail(st);
    cudaError_t ce = cudaSuccess;
    for (int f = 0; f < 6 && ce == cudaSuccess; ++f)
      ce = cudaMemcpy((uint8_t*)d_blocks + f * dds.face_bytes, dds.face[f], dds.face_bytes, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) {
      st = decode_bc6h_device(d_blocks, N, N, 6, dds.format == kDdsBc6hSf16, (float4*)texels, 0);
      if (!st) ce = cudaMemcpy(host.data(), texels, n_texels * sizeof(float4), cudaMemcpyDeviceToHost);
    }
    blocks.release();
    if (st) return bail(st);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaMemcpy(env blocks)"));
  } else {
    const size_t face_texels = (size_t)N * N;
    for (int f = 0; f < 6; ++f) {
      float* dst = host.data() + f * face_texels * 4;
      if (dds.format == kDdsRgba32f) {
        std::memcpy(dst, dds.face[f], face_texels * 16);
      } else {
        for (size_t i = 0; i < face_texels * 4; ++i) {
          __half_raw raw;
          std::memcpy(&raw.x, dds.face[f] + 2 * i, 2);
          dst[i] = __half2float(__half(raw));
        }
      }
    }
    cudaError_t ce = cudaMemcpy(texels, host.data(), n_texels * sizeof(float4), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "cudaMemcpy(env)"));
  }
  e->dev.kind = NB_ENV_CUBE;
  e->dev.texels = (const float4*)texels;
  e->dev.width = N;
  e->dev.height = 6 * N;
  if ((st = build_env_distribution(e, host.data(), N, 6 * N, true))) return bail(st);
  *out = e;
  return NB_OK;
}

int nb_bc6h_decode(const void* blocks, uint32_t width, uint32_t height, uint32_t layers, uint32_t is_signed,
                   float* out) {
  if (is_signed > 1) return fail(NB_ERR_INVALID_ARG, "is_signed must be 0 or 1");
  if (width == 0 || height == 0 || layers == 0) return NB_OK;
  if (!blocks || !out) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (width > 65536 || height > 65536 || layers > 65536)
    return fail(NB_ERR_INVALID_ARG, "BC6H size %u x %u x %u layers", width, height, layers);
  int st = check_device();
  if (st) return st;
  const size_t in_bytes = (size_t)((width + 3) / 4) * ((height + 3) / 4) * layers * 16;
  const size_t out_bytes = (size_t)width * height * layers * sizeof(float4);
  DeviceArena tmp;
  void *d_in = nullptr, *d_out = nullptr;
  if ((st = tmp.alloc(in_bytes, &d_in)) || (st = tmp.alloc(out_bytes, &d_out))) {
    tmp.release();
    return st;
  }
  cudaError_t ce = cudaMemcpy(d_in, blocks, in_bytes, cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) {
    st = decode_bc6h_device(d_in, width, height, layers, is_signed != 0, (float4*)d_out, 0);
    if (!st) ce = cudaMemcpy(out, d_out, out_bytes, cudaMemcpyDeviceToHost);
  }
  tmp.release();
  if (st) return st;
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpy(bc6h)");
  return NB_OK;
}

void nb_env_destroy(nb_env* e) {
  if (!e) return;
  e->arena.release();
  delete e;
}

// ---- pathtracer --------------------------------------------------------------------------
static int alloc_image(nb_pathtracer* pt, uint32_t w, uint32_t h) {
  pt->image.release();
  pt->d_out = nullptr;
  pt->width = w;
  pt->height = h;
  if (w == 0 || h == 0) return NB_OK;
  void* p = nullptr;
  int st = pt->image.alloc((size_t)w * h * 4 * sizeof(float), &p);
  if (st) return st;
  NB_CUDA(cudaMemset(p, 0, (size_t)w * h * 4 * sizeof(float)), "cudaMemset(image)");
  pt->d_out = (float*)p;
  return NB_OK;
}

int nb_pathtracer_create(uint32_t width, uint32_t height, const nb_globals* globals, const float* sobol_table,
                         uint32_t sobol_rows, nb_pathtracer** out) {
  if (!out) return fail(NB_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if ((uint64_t)width * height > 0x7FFFFFFFull) return fail(NB_ERR_INVALID_ARG, "image too large");
  if (globals && globals->bounces + 2 > kMaxBounceSlots)
    return fail(NB_ERR_INVALID_ARG, "bounces must be <= %u", kMaxBounceSlots - 2);
  int st = check_device();
  if (st) return st;
  nb_pathtracer* pt = new (std::nothrow) nb_pathtracer();
  if (!pt) return fail(NB_ERR_OOM, "host allocation failed");
  if (globals) pt->globals = *globals;
  std::vector<float> table;
  const float* src = sobol_table;
  uint32_t rows = sobol_rows;
  if (!src) {
    rows = kMaxSampleCount;
    table.resize((size_t)rows * kLdsStride * 4);
    sobol_burley_table(rows, kLdsStride, 0, table.data());
    src = table.data();
  } else if (rows == 0) {
    delete pt;
    return fail(NB_ERR_INVALID_ARG, "sobol_rows must be > 0 with a caller table");
  }
  pt->max_sample_count = rows;
  pt->sobol_entries = rows * kLdsStride;
  void* p = nullptr;
  if (!(st = pt->tables.alloc((size_t)pt->sobol_entries * 16, &p))) {
    pt->d_sobol = (float4*)p;
    cudaError_t ce = cudaMemcpy(p, src, (size_t)pt->sobol_entries * 16, cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) st = cuda_fail(ce, "cudaMemcpy(sobol)");
  }
  if (!st && !(st = pt->tables.alloc(2 * kMaxBounceSlots * sizeof(uint32_t) + 16 + sizeof(unsigned long long), &p))) {
    pt->d_counts = (uint32_t*)p;
    pt->d_fetch = pt->d_counts + kMaxBounceSlots;
    pt->d_status = pt->d_fetch + kMaxBounceSlots;
    pt->d_rays = (unsigned long long*)((char*)p + 2 * kMaxBounceSlots * sizeof(uint32_t) + 16);
    cudaError_t ce = cudaMemset(p, 0, 2 * kMaxBounceSlots * sizeof(uint32_t) + 16 + sizeof(unsigned long long));
    if (ce != cudaSuccess) st = cuda_fail(ce, "cudaMemset");
  }
  if (!st) st = alloc_image(pt, width, height);
  if (st) {
    pt->image.release();
    pt->tables.release();
    delete pt;
    return st;
  }
  pt->sms = sm_count();
  *out = pt;
  return NB_OK;
}

void nb_pathtracer_destroy(nb_pathtracer* pt) {
  if (!pt) return;
  for (auto& t : pt->timed) {
    cudaEventDestroy(std::get<1>(t));
    cudaEventDestroy(std::get<2>(t));
  }
  for (cudaEvent_t e : pt->event_pool) cudaEventDestroy(e);
  pt->work.release();
  pt->tables.release();
  pt->image.release();
  pt->shadow.release();
  pt->counter_mem.release();
  delete pt;
}

static int ensure_capacity(nb_pathtracer* pt, uint32_t paths) {
  if (pt->capacity >= paths) return NB_OK;
  pt->work.release();
  pt->capacity = 0;
  size_t n = paths;
  void* p = nullptr;
  int st;
  float4* f4[8];
  for (int k = 0; k < 8; ++k) {
    if ((st = pt->work.alloc(n * sizeof(float4), &p))) { pt->work.release(); return st; }
    f4[k] = (float4*)p;
  }
  if ((st = pt->work.alloc(n * sizeof(uint32_t), &p))) { pt->work.release(); return st; }
  PathBatch& b = pt->pb;
  b.q_o[0] = f4[0]; b.q_o[1] = f4[1];
  b.q_d[0] = f4[2]; b.q_d[1] = f4[3];
  b.q_t[0] = f4[4]; b.q_t[1] = f4[5];
  b.hits = f4[6];
  b.radiance = f4[7];
  b.hit_inst = (uint32_t*)p;
  pt->capacity = paths;
  return NB_OK;
}

// shadow-ray queue for `paths` paths (one ray per path and bounce at most) + its counters
static int ensure_shadow(nb_pathtracer* pt, uint32_t paths) {
  if (pt->shadow_capacity >= paths) return NB_OK;
  pt->shadow.release();
  pt->shadow_capacity = 0;
  void* p[4] = {nullptr, nullptr, nullptr, nullptr};
  int st = NB_OK;
  for (int k = 0; k < 3 && !st; ++k) st = pt->shadow.alloc((size_t)paths * sizeof(float4), &p[k]);
  if (!st) st = pt->shadow.alloc(2 * kMaxBounceSlots * sizeof(uint32_t), &p[3]);
  if (st) {
    pt->shadow.release();
    return st;
  }
  pt->sq.o = (float4*)p[0];
  pt->sq.d = (float4*)p[1];
  pt->sq.c = (float4*)p[2];
  pt->sq.counts = (uint32_t*)p[3];
  pt->sq.fetch = pt->sq.counts + kMaxBounceSlots;
  pt->shadow_capacity = paths;
  return NB_OK;
}

// samples per batch: enough paths in flight to fill the GPU, bounded memory
static uint32_t batch_samples(const nb_pathtracer* pt, uint32_t remaining) {
  const uint64_t npix = (uint64_t)pt->width * pt->height;
  uint64_t s = std::max<uint64_t>(1, pt->batch_paths / std::max<uint64_t>(1, npix));
  return (uint32_t)std::min<uint64_t>(s, remaining);
}

static int render_samples(nb_pathtracer* pt, const nb_scene* scene, const nb_camera* camera, const nb_env* env,
                          uint32_t n_samples, void* stream) {
  if (!pt || !scene || !camera || !env) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (!scene->uploaded) return fail(NB_ERR_INVALID_ARG, "scene was built with NB_SCENE_HOST_ONLY");
  if (pt->globals.bounces + 2 > kMaxBounceSlots) return fail(NB_ERR_INVALID_ARG, "bounces too large");
  cudaStream_t st = (cudaStream_t)stream;
  NB_CUDA(cudaMemsetAsync(pt->d_status, 0, sizeof(uint32_t), st), "cudaMemsetAsync");
  NB_CUDA(cudaMemsetAsync(pt->d_rays, 0, sizeof(unsigned long long), st), "cudaMemsetAsync");
  if (pt->globals.sample >= pt->max_sample_count) return fail(NB_ERR_EXHAUSTED, "sample count exhausted");
  const uint32_t npix = pt->width * pt->height;
  if (npix == 0 || n_samples == 0) return NB_OK;
  uint32_t remaining = std::min(n_samples, pt->max_sample_count - pt->globals.sample);
  // one job, one segment per batch
  WaveTables& wt = *pt->wt;
  wt.n_jobs = 1;
  wt.n_scenes = 1;
  wt.n_segs = 1;
  wt.scenes[0] = scene->dev;
  JobParams& jp = wt.jobs[0];
  std::memcpy(jp.c2w, camera->clip_to_world, sizeof(jp.c2w));
  jp.env = env->dev;
  jp.out = (float4*)pt->d_out;
  jp.scene = 0;
  jp.width = pt->width;
  jp.height = pt->height;
  jp.npix = npix;
  jp.bounces = pt->globals.bounces;
  jp.cf = pt->globals.contribution_factor;
  jp.rr_start = pt->rr_start;
  while (remaining > 0) {
    uint32_t S = batch_samples(pt, remaining);
    int rc = ensure_capacity(pt, npix * S);
    if (rc) return rc;
    PathBatch pb = pt->pb;
    pb.counts = pt->d_counts;
    pb.fetch = pt->d_fetch;
    pb.status = pt->d_status;
    pb.sobol = pt->d_sobol;
    pb.sobol_entries = pt->sobol_entries;
    // dispatch increments the sample counter before use (pathtracer.rs:234)
    wt.segs[0] = Segment{0u, pt->globals.sample + 1, S, 0u, 0u};
    wt.n_paths = npix * S;
    wt.n_pix = npix;
    const uint32_t B = pt->globals.bounces;
    const bool nee = (pt->sampling & NB_SAMPLE_ENV_NEE) != 0 && !pt->cache;
    jp.flags = nee ? kJobEnvNee : 0u;
    wt.flags = (nee || pt->cache) ? kWaveZeroRadiance : 0u;  // their shading adds to radiance
    if (nee) {
      if ((rc = ensure_shadow(pt, npix * S))) return rc;
      NB_CUDA(cudaMemsetAsync(pt->sq.counts, 0, 2 * kMaxBounceSlots * sizeof(uint32_t), st), "cudaMemsetAsync");
    }
    CacheWave cw{};
    if (pt->cache) {
      rc = cache_wave_begin(pt->cache, scene, wt.n_paths, &cw, st);
      if (rc) return rc;
    }
    cudaError_t e = timed_launch(pt, kKindRaygen, st, [&] { return launch_raygen(pb, wt, pt->sms, st); });
    for (uint32_t b = 0; b <= B && e == cudaSuccess; ++b) {
      e = timed_launch(pt, kKindTrace, st, [&] {
        return launch_trace_wave(pb, wt, true, b, pt->d_rays, pt->sms, st, pt->d_trace_counts);
      });
      if (e == cudaSuccess)
        e = timed_launch(pt, kKindShade, st, [&] {
          if (pt->cache) return launch_shade_cache(pb, wt, cw, b, pt->sms, st);
          if (nee) return launch_shade_nee(pb, wt, pt->sq, b, pt->sms, st);
          return launch_shade(pb, wt, b, pt->sms, st);
        });
      if (e == cudaSuccess && nee)
        e = timed_launch(pt, kKindTrace, st, [&] { return launch_trace_shadow(pb, wt, pt->sq, b, pt->sms, st); });
    }
    if (e == cudaSuccess && pt->cache) {
      rc = NB_OK;
      e = timed_launch(pt, kKindCacheInfer, st, [&] {
        rc = cache_wave_infer(pt->cache, pb, pt->sms, st);
        return cudaSuccess;
      });
      if (rc) return rc;
      if (e == cudaSuccess)
        e = timed_launch(pt, kKindCacheTrain, st, [&] {
          rc = cache_wave_train(pt->cache, wt.n_paths, pt->sms, st);
          return cudaSuccess;
        });
      if (rc) return rc;
    }
    if (e == cudaSuccess) e = timed_launch(pt, kKindAccumulate, st, [&] { return launch_accumulate(pb, wt, pt->sms, st); });
    if (e != cudaSuccess) return cuda_fail(e, "path batch launch");
    pt->globals.sample += S;
    pt->globals.weight = 1.0f / (float)pt->globals.sample;
    remaining -= S;
  }
  return NB_OK;
}

int nb_pathtracer_dispatch(nb_pathtracer* pt, const nb_scene* scene, const nb_camera* camera, const nb_env* env,
                           void* stream) {
  return render_samples(pt, scene, camera, env, 1, stream);
}

int nb_pathtracer_render(nb_pathtracer* pt, const nb_scene* scene, const nb_camera* camera, const nb_env* env,
                         uint32_t n_samples, void* stream) {
  return render_samples(pt, scene, camera, env, n_samples, stream);
}

int nb_pathtracer_set_batch_paths(nb_pathtracer* pt, uint32_t paths) {
  if (!pt || paths == 0 || paths > 0x7FFFFFFFu) return fail(NB_ERR_INVALID_ARG, "invalid batch size");
  pt->batch_paths = paths;
  return NB_OK;
}

int nb_pathtracer_enable_timing(nb_pathtracer* pt, int enable) {
  if (!pt) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  pt->timing = enable != 0;
  return NB_OK;
}

int nb_pathtracer_kernel_times(nb_pathtracer* pt, nb_kernel_times* out, int reset, void* stream) {
  if (!pt || !out) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  NB_CUDA(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize");
  std::memset(out, 0, sizeof(*out));
  double* ms[6] = {&out->raygen_ms, &out->trace_ms, &out->shade_ms, &out->accumulate_ms, &out->cache_infer_ms,
                   &out->cache_train_ms};
  uint64_t* cnt[6] = {&out->raygen_launches, &out->trace_launches, &out->shade_launches, &out->accumulate_launches,
                      &out->cache_infer_launches, &out->cache_train_launches};
  for (auto& t : pt->timed) {
    float m = 0.0f;
    NB_CUDA(cudaEventSynchronize(std::get<2>(t)), "cudaEventSynchronize");
    NB_CUDA(cudaEventElapsedTime(&m, std::get<1>(t), std::get<2>(t)), "cudaEventElapsedTime");
    *ms[std::get<0>(t)] += m;
    *cnt[std::get<0>(t)] += 1;
  }
  if (reset) {
    for (auto& t : pt->timed) {
      pt->event_pool.push_back(std::get<1>(t));
      pt->event_pool.push_back(std::get<2>(t));
    }
    pt->timed.clear();
  }
  return NB_OK;
}

int nb_pathtracer_enable_trace_counters(nb_pathtracer* pt, int enable) {
  if (!pt) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (!enable) {
    pt->counter_mem.release();
    pt->d_trace_counts = nullptr;
    return NB_OK;
  }
  if (pt->d_trace_counts) return NB_OK;
  void* p = nullptr;
  const size_t bytes = nb::kTraceCounterSlots * kMaxBounceSlots * sizeof(unsigned long long);
  int rc = pt->counter_mem.alloc(bytes, &p);
  if (rc) return rc;
  NB_CUDA(cudaMemset(p, 0, bytes), "cudaMemset(trace counters)");
  pt->d_trace_counts = (unsigned long long*)p;
  return NB_OK;
}

int nb_pathtracer_trace_counters(nb_pathtracer* pt, nb_trace_counters* out, uint32_t n_bounces, int reset,
                                 void* stream) {
  if (!pt || (!out && n_bounces)) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (!pt->d_trace_counts) return fail(NB_ERR_INVALID_ARG, "trace counters are not enabled");
  if (n_bounces > kMaxBounceSlots) return fail(NB_ERR_INVALID_ARG, "at most %u bounce slots", kMaxBounceSlots);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<unsigned long long> h(nb::kTraceCounterSlots * kMaxBounceSlots);
  NB_CUDA(cudaMemcpyAsync(h.data(), pt->d_trace_counts, h.size() * sizeof(h[0]), cudaMemcpyDeviceToHost, st),
          "cudaMemcpyAsync(trace counters)");
  NB_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  for (uint32_t b = 0; b < n_bounces; ++b) {
    const unsigned long long* c = h.data() + nb::kTraceCounterSlots * b;
    out[b] = nb_trace_counters{c[5], c[0], c[1], c[2], c[3], c[4], c[6], c[7], c[8], c[9], c[10]};
  }
  if (reset) NB_CUDA(cudaMemsetAsync(pt->d_trace_counts, 0, h.size() * sizeof(h[0]), st), "cudaMemsetAsync");
  return NB_OK;
}

int nb_pathtracer_set_sampling(nb_pathtracer* pt, uint32_t flags) {
  if (!pt) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (flags & ~(uint32_t)NB_SAMPLE_ENV_NEE) return fail(NB_ERR_INVALID_ARG, "unknown sampling flags 0x%x", flags);
  pt->sampling = flags;
  return NB_OK;
}

int nb_pathtracer_set_rr_start_bounce(nb_pathtracer* pt, uint32_t bounce) {
  if (!pt) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  pt->rr_start = bounce;
  return NB_OK;
}

int nb_pathtracer_get_sampling(const nb_pathtracer* pt, uint32_t* flags) {
  if (!pt || !flags) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  *flags = pt->sampling;
  return NB_OK;
}

int nb_env_sample(const nb_env* env, const float* u, size_t n, float* out, void* stream) {
  if (!env || (!u && n) || (!out && n)) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (n > 0x7FFFFFFFull) return fail(NB_ERR_INVALID_ARG, "too many samples");
  NB_CUDA(launch_env_sample(env->dev, u, (uint32_t)n, (float4*)out, sm_count(), (cudaStream_t)stream),
          "env sample launch");
  return NB_OK;
}

int nb_pathtracer_set_cache(nb_pathtracer* pt, nb_cache* cache) {
  if (!pt) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  pt->cache = cache;
  return NB_OK;
}

int nb_pathtracer_invalidate(nb_pathtracer* pt) {
  if (!pt) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  pt->globals.sample = 0;
  return NB_OK;
}

int nb_pathtracer_resize(nb_pathtracer* pt, uint32_t width, uint32_t height) {
  if (!pt) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if ((uint64_t)width * height > 0x7FFFFFFFull) return fail(NB_ERR_INVALID_ARG, "image too large");
  return alloc_image(pt, width, height);
}

int nb_pathtracer_get_globals(const nb_pathtracer* pt, nb_globals* out) {
  if (!pt || !out) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  *out = pt->globals;
  return NB_OK;
}

int nb_pathtracer_set_globals(nb_pathtracer* pt, const nb_globals* g) {
  if (!pt || !g) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (g->bounces + 2 > kMaxBounceSlots) return fail(NB_ERR_INVALID_ARG, "bounces must be <= %u", kMaxBounceSlots - 2);
  pt->globals = *g;
  return NB_OK;
}

uint32_t nb_pathtracer_sample_count(const nb_pathtracer* pt) { return pt ? pt->globals.sample : 0; }
uint32_t nb_pathtracer_max_sample_count(const nb_pathtracer* pt) { return pt ? pt->max_sample_count : 0; }

int nb_pathtracer_output(const nb_pathtracer* pt, float** device_rgba, uint32_t* width, uint32_t* height) {
  if (!pt) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (device_rgba) *device_rgba = pt->d_out;
  if (width) *width = pt->width;
  if (height) *height = pt->height;
  return NB_OK;
}

int nb_pathtracer_download(const nb_pathtracer* pt, float* host_rgba, void* stream) {
  if (!pt || (!host_rgba && pt->width != 0 && pt->height != 0)) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  size_t n = (size_t)pt->width * pt->height * 4 * sizeof(float);
  if (!n) return NB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  NB_CUDA(cudaMemcpyAsync(host_rgba, pt->d_out, n, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync(image)");
  NB_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  return NB_OK;
}

int nb_pathtracer_last_stats(const nb_pathtracer* pt, uint64_t* rays, uint32_t* status, void* stream) {
  if (!pt) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long r = 0;
  uint32_t s = 0;
  NB_CUDA(cudaMemcpyAsync(&r, pt->d_rays, sizeof(r), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
  NB_CUDA(cudaMemcpyAsync(&s, pt->d_status, sizeof(s), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
  NB_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (rays) *rays = r;
  if (status) *status = s;
  if (s & nbd::kStatusStackOverflow) return fail(NB_ERR_STACK_OVERFLOW, "traversal stack overflow");
  if (s & nbd::kStatusIterationCap) return fail(NB_ERR_TIMEOUT, "traversal iteration cap reached");
  return NB_OK;
}

// ---- traversal queries -------------------------------------------------------------------
static int check_status(const nb_scene* scene, cudaStream_t st, uint32_t* out = nullptr) {
  uint32_t s = 0;
  NB_CUDA(cudaMemcpyAsync(&s, scene->d_status, sizeof(s), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
  NB_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (out) *out = s;
  if (s & nbd::kStatusStackOverflow) return fail(NB_ERR_STACK_OVERFLOW, "traversal stack overflow");
  if (s & nbd::kStatusIterationCap) return fail(NB_ERR_TIMEOUT, "traversal iteration cap reached");
  return NB_OK;
}

int nb_scene_status(const nb_scene* scene, uint32_t* status, void* stream) {
  if (!scene) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  return check_status(scene, (cudaStream_t)stream, status);
}

int nb_trace_rays(const nb_scene* scene, const float* rays, size_t n, uint32_t flags, float* hits,
                  uint32_t* instances, void* stream) {
  if (!scene || (n && (!rays || !hits))) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (flags & ~(uint32_t)(NB_TRACE_ANY | NB_TRACE_INCOHERENT))
    return fail(NB_ERR_INVALID_ARG, "unknown trace flags 0x%x", flags);
  if (n > 0xFFFFFFE0ull) return fail(NB_ERR_INVALID_ARG, "too many rays in one call");
  if (!scene->uploaded) return fail(NB_ERR_INVALID_ARG, "scene was built with NB_SCENE_HOST_ONLY");
  cudaStream_t st = (cudaStream_t)stream;
  NB_CUDA(cudaMemsetAsync(scene->d_status, 0, sizeof(uint32_t), st), "cudaMemsetAsync");
  cudaError_t e = launch_trace_rays(scene->dev, rays, (uint32_t)n, (flags & NB_TRACE_ANY) != 0,
                                    (flags & NB_TRACE_INCOHERENT) != 0, hits, instances,
                                    scene->d_fetch, scene->d_status, scene->sms, st);
  if (e != cudaSuccess) return cuda_fail(e, "trace launch");
  return NB_OK;
}

int nb_trace_rays_host(const nb_scene* scene, const float* rays, size_t n, uint32_t flags, float* hits,
                       uint32_t* instances, void* stream) {
  if (!scene || (n && (!rays || !hits))) return fail(NB_ERR_INVALID_ARG, "NULL argument");
  if (n > 0xFFFFFFE0ull) return fail(NB_ERR_INVALID_ARG, "too many rays in one call");
  if (!scene->uploaded) return fail(NB_ERR_INVALID_ARG, "scene was built with NB_SCENE_HOST_ONLY");
  cudaStream_t st = (cudaStream_t)stream;
  DeviceArena tmp;
  void *dr = nullptr, *dh = nullptr, *di = nullptr;
  int rc;
  if ((rc = tmp.alloc(std::max<size_t>(1, n) * 32, &dr)) || (rc = tmp.alloc(std::max<size_t>(1, n) * 16, &dh)) ||
      (instances && (rc = tmp.alloc(std::max<size_t>(1, n) * 4, &di)))) {
    tmp.release();
    return rc;
  }
  cudaError_t e = cudaMemcpyAsync(dr, rays, n * 32, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    rc = nb_trace_rays(scene, (const float*)dr, n, flags, (float*)dh, (uint32_t*)di, stream);
    if (!rc) e = cudaMemcpyAsync(hits, dh, n * 16, cudaMemcpyDeviceToHost, st);
    if (!rc && e == cudaSuccess && instances) e = cudaMemcpyAsync(instances, di, n * 4, cudaMemcpyDeviceToHost, st);
  }
  if (!rc && e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpyAsync(trace)");
  if (!rc) rc = check_status(scene, st);
  else cudaStreamSynchronize(st);
  tmp.release();
  return rc;
}

}  // extern "C"

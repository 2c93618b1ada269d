/*
 * nbounce.h - C ABI of the GB300-native nBounce path-tracing pass.
 *
 * This library is a drop-in for the reference's path-tracing compute pass
 * (julcst/nbounce, src/pathtracing/pathtracer.rs + pathtracing.wgsl + raytracing_sw.wgsl +
 * common.wgsl, with the scene/BVH assembly of src/pathtracing/scene.rs and bvh.rs).
 * A Rust caller binds these symbols with an `extern "C"` block.
 *
 * Conventions
 *  - Every entry point returns an nb_status; NB_OK is 0.  On error, nb_last_error() returns a
 *    thread-local message.  Nothing aborts or traps.
 *  - Matrices are 16 floats, column-major (glam's Mat4 memory layout).
 *  - `stream` arguments are cudaStream_t passed as void*; NULL means the legacy default stream.
 *    Work is stream-ordered; entry points that return host data synchronise that stream.
 *  - Host arrays passed to *_create calls are only read during the call.  The library owns all
 *    device memory it allocates; handles are freed with the matching *_destroy.
 */
#ifndef NBOUNCE_H
#define NBOUNCE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NB_VERSION 100

/* Status codes (the reference returns Result<(), MeshError> from scene.rs:69-98 and panics
 * elsewhere; this ABI turns every failure into a code). */
typedef enum nb_status {
  NB_OK = 0,
  NB_ERR_INVALID_ARG = 1,     /* bad pointer, size, index or layout */
  NB_ERR_OOM = 2,             /* device or host allocation failed */
  NB_ERR_CUDA = 3,            /* a CUDA runtime call failed */
  NB_ERR_TIMEOUT = 4,         /* a bounded device loop gave up (traversal iteration cap) */
  NB_ERR_STACK_OVERFLOW = 5,  /* a traversal stack overflowed; results of that launch are suspect */
  NB_ERR_NO_DEVICE = 6,       /* no CUDA device is available */
  NB_ERR_EXHAUSTED = 7,       /* the Sobol table has no rows left (sample >= max_sample_count) */
  NB_ERR_BUSY = 8,            /* the render-job server's queue is full: the job was not queued */
  NB_ERR_CANCELLED = 9,       /* the job was cancelled (nb_server_cancel) */
  NB_ERR_EXPIRED = 10         /* the job's deadline passed before it finished */
} nb_status;

/* ---------------------------------------------------------------------------------------
 * Reference data layouts (byte-compatible with the reference's bytemuck uploads)
 * ------------------------------------------------------------------------------------- */

/* src/pathtracing/scene.rs:13-21 (48 bytes) */
typedef struct nb_vertex {
  float position[3];
  float u;
  float normal[3];
  float v;
  float tangent[4];
} nb_vertex;

/* src/pathtracing/bvh.rs:15-24 (32 bytes).  Leaf iff end > 0, covering primitives
 * [start, end); an inner node has end == 0 and children start, start + 1. */
typedef struct nb_bvh_node {
  float min[3];
  uint32_t start;
  float max[3];
  uint32_t end;
} nb_bvh_node;

/* src/pathtracing/scene.rs:220-230 (160 bytes), stored in TLAS-permuted order. */
typedef struct nb_instance {
  float world_to_local[16];
  float local_to_world[16];
  float color[4];
  float roughness;
  float metallic;
  float emissive;
  uint32_t node; /* BLAS root node index */
} nb_instance;

/* One glTF node-primitive as Scene::parse_gltf emits it (src/pathtracing/scene.rs:59-67,
 * 185-207): transform, material and a range [index_start, index_end) of the index buffer.
 * If world_to_local is all zeros the library inverts local_to_world itself. */
typedef struct nb_primitive {
  float local_to_world[16];
  float world_to_local[16];
  float color[4];
  float roughness;
  float metallic;
  float emissive;
  uint32_t index_start;
  uint32_t index_end;
} nb_primitive;

/* src/pathtracing/pathtracer.rs:26-44 / pathtracing.wgsl:17-22 (16 bytes). */
typedef struct nb_globals {
  uint32_t sample;            /* samples accumulated so far (1-based row of the last one) */
  float weight;               /* 1 / sample of the last dispatch */
  uint32_t bounces;           /* default 8 */
  float contribution_factor;  /* default 4 */
} nb_globals;

/* src/common/camera.rs:7-12.  The pass reads clip_to_world only. */
typedef struct nb_camera {
  float world_to_clip[16];
  float clip_to_world[16];
} nb_camera;

/* Environment seen by rays that miss (pathtracing.wgsl:167-170).  The reference samples a
 * BC6H cube map: nb_env_create_dds takes that file; this descriptor takes a constant colour,
 * an equirect RGBA32F map or six RGBA32F cube faces. */
enum { NB_ENV_CONSTANT = 0, NB_ENV_EQUIRECT = 1, NB_ENV_CUBE = 2 };
typedef struct nb_env_desc {
  uint32_t kind;
  float color[4];          /* NB_ENV_CONSTANT */
  const float* texels;     /* NB_ENV_EQUIRECT: height rows of width RGBA32F texels (host);
                              NB_ENV_CUBE: 6 faces (+X, -X, +Y, -Y, +Z, -Z: the layer order
                              of the reference's cube texture, texture.rs:89-144) of height
                              rows of width texels each, width == height; at most 32768
                              texels per side */
  uint32_t width, height;
} nb_env_desc;

typedef struct nb_scene nb_scene;
typedef struct nb_env nb_env;
typedef struct nb_pathtracer nb_pathtracer;

typedef struct nb_scene_info {
  uint64_t n_vertices, n_triangles, n_instances, n_blas_roots;
  uint64_t n_blas_nodes_ref, n_tlas_nodes_ref;   /* reference-layout node counts */
  uint64_t n_blas_nodes_gpu, n_tlas_nodes_gpu;   /* device 8-wide node records */
  uint64_t n_tlas_entries;                       /* device TLAS leaves: one per instance, one per
                                                    BLAS-root child of a large instance */
  uint64_t device_bytes;
  double build_ms;                               /* host BVH build time */
} nb_scene_info;

/* ---------------------------------------------------------------------------------------
 * Library
 * ------------------------------------------------------------------------------------- */
int nb_version(void);
/* Thread-local message describing the last failure on this thread ("" if none). */
const char* nb_last_error(void);
const char* nb_status_string(int status);

/* ---------------------------------------------------------------------------------------
 * Host-side builders (no GPU needed)
 * ------------------------------------------------------------------------------------- */

/* Sobol-Burley sample table in the reference's layout: row-major [sample][dimension set]
 * vec4, filled with 4D Owen-scrambled Sobol points (replaces sobol_burley::sample_4d at
 * src/pathtracing/pathtracer.rs:56-64).  out holds n_samples * n_dimsets * 4 floats. */
int nb_sobol_burley_table(uint32_t n_samples, uint32_t n_dimsets, uint32_t seed, float* out);

/* SAH BVH over one triangle list, node for node as BVHTree::append (src/pathtracing/bvh.rs:
 * 162-190) builds it.  positions: n_vertices * 3 floats.  Writes up to nodes_capacity nodes
 * (2 * n_triangles suffices) and the triangle-permuted index list (flatten_triangle_list,
 * bvh.rs:106-110) into indices_out (n_indices entries). */
int nb_bvh_build(const float* positions, size_t n_vertices, const uint32_t* indices, size_t n_indices,
                 nb_bvh_node* nodes_out, size_t nodes_capacity, size_t* n_nodes_out, uint32_t* indices_out);

/* ---------------------------------------------------------------------------------------
 * Scenes (SceneBuffers::from_scene, src/pathtracing/scene.rs:280-453)
 * ------------------------------------------------------------------------------------- */
enum {
  /* Build one BLAS per distinct index range instead of one per primitive.  The reference
   * builds one per glTF node-primitive (scene.rs:285-299), rebuilding a shared range in place;
   * those rebuilds are not idempotent (brute-force SAH ties resolve differently once the
   * triangles are permuted), so the reference's first BLAS of a shared mesh can go stale
   * against the final index buffer.  Without the flag the library reproduces that; with it
   * every instance of a mesh uses one consistent tree. */
  NB_SCENE_DEDUP_MESHES = 1u << 0,
  /* Build and validate on the host only (no device needed, nothing uploaded): the scene can
   * be exported and inspected but not rendered or traced. */
  NB_SCENE_HOST_ONLY = 1u << 1
};

/* Builds BLAS + TLAS on the host (parallel over BLASes) and uploads the scene in the
 * device layout.  indices are global vertex ids (scene.rs:173). */
int nb_scene_create(const nb_vertex* vertices, size_t n_vertices, const uint32_t* indices, size_t n_indices,
                    const nb_primitive* primitives, size_t n_primitives, uint32_t flags, nb_scene** out);

/* Takes the reference's own prebuilt buffers (the five storage buffers of bind group 1,
 * scene.rs:309-341 / raytracing_sw.wgsl:33-37) and uploads them in the device layout. */
int nb_scene_create_from_bvh(const nb_bvh_node* blas, size_t n_blas, const nb_bvh_node* tlas, size_t n_tlas,
                             const nb_instance* instances, size_t n_instances, const nb_vertex* vertices,
                             size_t n_vertices, const uint32_t* indices, size_t n_indices, nb_scene** out);

/* Copies the reference-layout buffers a scene was built from (NULL skips a buffer; sizes
 * come from nb_scene_get_info). */
int nb_scene_export(const nb_scene* scene, nb_bvh_node* blas, nb_bvh_node* tlas, nb_instance* instances,
                    uint32_t* indices);
int nb_scene_get_info(const nb_scene* scene, nb_scene_info* info);
void nb_scene_destroy(nb_scene* scene);

/* ---------------------------------------------------------------------------------------
 * Environment
 * ------------------------------------------------------------------------------------- */
int nb_env_create(const nb_env_desc* desc, nb_env** out);
void nb_env_destroy(nb_env* env);
/* EnvMap::load / Texture::create_cubemap (envmap.rs:12-17, texture.rs:89-144): an environment
 * from the bytes of a DDS cube-map file.  DXGI BC6H_UF16 - the reference's only format - and
 * BC6H_SF16 are decoded on the device; R16G16B16A16_FLOAT and R32G32B32A32_FLOAT (DX10 header,
 * or the legacy FourCC codes 113 / 116 with the cube-map caps bit) are read as they are.  A DX10
 * file is read as six array layers (+X, -X, +Y, -Y, +Z, -Z) whatever its array size says, as
 * texture.rs:95-96 forces them; of each layer's mip chain only level 0 is kept, the level the
 * pass samples (pathtracing.wgsl:168).  The result is an NB_ENV_CUBE environment. */
int nb_env_create_dds(const void* bytes, size_t n, nb_env** out);
/* BC6H block decoding on the device, host buffers in and out: blocks holds layers x
 * ceil(height / 4) x ceil(width / 4) 16-byte blocks in row-major block order; out receives
 * layers x height x width RGBA32F texels (alpha 1).  is_signed: 0 = BC6H_UF16, 1 = BC6H_SF16.
 * Width, height and layers up to 65536 each (NB_ERR_INVALID_ARG beyond). */
int nb_bc6h_decode(const void* blocks, uint32_t width, uint32_t height, uint32_t layers, uint32_t is_signed,
                   float* out);

/* ---------------------------------------------------------------------------------------
 * The pass (Pathtracer, src/pathtracing/pathtracer.rs:15-239)
 * ------------------------------------------------------------------------------------- */

/* Pathtracer::new (pathtracer.rs:51-161): allocates the RGBA32F width x height accumulation
 * image and the Sobol table.  sobol_table may be NULL (the library builds its own,
 * max_sample_count rows of 17 vec4, seed 0) or point to a caller-built table of
 * sobol_rows * 17 vec4 in the reference's layout (e.g. from the sobol_burley crate).
 * globals may be NULL (sample 0, weight 0, bounces 8, contribution_factor 4). */
int nb_pathtracer_create(uint32_t width, uint32_t height, const nb_globals* globals, const float* sobol_table,
                         uint32_t sobol_rows, nb_pathtracer** out);
void nb_pathtracer_destroy(nb_pathtracer* pt);

/* Pathtracer::dispatch (pathtracer.rs:225-239): adds one sample per pixel to the running
 * mean.  Returns NB_ERR_EXHAUSTED without work once sample >= max_sample_count. */
int nb_pathtracer_dispatch(nb_pathtracer* pt, const nb_scene* scene, const nb_camera* camera, const nb_env* env,
                           void* stream);
/* n_samples consecutive dispatches in one batched launch sequence; the image is identical to
 * n_samples calls of nb_pathtracer_dispatch.  Stops early at max_sample_count. */
int nb_pathtracer_render(nb_pathtracer* pt, const nb_scene* scene, const nb_camera* camera, const nb_env* env,
                         uint32_t n_samples, void* stream);

/* Paths in flight per wavefront batch (default 2^27).  Work buffers take ~132 bytes per
 * path; more paths keep late bounces busier.  No counterpart in the reference (it traces one
 * sample per pixel per dispatch). */
int nb_pathtracer_set_batch_paths(nb_pathtracer* pt, uint32_t paths);

int nb_pathtracer_invalidate(nb_pathtracer* pt);                           /* pathtracer.rs:221-223 */
int nb_pathtracer_resize(nb_pathtracer* pt, uint32_t width, uint32_t height); /* pathtracer.rs:208-210 */
int nb_pathtracer_get_globals(const nb_pathtracer* pt, nb_globals* out);
int nb_pathtracer_set_globals(nb_pathtracer* pt, const nb_globals* globals); /* pub globals (pathtracer.rs:21) */
uint32_t nb_pathtracer_sample_count(const nb_pathtracer* pt);               /* pathtracer.rs:217-219 */
uint32_t nb_pathtracer_max_sample_count(const nb_pathtracer* pt);           /* pathtracer.rs:23 */

/* output_texture() (pathtracer.rs:204-206): device pointer of the RGBA32F image, row-major,
 * row 0 first (the reference blit shows row 0 at the bottom of the screen). */
int nb_pathtracer_output(const nb_pathtracer* pt, float** device_rgba, uint32_t* width, uint32_t* height);
/* Copies the image into host memory (width * height * 4 floats) and synchronises stream. */
int nb_pathtracer_download(const nb_pathtracer* pt, float* host_rgba, void* stream);
/* Traversal queries issued by the last dispatch/render call (primary + extension rays) and
 * the device status word of that call (0 = clean).  Synchronises stream. */
int nb_pathtracer_last_stats(const nb_pathtracer* pt, uint64_t* rays, uint32_t* status, void* stream);

/* Per-kernel CUDA-event timing of the pass's launches, recorded on the launch stream (the
 * reference leaves GPU timestamps off, pathtracer.rs:229; "timer queries" is an open item of
 * its feature list).  Off by default.  raygen_ms covers the wave's start (counters, and radiance
 * zeroed for NEE and cache waves); camera rays are made inside the bounce-0 traversal and count
 * in trace_ms. */
typedef struct nb_kernel_times {
  double raygen_ms, trace_ms, shade_ms, accumulate_ms;
  uint64_t raygen_launches, trace_launches, shade_launches, accumulate_launches;
  double cache_infer_ms;        /* radiance-cache lookups (cache mode only) */
  double cache_train_ms;        /* training records + optimiser steps (cache mode only) */
  uint64_t cache_infer_launches, cache_train_launches;
} nb_kernel_times;
int nb_pathtracer_enable_timing(nb_pathtracer* pt, int enable);
/* Sums the recorded launch times (synchronises stream); reset != 0 clears the record. */
int nb_pathtracer_kernel_times(nb_pathtracer* pt, nb_kernel_times* out, int reset, void* stream);

/* Traversal work counters, per bounce: what the device's own layout fetches for the closest-hit
 * queries of that bounce - 80-byte 8-wide nodes (TLAS and BLAS), 48-byte triangle records,
 * 64-byte instance records - and the 8-byte stack entries pushed (each popped once).  While
 * enabled, renders run an instrumented copy of the traversal kernel (same results, slower);
 * the measurement counterpart of the reference's n_aabb / n_tri counters
 * (raytracing_sw.wgsl:187,207-208,261,280).  Off by default; no counterpart in the reference's
 * API. */
typedef struct nb_trace_counters {
  uint64_t rays;                 /* closest-hit queries traced */
  uint64_t tlas_node_tests;      /* 8-wide TLAS nodes tested */
  uint64_t blas_node_tests;      /* 8-wide BLAS nodes tested */
  uint64_t triangle_tests;       /* Moller-Trumbore tests */
  uint64_t instance_entries;     /* world-to-local ray transforms */
  uint64_t stack_pushes;         /* traversal stack entries written */
  /* how the 32 lanes of a warp share the node steps (lanes that test a node together count
   * one warp step): lane_steps / warp_steps = lanes per step; leaf_steps = warp steps in which
   * some lane tests leaf triangles, leaf_lanes = the lanes that do, leaf_warp_triangles = the
   * sum over those steps of the largest triangle count of a lane (the warp's iterations) */
  uint64_t warp_steps, lane_steps, leaf_steps, leaf_lanes, leaf_warp_triangles;
} nb_trace_counters;
int nb_pathtracer_enable_trace_counters(nb_pathtracer* pt, int enable);
/* Copies the counters of bounces 0 .. n_bounces-1 since the last reset into out[0 .. n_bounces-1]
 * (synchronises stream); reset != 0 clears them. */
int nb_pathtracer_trace_counters(nb_pathtracer* pt, nb_trace_counters* out, uint32_t n_bounces, int reset,
                                 void* stream);

/* Estimator options.  0 (default) is the reference's: BSDF sampling only, the environment
 * reached only by rays that escape.  NB_SAMPLE_ENV_NEE adds next-event estimation toward the
 * environment (the reference's README lists environment importance sampling as planned work,
 * README.md:20, pathtracing.wgsl:191 TODO): each non-emissive vertex also samples one
 * direction from the environment's radiance distribution (luminance x sin(theta) per equirect
 * texel; uniform for a constant environment) and traces a shadow ray; the two techniques are
 * combined per BRDF lobe by the power heuristic, so the image converges to the same result
 * with far less variance from small bright sources (a sun disc).  Ignored while a radiance
 * cache is attached. */
enum { NB_SAMPLE_ENV_NEE = 1u << 0 };
int nb_pathtracer_set_sampling(nb_pathtracer* pt, uint32_t flags);
/* Russian roulette schedule.  0 (default): the reference's, survival min(1 - (b/B)^8, 1) x
 * min(lum(T) cf, 1) at every bounce b (pathtracing.wgsl:225-236).  n > 0: survival 1 at
 * bounces b < n, the reference's from b = n on - the "RR from bounce 3" of the benchmark
 * configurations (n = 3).  The expected image is the same; only the noise and cost change. */
int nb_pathtracer_set_rr_start_bounce(nb_pathtracer* pt, uint32_t bounce);
int nb_pathtracer_get_sampling(const nb_pathtracer* pt, uint32_t* flags);
/* Environment importance samples: for n uniform pairs u (device, 2n floats) writes n x
 * (direction xyz, solid-angle density) to out (device, 4n floats).  Stream-ordered. */
int nb_env_sample(const nb_env* env, const float* u, size_t n, float* out, void* stream);

/* ---------------------------------------------------------------------------------------
 * Traversal (the intersect_scene query, raytracing_sw.wgsl:138-250, on caller rays)
 * ------------------------------------------------------------------------------------- */
enum {
  NB_TRACE_CLOSEST = 0,
  NB_TRACE_ANY = 1u << 0,       /* stop at the first accepted triangle (occlusion query) */
  NB_TRACE_INCOHERENT = 1u << 1 /* neighbouring rays of the array are unrelated (scattered origins or
                                   directions): a warp's lanes take new rays as theirs finish instead
                                   of tracing 32 neighbours to the end.  Same results; faster for
                                   such rays, slower for coherent ones (camera grids) */
};
/* rays: n records of 8 floats (origin.xyz, unused, direction.xyz, unused) in device memory.
 * hits: n float4 (t, u, v, triangle) with t = FLT_MAX (0x1.fffffep+127) on a miss and the
 * triangle as a u32 bit pattern (index into the scene's permuted triangle list).
 * instances: optional n u32 (TLAS-permuted instance index of the hit).
 * Asynchronous: nb_scene_status() reads the device status word of the last query. */
int nb_trace_rays(const nb_scene* scene, const float* rays, size_t n, uint32_t flags, float* hits,
                  uint32_t* instances, void* stream);
/* Synchronises stream and returns NB_ERR_STACK_OVERFLOW / NB_ERR_TIMEOUT if the last
 * traversal query on this scene raised the corresponding device status bit. */
int nb_scene_status(const nb_scene* scene, uint32_t* status, void* stream);
/* Renders samples first_sample .. first_sample + n_samples - 1 (1-based Sobol rows of the
 * library's 1024-row table) into the caller's device RGBA32F image `out_rgba` (width * height,
 * running mean as nb_pathtracer_dispatch keeps it) without allocating anything: for callers
 * that cannot allocate device memory while they render (an engine that owns all GPU memory
 * through its own allocator, a real-time loop whose footprint must stay fixed).  All scratch
 * lives in one static device array of 34.9 MB reserved per GPU at library load; images above
 * 262,144 pixels are rejected with NB_ERR_INVALID_ARG.  The first call on a device does a
 * one-time set-up there (looks up that array's device address and uploads the Sobol table
 * into it, synchronously).  Every call checks that the array still holds the table and repeats the set-up if not (after a
 * device reset the module is reloaded and its arrays start zeroed); scenes and environments
 * do not survive a device reset and must be created again.  Calls share the array (it keeps
 * the last call's contents); calls that overlap on the GPU race on it.  Synchronises stream.
 * No counterpart in the reference. */
int nb_render_static(const nb_scene* scene, const nb_env* env, const nb_camera* camera, uint32_t width,
                     uint32_t height, uint32_t first_sample, uint32_t n_samples, uint32_t bounces,
                     float contribution_factor, float* out_rgba, void* stream);

/* Same query with host buffers: copies rays in and hits out inside the call and checks the
 * status word. */
int nb_trace_rays_host(const nb_scene* scene, const float* rays, size_t n, uint32_t flags, float* hits,
                       uint32_t* instances, void* stream);

/* ---------------------------------------------------------------------------------------
 * Render-job server (continuous batching).  No counterpart in the reference, which renders
 * one progressive image per window: this serves many render requests against resident
 * scenes.  A scheduler thread admits queued jobs while their images fit the HBM budget,
 * packs samples of all admitted jobs into shared wavefronts (one segment of consecutive
 * Sobol rows per job per wave, paths of several scenes in one trace launch), and keeps up to
 * two waves in flight.  A job's image is bit-identical to rendering it alone with
 * nb_pathtracer_render: every path depends only on its own job, pixel and sample, and each
 * job's samples are accumulated in sample order.
 * ------------------------------------------------------------------------------------- */
typedef struct nb_server nb_server;

/* Per-job options.  NB_JOB_ENV_NEE: environment next-event estimation (as
 * NB_SAMPLE_ENV_NEE); such jobs share waves with the others, whose images stay the same.
 * NB_JOB_CACHE: render with the server's radiance cache of the job's scene (created on its
 * first such job, trained online by every cache job on that scene; nb_cache_default_config);
 * cache jobs run in cache waves of their own (one scene per wave), and a job's image depends
 * on what the cache learned before, so it is not reproducible alone vs in a mix.  The two
 * flags are exclusive; an
 * NB_JOB_ENV_NEE job's image is bit-identical to nb_pathtracer_render with NB_SAMPLE_ENV_NEE. */
enum { NB_JOB_ENV_NEE = 1u << 0, NB_JOB_CACHE = 1u << 1 };

typedef struct nb_job_desc {
  uint32_t scene;               /* slot from nb_server_add_scene */
  uint32_t env;                 /* slot from nb_server_add_env */
  nb_camera camera;
  uint32_t width, height;
  uint32_t spp;                 /* samples: Sobol rows 1..spp of the server's table */
  uint32_t bounces;
  float contribution_factor;
  uint32_t flags;               /* NB_JOB_* options (0: the reference estimator) */
  uint32_t deadline_ms;         /* 0: none; else the job fails with NB_ERR_EXPIRED if it has not
                                   finished this long after its submission (checked between waves) */
  float* host_out;              /* optional: width*height RGBA32F copied here when done */
} nb_job_desc;

typedef struct nb_job_info {
  int status;                   /* NB_OK once finished, else the job's error */
  uint32_t done;                /* 1 when finished (or failed) */
  double submit_ms, admit_ms, finish_ms;  /* server clock (ms since nb_server_create) */
} nb_job_info;

typedef struct nb_server_stats {
  uint64_t jobs_submitted, jobs_done, jobs_failed, waves;
  uint64_t rays;                /* traversal queries of all waves so far */
  double gpu_busy_ms;           /* sum of wave durations (CUDA events) */
  uint64_t bytes_in_use, peak_bytes_in_use, budget_bytes;
  uint32_t queued, active;      /* waiting for admission / admitted and unfinished */
  uint64_t jobs_rejected;       /* submissions refused with NB_ERR_BUSY (not counted as submitted) */
  uint64_t jobs_cancelled;      /* finished with NB_ERR_CANCELLED (also counted in jobs_failed) */
  uint64_t jobs_expired;        /* finished with NB_ERR_EXPIRED (also counted in jobs_failed) */
  uint32_t queue_limit;         /* nb_server_set_queue_limit (0: none) */
  uint32_t reserved;
} nb_server_stats;

/* hbm_budget_bytes bounds the server's device memory (path buffers + job images);
 * paths_per_wave sizes the shared path buffers (at least one image of the largest job). */
int nb_server_create(uint64_t hbm_budget_bytes, uint32_t paths_per_wave, nb_server** out);
/* Registers a resident scene / environment (the caller keeps them alive until destroy). */
int nb_server_add_scene(nb_server* server, const nb_scene* scene, uint32_t* slot);
int nb_server_add_env(nb_server* server, const nb_env* env, uint32_t* slot);
/* Configuration of the radiance caches the server creates for NB_JOB_CACHE jobs from now on
 * (NULL: nb_cache_default_config).  It is checked when a scene's cache is created, at its
 * first cache job; if nb_cache_create rejects it, that scene's queued and active cache jobs
 * fail with its status and every other job goes on.  Thread-safe. */
struct nb_cache_config; /* defined with the radiance cache API below */
int nb_server_set_cache_config(nb_server* server, const struct nb_cache_config* cfg);
/* Queues a job; thread-safe, returns at once.  NB_ERR_INVALID_ARG for bad slots or sizes,
 * NB_ERR_OOM if the job can never fit the budget, NB_ERR_BUSY if the queue limit is reached
 * (load shedding: the caller may retry later). */
int nb_server_submit(nb_server* server, const nb_job_desc* job, uint64_t* job_id);
/* Admission beyond saturation: at most max_queued jobs wait for admission (0, the default:
 * no limit, so above the GPU's throughput the queue and the latency grow without bound);
 * submissions beyond the limit return NB_ERR_BUSY at once.  Thread-safe. */
int nb_server_set_queue_limit(nb_server* server, uint32_t max_queued);
/* Cancels an unfinished job: a queued job leaves the queue; an admitted job gets no further
 * waves, its waves already on the GPU run to completion and its image is freed after them.
 * The job then finishes with NB_ERR_CANCELLED (nb_server_wait reports it) and every other
 * job's image is unchanged.  NB_ERR_INVALID_ARG for an unknown or already finished job. */
int nb_server_cancel(nb_server* server, uint64_t job_id);
/* Test hook for the allocation failure path: the nth job-image allocation from now on
 * (n >= 1; 0 disarms) fails as cudaMallocAsync does when device memory runs out, so that job
 * finishes with NB_ERR_OOM while the others go on, without exhausting the device. */
int nb_server_fail_alloc(nb_server* server, uint32_t nth);
/* Waits up to timeout_ms (< 0: forever) for a job; NB_ERR_TIMEOUT if it is not done yet. */
int nb_server_wait(nb_server* server, uint64_t job_id, int timeout_ms, nb_job_info* info);
/* Copies a finished job's image (when it was submitted without host_out) and frees it. */
int nb_server_fetch(nb_server* server, uint64_t job_id, float* host_rgba);
/* Forgets a finished job's record (a failed job's record is kept internally until its waves
 * still on the GPU have finished). */
int nb_server_release(nb_server* server, uint64_t job_id);
int nb_server_get_stats(nb_server* server, nb_server_stats* stats);
/* Finishes the queued and active jobs, then stops the scheduler and frees its memory. */
void nb_server_destroy(nb_server* server);

/* ---------------------------------------------------------------------------------------
 * Radiance cache.  No counterpart in the reference: its README lists neural radiance caching
 * (Mueller et al. 2021) as planned work (README.md:12,23,50-53).  A 64 -> 5 x 64 (ReLU) -> 3
 * MLP with BF16 weights/activations and FP32 accumulation, trained online on radiance from
 * training paths the tracer extends, queried where the other paths end their prefix.
 * Attach it to a path tracer with nb_pathtracer_set_cache; every render call is then one
 * frame: its paths terminate into the cache and the call trains it.
 * ------------------------------------------------------------------------------------- */
#define NB_CACHE_PARAMS 21504   /* 5 x 64 x 64 + 16 x 64 weights, rows [out][in] per layer */
#define NB_CACHE_INPUTS 64

typedef struct nb_cache nb_cache;

typedef struct nb_cache_config {
  float learning_rate;          /* Adam step size (1e-2) */
  float beta1, beta2, epsilon;  /* Adam (0.9, 0.99, 1e-8) */
  float spread;                 /* end a path's prefix once its spread exceeds spread * a0
                                   (0.01); < 0: at the primary hit; +inf: only at the last
                                   bounce */
  uint32_t train_records;       /* training records per frame (65,536); 0 with train_steps 0
                                   freezes the cache */
  uint32_t train_steps;         /* optimiser steps per frame over those records (4) */
  uint32_t extra_vertices;      /* vertices a training path records past its query vertex (3) */
  uint32_t seed;                /* weight initialisation */
  float ema;                    /* renders query an exponential moving average of the weights
                                   with this decay per step (0.99); 0: the weights themselves */
  float grad_clip;              /* bound on |dloss/doutput| per record and channel (0: none);
                                   limits the pull of rare very bright targets (sun hits) */
  uint32_t tensor_path;         /* lookups and training on NB_CACHE_TCGEN05 (default) or NB_CACHE_MMA_SYNC */
} nb_cache_config;

enum { NB_CACHE_TCGEN05 = 0, NB_CACHE_MMA_SYNC = 1 };

/* One cache input before encoding (64 bytes). */
typedef struct nb_cache_vertex {
  float pos[3];
  float roughness;
  float wo[3];                  /* unit direction towards the previous vertex */
  float metallic;
  float n[3];                   /* unit shading normal */
  uint32_t tag;                 /* ignored */
  float color[3];
  float pad;
} nb_cache_vertex;

typedef struct nb_cache_stats {
  uint64_t frames, adam_steps;
  uint32_t queries;             /* cache lookups of the last frame (image + training tails) */
  uint32_t records_found;       /* training records the last frame produced */
  uint32_t records_used;        /* of which trained on (at most train_records) */
  uint32_t training_groups;     /* groups of `stride` paths holding one training path each */
  uint32_t stride;              /* group size for the next frame (adapted to the budget) */
  float loss;                   /* mean relative L2 loss of the last frame's steps */
} nb_cache_stats;

void nb_cache_default_config(nb_cache_config* cfg);
int nb_cache_create(const nb_cache_config* cfg /* NULL: defaults */, nb_cache** out);
void nb_cache_destroy(nb_cache* cache);
int nb_cache_get_config(const nb_cache* cache, nb_cache_config* out);
/* Position normalisation box; defaults to the world bounds of the first scene rendered. */
int nb_cache_set_bounds(nb_cache* cache, const float lo[3], const float hi[3]);
/* FP32 master weights, NB_CACHE_PARAMS floats (host arrays).  Setting resets Adam. */
int nb_cache_get_weights(const nb_cache* cache, float* weights, size_t n);
int nb_cache_set_weights(nb_cache* cache, const float* weights, size_t n);
/* The network's inputs of n vertices: device arrays, out is n x NB_CACHE_INPUTS floats. */
int nb_cache_encode(nb_cache* cache, const nb_cache_vertex* vertices, size_t n, float* out, void* stream);
/* Network outputs (n x 3) of encoded inputs (n x 64); device arrays, BF16 inside.  With the
 * tcgen05 path it synchronises stream (NB_ERR_TIMEOUT if a tensor-core wait gave up). */
int nb_cache_infer(nb_cache* cache, const float* inputs, size_t n, float* out, void* stream);
/* Mean gradient (NB_CACHE_PARAMS floats, device) and loss (host, may be NULL) of the relative
 * L2 loss sum((p - y)^2 / (p^2 + 0.01)) / (3 n), the denominator held constant; targets n x 3.
 * Synchronises stream. */
int nb_cache_gradient(nb_cache* cache, const float* inputs, const float* targets, size_t n, float* grad,
                      float* loss, void* stream);
/* One Adam step on that loss over the batch.  Synchronises stream. */
int nb_cache_train_step(nb_cache* cache, const float* inputs, const float* targets, size_t n, float* loss,
                        void* stream);
/* Counters of the last frame (synchronises stream). */
int nb_cache_get_stats(nb_cache* cache, nb_cache_stats* out, void* stream);
/* Renders with the cache (NULL: plain path tracing).  The cache must outlive the attachment. */
int nb_pathtracer_set_cache(nb_pathtracer* pt, nb_cache* cache);

#ifdef __cplusplus
}
#endif

#endif /* NBOUNCE_H */

"""ctypes binding of libnbounce.so (the C ABI in include/nbounce.h).

Loading fails loudly when the library has not been built: there is no fallback path.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libnbounce.so")

NB_OK = 0
NB_ERR_INVALID_ARG = 1
NB_ERR_OOM = 2
NB_ERR_CUDA = 3
NB_ERR_TIMEOUT = 4
NB_ERR_STACK_OVERFLOW = 5
NB_ERR_NO_DEVICE = 6
NB_ERR_EXHAUSTED = 7
NB_ERR_BUSY = 8
NB_ERR_CANCELLED = 9
NB_ERR_EXPIRED = 10

NB_SCENE_DEDUP_MESHES = 1
NB_SCENE_HOST_ONLY = 2
NB_ENV_CONSTANT = 0
NB_ENV_EQUIRECT = 1
NB_ENV_CUBE = 2
NB_TRACE_CLOSEST = 0
NB_TRACE_ANY = 1
NB_TRACE_INCOHERENT = 2
NB_SAMPLE_ENV_NEE = 1
NB_JOB_ENV_NEE = 1
NB_JOB_CACHE = 2

VERTEX_DTYPE = np.dtype([("pos", "<f4", 3), ("u", "<f4"), ("nrm", "<f4", 3), ("v", "<f4"), ("tan", "<f4", 4)])
NODE_DTYPE = np.dtype([("min", "<f4", 3), ("start", "<u4"), ("max", "<f4", 3), ("end", "<u4")])
INSTANCE_DTYPE = np.dtype([("w2l", "<f4", 16), ("l2w", "<f4", 16), ("color", "<f4", 4), ("roughness", "<f4"),
                           ("metallic", "<f4"), ("emissive", "<f4"), ("node", "<u4")])
PRIMITIVE_DTYPE = np.dtype([("l2w", "<f4", 16), ("w2l", "<f4", 16), ("color", "<f4", 4), ("roughness", "<f4"),
                            ("metallic", "<f4"), ("emissive", "<f4"), ("index_start", "<u4"), ("index_end", "<u4")])


class NbGlobals(C.Structure):
    _fields_ = [("sample", C.c_uint32), ("weight", C.c_float), ("bounces", C.c_uint32),
                ("contribution_factor", C.c_float)]


class NbCamera(C.Structure):
    _fields_ = [("world_to_clip", C.c_float * 16), ("clip_to_world", C.c_float * 16)]


class NbEnvDesc(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("color", C.c_float * 4), ("texels", C.c_void_p), ("width", C.c_uint32),
                ("height", C.c_uint32)]


class NbSceneInfo(C.Structure):
    _fields_ = [("n_vertices", C.c_uint64), ("n_triangles", C.c_uint64), ("n_instances", C.c_uint64),
                ("n_blas_roots", C.c_uint64), ("n_blas_nodes_ref", C.c_uint64), ("n_tlas_nodes_ref", C.c_uint64),
                ("n_blas_nodes_gpu", C.c_uint64), ("n_tlas_nodes_gpu", C.c_uint64), ("n_tlas_entries", C.c_uint64),
                ("device_bytes", C.c_uint64),
                ("build_ms", C.c_double)]


class NbKernelTimes(C.Structure):
    _fields_ = [("raygen_ms", C.c_double), ("trace_ms", C.c_double), ("shade_ms", C.c_double),
                ("accumulate_ms", C.c_double), ("raygen_launches", C.c_uint64), ("trace_launches", C.c_uint64),
                ("shade_launches", C.c_uint64), ("accumulate_launches", C.c_uint64), ("cache_infer_ms", C.c_double),
                ("cache_train_ms", C.c_double), ("cache_infer_launches", C.c_uint64),
                ("cache_train_launches", C.c_uint64)]


class NbTraceCounters(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("tlas_node_tests", C.c_uint64), ("blas_node_tests", C.c_uint64),
                ("triangle_tests", C.c_uint64), ("instance_entries", C.c_uint64), ("stack_pushes", C.c_uint64),
                ("warp_steps", C.c_uint64), ("lane_steps", C.c_uint64), ("leaf_steps", C.c_uint64),
                ("leaf_lanes", C.c_uint64), ("leaf_warp_triangles", C.c_uint64)]


NB_CACHE_PARAMS = 21504
NB_CACHE_TCGEN05 = 0
NB_CACHE_MMA_SYNC = 1
NB_CACHE_INPUTS = 64
CACHE_VERTEX_DTYPE = np.dtype([("pos", "<f4", 3), ("roughness", "<f4"), ("wo", "<f4", 3), ("metallic", "<f4"),
                               ("n", "<f4", 3), ("tag", "<u4"), ("color", "<f4", 3), ("pad", "<f4")])


class NbCacheConfig(C.Structure):
    _fields_ = [("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("spread", C.c_float), ("train_records", C.c_uint32), ("train_steps", C.c_uint32),
                ("extra_vertices", C.c_uint32), ("seed", C.c_uint32), ("ema", C.c_float), ("grad_clip", C.c_float),
                ("tensor_path", C.c_uint32)]


class NbCacheStats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("adam_steps", C.c_uint64), ("queries", C.c_uint32),
                ("records_found", C.c_uint32), ("records_used", C.c_uint32), ("training_groups", C.c_uint32),
                ("stride", C.c_uint32), ("loss", C.c_float)]


class NbJobDesc(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("env", C.c_uint32), ("camera", NbCamera), ("width", C.c_uint32),
                ("height", C.c_uint32), ("spp", C.c_uint32), ("bounces", C.c_uint32),
                ("contribution_factor", C.c_float), ("flags", C.c_uint32), ("deadline_ms", C.c_uint32),
                ("host_out", C.c_void_p)]


class NbJobInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("done", C.c_uint32), ("submit_ms", C.c_double), ("admit_ms", C.c_double),
                ("finish_ms", C.c_double)]


class NbServerStats(C.Structure):
    _fields_ = [("jobs_submitted", C.c_uint64), ("jobs_done", C.c_uint64), ("jobs_failed", C.c_uint64),
                ("waves", C.c_uint64), ("rays", C.c_uint64), ("gpu_busy_ms", C.c_double),
                ("bytes_in_use", C.c_uint64), ("peak_bytes_in_use", C.c_uint64), ("budget_bytes", C.c_uint64),
                ("queued", C.c_uint32), ("active", C.c_uint32), ("jobs_rejected", C.c_uint64),
                ("jobs_cancelled", C.c_uint64), ("jobs_expired", C.c_uint64), ("queue_limit", C.c_uint32),
                ("reserved", C.c_uint32)]


class NbError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


_lib = None


def lib():
    """Loads libnbounce.so; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built; run nbounce_gb300.build.build() first")
    L = C.CDLL(LIB_PATH)
    vp, u32, u64, i32, sz = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_size_t
    sig = {
        "nb_version": ([], i32),
        "nb_last_error": ([], C.c_char_p),
        "nb_status_string": ([i32], C.c_char_p),
        "nb_sobol_burley_table": ([u32, u32, u32, vp], i32),
        "nb_bvh_build": ([vp, sz, vp, sz, vp, sz, vp, vp], i32),
        "nb_scene_create": ([vp, sz, vp, sz, vp, sz, u32, vp], i32),
        "nb_scene_create_from_bvh": ([vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp], i32),
        "nb_scene_export": ([vp, vp, vp, vp, vp], i32),
        "nb_scene_get_info": ([vp, vp], i32),
        "nb_scene_status": ([vp, vp, vp], i32),
        "nb_scene_destroy": ([vp], None),
        "nb_env_create": ([vp, vp], i32),
        "nb_env_destroy": ([vp], None),
        "nb_env_create_dds": ([vp, sz, vp], i32),
        "nb_bc6h_decode": ([vp, u32, u32, u32, u32, vp], i32),
        "nb_pathtracer_create": ([u32, u32, vp, vp, u32, vp], i32),
        "nb_pathtracer_destroy": ([vp], None),
        "nb_pathtracer_dispatch": ([vp, vp, vp, vp, vp], i32),
        "nb_pathtracer_render": ([vp, vp, vp, vp, u32, vp], i32),
        "nb_pathtracer_invalidate": ([vp], i32),
        "nb_pathtracer_resize": ([vp, u32, u32], i32),
        "nb_pathtracer_get_globals": ([vp, vp], i32),
        "nb_pathtracer_set_globals": ([vp, vp], i32),
        "nb_pathtracer_sample_count": ([vp], u32),
        "nb_pathtracer_max_sample_count": ([vp], u32),
        "nb_pathtracer_output": ([vp, vp, vp, vp], i32),
        "nb_pathtracer_download": ([vp, vp, vp], i32),
        "nb_pathtracer_last_stats": ([vp, vp, vp, vp], i32),
        "nb_pathtracer_set_batch_paths": ([vp, u32], i32),
        "nb_pathtracer_enable_timing": ([vp, i32], i32),
        "nb_pathtracer_kernel_times": ([vp, vp, i32, vp], i32),
        "nb_pathtracer_enable_trace_counters": ([vp, i32], i32),
        "nb_pathtracer_trace_counters": ([vp, vp, u32, i32, vp], i32),
        "nb_trace_rays": ([vp, vp, sz, u32, vp, vp, vp], i32),
        "nb_trace_rays_host": ([vp, vp, sz, u32, vp, vp, vp], i32),
        "nb_render_static": ([vp, vp, vp, u32, u32, u32, u32, u32, C.c_float, vp, vp], i32),
        "nb_server_create": ([u64, u32, vp], i32),
        "nb_server_add_scene": ([vp, vp, vp], i32),
        "nb_server_add_env": ([vp, vp, vp], i32),
        "nb_server_submit": ([vp, vp, vp], i32),
        "nb_server_set_cache_config": ([vp, vp], i32),
        "nb_server_wait": ([vp, u64, i32, vp], i32),
        "nb_server_fetch": ([vp, u64, vp], i32),
        "nb_server_release": ([vp, u64], i32),
        "nb_server_get_stats": ([vp, vp], i32),
        "nb_server_set_queue_limit": ([vp, u32], i32),
        "nb_server_cancel": ([vp, u64], i32),
        "nb_server_fail_alloc": ([vp, u32], i32),
        "nb_server_destroy": ([vp], None),
        "nb_cache_default_config": ([vp], None),
        "nb_cache_create": ([vp, vp], i32),
        "nb_cache_destroy": ([vp], None),
        "nb_cache_get_config": ([vp, vp], i32),
        "nb_cache_set_bounds": ([vp, vp, vp], i32),
        "nb_cache_get_weights": ([vp, vp, sz], i32),
        "nb_cache_set_weights": ([vp, vp, sz], i32),
        "nb_cache_encode": ([vp, vp, sz, vp, vp], i32),
        "nb_cache_infer": ([vp, vp, sz, vp, vp], i32),
        "nb_cache_gradient": ([vp, vp, vp, sz, vp, vp, vp], i32),
        "nb_cache_train_step": ([vp, vp, vp, sz, vp, vp], i32),
        "nb_cache_get_stats": ([vp, vp, vp], i32),
        "nb_pathtracer_set_cache": ([vp, vp], i32),
        "nb_pathtracer_set_sampling": ([vp, u32], i32),
        "nb_pathtracer_set_rr_start_bounce": ([vp, u32], i32),
        "nb_pathtracer_get_sampling": ([vp, vp], i32),
        "nb_env_sample": ([vp, vp, sz, vp, vp], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def check(status):
    if status != NB_OK:
        msg = lib().nb_last_error().decode(errors="replace")
        raise NbError(status, msg or lib().nb_status_string(status).decode())
    return status


def ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)

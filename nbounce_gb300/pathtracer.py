"""Host-side mirror of the reference's path-tracing pass interface.

Same names and argument meaning as the reference's Rust API, over the C ABI:

* ``SceneBuffers.from_scene``  - ``SceneBuffers::from_scene`` (src/pathtracing/scene.rs:280-453)
* ``SceneBuffers.from_bvh``    - the five prebuilt storage buffers of bind group 1
* ``Globals``                  - the 16-byte push constants (src/pathtracing/pathtracer.rs:26-44)
* ``Pathtracer``               - ``Pathtracer::{new, dispatch, invalidate, resize, output_texture,
                                  sample_count}`` (src/pathtracing/pathtracer.rs:47-239)

Errors raise ``NbError`` carrying the library's status code.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import NbError, check, lib, ptr


def _mat_colmajor(m):
    return [float(x) for x in np.asarray(m, np.float32).ravel(order="F")]


def _stream(stream):
    return None if stream is None else C.c_void_p(int(stream))


@dataclass
class Globals:
    sample: int = 0
    weight: float = 0.0
    bounces: int = 8
    contribution_factor: float = 4.0

    def to_c(self):
        return L.NbGlobals(self.sample, self.weight, self.bounces, self.contribution_factor)

    @classmethod
    def from_c(cls, g):
        return cls(int(g.sample), float(g.weight), int(g.bounces), float(g.contribution_factor))


def camera_struct(world_to_clip, clip_to_world):
    cam = L.NbCamera()
    cam.world_to_clip[:] = _mat_colmajor(world_to_clip)
    cam.clip_to_world[:] = _mat_colmajor(clip_to_world)
    return cam


def primitives_array(prims):
    arr = np.zeros(len(prims), L.PRIMITIVE_DTYPE)
    for i, p in enumerate(prims):
        arr[i]["l2w"] = np.asarray(p["l2w"], np.float32).ravel(order="F")
        arr[i]["w2l"] = np.asarray(p["w2l"], np.float32).ravel(order="F")
        arr[i]["color"] = p["color"]
        arr[i]["roughness"] = p["roughness"]
        arr[i]["metallic"] = p["metallic"]
        arr[i]["emissive"] = p["emissive"]
        arr[i]["index_start"] = p["index_start"]
        arr[i]["index_end"] = p["index_end"]
    return arr


class SceneBuffers:
    """A scene resident on the device (or host-only for inspection)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    @classmethod
    def from_scene(cls, vertices, indices, primitives, dedup=True, host_only=False):
        v = np.ascontiguousarray(vertices, dtype=L.VERTEX_DTYPE)
        i = np.ascontiguousarray(indices, dtype=np.uint32)
        p = primitives if isinstance(primitives, np.ndarray) else primitives_array(primitives)
        p = np.ascontiguousarray(p, dtype=L.PRIMITIVE_DTYPE)
        flags = (L.NB_SCENE_DEDUP_MESHES if dedup else 0) | (L.NB_SCENE_HOST_ONLY if host_only else 0)
        h = C.c_void_p()
        check(lib().nb_scene_create(ptr(v), v.size, ptr(i), i.size, ptr(p), p.size, flags, C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_desc(cls, desc, dedup=True, host_only=False):
        return cls.from_scene(desc.vertices, desc.indices, desc.primitives(), dedup=dedup, host_only=host_only)

    @classmethod
    def from_bvh(cls, blas, tlas, instances, vertices, indices):
        arrs = [np.ascontiguousarray(blas, dtype=L.NODE_DTYPE), np.ascontiguousarray(tlas, dtype=L.NODE_DTYPE),
                np.ascontiguousarray(instances, dtype=L.INSTANCE_DTYPE),
                np.ascontiguousarray(vertices, dtype=L.VERTEX_DTYPE), np.ascontiguousarray(indices, dtype=np.uint32)]
        h = C.c_void_p()
        check(lib().nb_scene_create_from_bvh(ptr(arrs[0]), arrs[0].size, ptr(arrs[1]), arrs[1].size, ptr(arrs[2]),
                                             arrs[2].size, ptr(arrs[3]), arrs[3].size, ptr(arrs[4]), arrs[4].size,
                                             C.byref(h)))
        return cls(h.value)

    @property
    def handle(self):
        return self._h

    def info(self):
        inf = L.NbSceneInfo()
        check(lib().nb_scene_get_info(self._h, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in L.NbSceneInfo._fields_}

    def export(self):
        inf = self.info()
        blas = np.zeros(inf["n_blas_nodes_ref"], L.NODE_DTYPE)
        tlas = np.zeros(inf["n_tlas_nodes_ref"], L.NODE_DTYPE)
        inst = np.zeros(inf["n_instances"], L.INSTANCE_DTYPE)
        idx = np.zeros(inf["n_triangles"] * 3, np.uint32)
        check(lib().nb_scene_export(self._h, ptr(blas), ptr(tlas), ptr(inst), ptr(idx)))
        return dict(blas=blas, tlas=tlas, instances=inst, indices=idx)

    @staticmethod
    def _trace_flags(any_hit, incoherent):
        return (L.NB_TRACE_ANY if any_hit else 0) | (L.NB_TRACE_INCOHERENT if incoherent else 0)

    def trace_host(self, rays, any_hit=False, with_instances=True, stream=None, incoherent=False):
        """rays (n, 8) float32 on the host -> (hits (n, 4) float32, instances (n,) u32 or None).
        incoherent: the rays' neighbours are unrelated (lanes refill; same results)."""
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = r.shape[0]
        hits = np.zeros((n, 4), np.float32)
        inst = np.zeros(n, np.uint32) if with_instances else None
        check(lib().nb_trace_rays_host(self._h, ptr(r), n, self._trace_flags(any_hit, incoherent), ptr(hits),
                                       ptr(inst), _stream(stream)))
        return hits, inst

    def trace_device(self, rays_ptr, n, hits_ptr, inst_ptr=None, any_hit=False, stream=None, incoherent=False):
        """Asynchronous query on device buffers given as integer addresses."""
        check(lib().nb_trace_rays(self._h, C.c_void_p(rays_ptr), n, self._trace_flags(any_hit, incoherent),
                                  C.c_void_p(hits_ptr), None if inst_ptr is None else C.c_void_p(inst_ptr),
                                  _stream(stream)))

    def status(self, stream=None):
        s = C.c_uint32()
        check(lib().nb_scene_status(self._h, C.byref(s), _stream(stream)))
        return s.value

    def close(self):
        if self._h:
            lib().nb_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class EnvMap:
    """Constant colour, equirect RGBA32F (texels: (h, w, 4)) or cube-map RGBA32F (cube:
    (6, n, n, 4), faces +X, -X, +Y, -Y, +Z, -Z) environment on the device; ``from_dds`` loads
    a DDS cube-map file as EnvMap::load does (envmap.rs:12)."""

    def __init__(self, color=(0.5, 0.6, 0.8), texels=None, cube=None):
        d = L.NbEnvDesc()
        d.color[:] = [float(color[0]), float(color[1]), float(color[2]), 1.0]
        self._tex = None
        if cube is not None:
            self._tex = np.ascontiguousarray(cube, dtype=np.float32)
            if self._tex.ndim != 4 or self._tex.shape[0] != 6 or self._tex.shape[3] != 4:
                raise ValueError("cube faces must be (6, n, n, 4)")
            d.kind = L.NB_ENV_CUBE
            d.texels = self._tex.ctypes.data
            d.height, d.width = self._tex.shape[1], self._tex.shape[2]
        elif texels is not None:
            self._tex = np.ascontiguousarray(texels, dtype=np.float32)
            d.kind = L.NB_ENV_EQUIRECT
            d.texels = self._tex.ctypes.data
            d.height, d.width = self._tex.shape[0], self._tex.shape[1]
        else:
            d.kind = L.NB_ENV_CONSTANT
        h = C.c_void_p()
        check(lib().nb_env_create(C.byref(d), C.byref(h)))
        self._h = h
        self._tex = None

    @classmethod
    def from_dds(cls, source):
        """EnvMap::load (envmap.rs:12-17): the cube map in a DDS file (a path or its bytes).
        BC6H_UF16 - the reference's format - and BC6H_SF16 are decoded on the device; RGBA16F
        and RGBA32F cube files are read as they are.  Mip 0 of each face is kept."""
        if isinstance(source, (bytes, bytearray, memoryview)):
            data = bytes(source)
        else:
            with open(source, "rb") as f:
                data = f.read()
        buf = C.create_string_buffer(data, len(data))
        env = cls.__new__(cls)
        env._tex = None
        env._h = None
        h = C.c_void_p()
        check(lib().nb_env_create_dds(buf, len(data), C.byref(h)))
        env._h = h
        return env

    @property
    def handle(self):
        return self._h

    def sample(self, u_dev, n, out_dev, stream=None):
        """Importance samples of this environment: u (n x 2 uniform floats) -> out (n x 4:
        direction, solid-angle density).  Device arrays (objects with data_ptr() or addresses)."""
        up = u_dev.data_ptr() if hasattr(u_dev, "data_ptr") else int(u_dev)
        op = out_dev.data_ptr() if hasattr(out_dev, "data_ptr") else int(out_dev)
        check(lib().nb_env_sample(self._h, C.c_void_p(up), int(n), C.c_void_p(op), _stream(stream)))

    def close(self):
        if self._h:
            lib().nb_env_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pathtracer:
    """Pathtracer::new + dispatch/invalidate/resize/output_texture (pathtracer.rs:47-239)."""

    COMPUTE_SIZE = 8

    def __init__(self, width, height, globals=None, sobol_table=None):
        g = (globals or Globals()).to_c()
        tab = None
        rows = 0
        if sobol_table is not None:
            tab = np.ascontiguousarray(sobol_table, dtype=np.float32)
            rows = tab.size // (17 * 4)
        h = C.c_void_p()
        check(lib().nb_pathtracer_create(width, height, C.byref(g), ptr(tab), rows, C.byref(h)))
        self._h = h

    @staticmethod
    def output_size(surface_width, surface_height, resolution_factor=0.3):
        """create_output_texture's sizing (pathtracer.rs:192-194): scale, then round down to 8."""
        w = int(np.float32(surface_width) * np.float32(resolution_factor))
        h = int(np.float32(surface_height) * np.float32(resolution_factor))
        return w // 8 * 8, h // 8 * 8

    @property
    def globals(self):
        g = L.NbGlobals()
        check(lib().nb_pathtracer_get_globals(self._h, C.byref(g)))
        return Globals.from_c(g)

    @globals.setter
    def globals(self, g):
        c = g.to_c()
        check(lib().nb_pathtracer_set_globals(self._h, C.byref(c)))

    @property
    def sample_count(self):
        return int(lib().nb_pathtracer_sample_count(self._h))

    @property
    def max_sample_count(self):
        return int(lib().nb_pathtracer_max_sample_count(self._h))

    def dispatch(self, scene, camera, env, stream=None):
        check(lib().nb_pathtracer_dispatch(self._h, scene.handle, C.byref(camera), env.handle, _stream(stream)))

    def render(self, scene, camera, env, n_samples, stream=None):
        check(lib().nb_pathtracer_render(self._h, scene.handle, C.byref(camera), env.handle, n_samples,
                                         _stream(stream)))

    def invalidate(self):
        check(lib().nb_pathtracer_invalidate(self._h))

    def resize(self, width, height):
        check(lib().nb_pathtracer_resize(self._h, width, height))

    def output_texture(self):
        p = C.c_void_p()
        w = C.c_uint32()
        h = C.c_uint32()
        check(lib().nb_pathtracer_output(self._h, C.byref(p), C.byref(w), C.byref(h)))
        return p.value, w.value, h.value

    def download(self, out=None, stream=None):
        _, w, h = self.output_texture()
        if out is None:
            out = np.empty((h, w, 4), np.float32)
        check(lib().nb_pathtracer_download(self._h, ptr(out), _stream(stream)))
        return out

    def last_stats(self, stream=None):
        rays = C.c_uint64()
        st = C.c_uint32()
        check(lib().nb_pathtracer_last_stats(self._h, C.byref(rays), C.byref(st), _stream(stream)))
        return int(rays.value), int(st.value)

    def set_batch_paths(self, paths):
        check(lib().nb_pathtracer_set_batch_paths(self._h, int(paths)))

    def set_sampling(self, env_nee=False):
        """Estimator options: env_nee adds environment next-event estimation (MIS-weighted)."""
        check(lib().nb_pathtracer_set_sampling(self._h, L.NB_SAMPLE_ENV_NEE if env_nee else 0))

    @property
    def sampling(self):
        f = C.c_uint32()
        check(lib().nb_pathtracer_get_sampling(self._h, C.byref(f)))
        return {"env_nee": bool(f.value & L.NB_SAMPLE_ENV_NEE)}

    def set_rr_start_bounce(self, bounce=0):
        """Russian roulette from this bounce on (0: the reference schedule at every bounce)."""
        check(lib().nb_pathtracer_set_rr_start_bounce(self._h, int(bounce)))

    def set_cache(self, cache):
        """Attach a RadianceCache (None: plain path tracing).  Keep the cache alive meanwhile."""
        self._cache = cache
        check(lib().nb_pathtracer_set_cache(self._h, None if cache is None else cache.handle))

    def enable_timing(self, enable=True):
        check(lib().nb_pathtracer_enable_timing(self._h, int(enable)))

    def kernel_times(self, reset=True, stream=None):
        t = L.NbKernelTimes()
        check(lib().nb_pathtracer_kernel_times(self._h, C.byref(t), int(reset), _stream(stream)))
        return {k: getattr(t, k) for k, _ in L.NbKernelTimes._fields_}

    def enable_trace_counters(self, enable=True):
        """Runs the instrumented traversal (same images, slower) that counts per bounce the
        wide nodes, triangles and instances it fetches and the stack entries it pushes."""
        check(lib().nb_pathtracer_enable_trace_counters(self._h, int(enable)))

    def trace_counters(self, n_bounces, reset=True, stream=None):
        """[{rays, tlas_node_tests, blas_node_tests, triangle_tests, instance_entries,
        stack_pushes}] for bounces 0 .. n_bounces - 1 since the last reset."""
        arr = (L.NbTraceCounters * n_bounces)()
        check(lib().nb_pathtracer_trace_counters(self._h, arr, int(n_bounces), int(reset), _stream(stream)))
        return [{k: int(getattr(c, k)) for k, _ in L.NbTraceCounters._fields_} for c in arr]

    def close(self):
        if self._h:
            lib().nb_pathtracer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sobol_burley_table(n_samples=1024, n_dimsets=17, seed=0):
    out = np.zeros((n_samples, n_dimsets, 4), np.float32)
    check(lib().nb_sobol_burley_table(n_samples, n_dimsets, seed, ptr(out)))
    return out


def bvh_build(positions, indices):
    """bvh.rs over one triangle list -> (nodes NODE_DTYPE, permuted indices)."""
    pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices, dtype=np.uint32).ravel()
    cap = max(1, 2 * (idx.size // 3))
    nodes = np.zeros(cap, L.NODE_DTYPE)
    perm = np.zeros_like(idx)
    n = C.c_size_t()
    check(lib().nb_bvh_build(ptr(pos), pos.shape[0], ptr(idx), idx.size, ptr(nodes), cap, C.byref(n), ptr(perm)))
    return nodes[: n.value].copy(), perm

"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module; the product package never does.  Every function wraps one ``or_*`` entry of
``nb_oracle.cpp``, which restates the reference pass (see that file's header for the
reference file:line map and the arithmetic contract).
"""
import ctypes as C
import os

import numpy as np

from .build import build_oracle

_lib = None

VERTEX_DTYPE = np.dtype([("pos", "<f4", 3), ("u", "<f4"), ("nrm", "<f4", 3), ("v", "<f4"), ("tan", "<f4", 4)])
NODE_DTYPE = np.dtype([("min", "<f4", 3), ("start", "<u4"), ("max", "<f4", 3), ("end", "<u4")])
INSTANCE_DTYPE = np.dtype([("w2l", "<f4", 16), ("l2w", "<f4", 16), ("color", "<f4", 4), ("roughness", "<f4"),
                           ("metallic", "<f4"), ("emissive", "<f4"), ("node", "<u4")])


class OrPrimitive(C.Structure):
    _fields_ = [("l2w", C.c_float * 16), ("w2l", C.c_float * 16), ("color", C.c_float * 4),
                ("roughness", C.c_float), ("metallic", C.c_float), ("emissive", C.c_float),
                ("index_start", C.c_uint32), ("index_end", C.c_uint32)]


class OrEnv(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("color", C.c_float * 4), ("texels", C.c_void_p),
                ("width", C.c_uint32), ("height", C.c_uint32)]


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        L = C.CDLL(path)
        vp, u32, u64, i32, f32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
        L.or_hash4u.argtypes = [vp, vp]
        L.or_hash4f.argtypes = [vp, vp]
        L.or_sincos.argtypes = [vp, u64, vp, vp]
        L.or_sobol_u32.argtypes = [u32, u32]
        L.or_sobol_u32.restype = u32
        L.or_sobol_table.argtypes = [u32, u32, u32, vp]
        L.or_bvh_build_triangles.argtypes = [vp, vp, u32, vp, vp]
        L.or_bvh_build_triangles.restype = u32
        L.or_scene_build.argtypes = [vp, u32, vp, u32, vp, u32, i32]
        L.or_scene_build.restype = vp
        L.or_scene_sizes.argtypes = [vp, vp, vp, vp, vp]
        L.or_scene_export.argtypes = [vp, vp, vp, vp, vp]
        L.or_scene_free.argtypes = [vp]
        L.or_trace.argtypes = [vp, vp, u64, i32, vp, vp, vp, i32]
        L.or_primary_rays.argtypes = [vp, u32, u32, vp, u64, u32, vp]
        L.or_render.argtypes = [vp, vp, u32, u32, vp, u64, u32, u32, u32, f32, vp, u32, u32, u32, u32,
                                vp, vp, i32, i32, vp, vp, u32]
        L.or_render.restype = u64
        L.or_env_lookup.argtypes = [vp, vp, u64, i32, vp]
        L.or_bc6h_decode_blocks.argtypes = [vp, C.c_size_t, i32, vp]
        L.or_bc6h_decode.argtypes = [vp, u32, u32, u32, i32, vp]
        _lib = L
    return _lib


def make_env(color=(0.5, 0.6, 0.8), texels=None, cube=None):
    """OrEnv for a constant colour, an equirect map (h, w, 4) or cube faces (6, n, n, 4);
    returns (env, the array it points into, which must outlive it)."""
    e = OrEnv()
    tex = None
    if cube is not None:
        tex = np.ascontiguousarray(cube, dtype=np.float32)
        e.kind, e.texels = 2, tex.ctypes.data
        e.height, e.width = tex.shape[1], tex.shape[2]
    elif texels is not None:
        tex = np.ascontiguousarray(texels, dtype=np.float32)
        e.kind, e.texels = 1, tex.ctypes.data
        e.height, e.width = tex.shape[0], tex.shape[1]
    else:
        e.kind = 0
        e.color[:] = [float(color[0]), float(color[1]), float(color[2]), 1.0]
    return e, tex


def env_lookup(dirs, color=(0.5, 0.6, 0.8), texels=None, cube=None, precision=32):
    """Environment radiance along directions (n, 3) -> (n, 3) float32."""
    d = np.ascontiguousarray(dirs, dtype=np.float32).reshape(-1, 3)
    e, keep = make_env(color, texels, cube)
    out = np.zeros((d.shape[0], 3), np.float32)
    lib().or_env_lookup(C.byref(e), _p(d), d.shape[0], precision, _p(out))
    del keep
    return out


def default_threads():
    return max(1, os.cpu_count() or 1)


# ---- common.wgsl --------------------------------------------------------------------------
def hash4u(s):
    s = np.ascontiguousarray(s, dtype=np.uint32)
    out = np.zeros(4, np.uint32)
    lib().or_hash4u(_p(s), _p(out))
    return out


def hash4f(s):
    s = np.ascontiguousarray(s, dtype=np.uint32)
    out = np.zeros(4, np.float32)
    lib().or_hash4f(_p(s), _p(out))
    return out


def sincos(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    lib().or_sincos(_p(x), x.size, _p(s), _p(c))
    return s, c


# ---- Sobol ---------------------------------------------------------------------------------
def sobol_u32(index, dim):
    return int(lib().or_sobol_u32(index, dim))


def sobol_table(n_samples=1024, n_dimsets=17, seed=0):
    out = np.zeros((n_samples, n_dimsets, 4), np.float32)
    lib().or_sobol_table(n_samples, n_dimsets, seed, _p(out))
    return out


# ---- BVH / scene ---------------------------------------------------------------------------
def bvh_build_triangles(positions, indices):
    positions = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
    indices = np.ascontiguousarray(indices, dtype=np.uint32).ravel()
    nt = indices.size // 3
    nodes = np.zeros(max(1, 2 * nt), NODE_DTYPE)
    idx_out = np.zeros_like(indices)
    n = lib().or_bvh_build_triangles(_p(positions), _p(indices), indices.size, _p(nodes), _p(idx_out))
    return nodes[:n].copy(), idx_out


def _primitives_struct(prims):
    arr = (OrPrimitive * max(1, len(prims)))()
    for i, p in enumerate(prims):
        arr[i].l2w[:] = [float(x) for x in np.asarray(p["l2w"], np.float32).ravel(order="F")]
        arr[i].w2l[:] = [float(x) for x in np.asarray(p["w2l"], np.float32).ravel(order="F")]
        arr[i].color[:] = [float(x) for x in p["color"]]
        arr[i].roughness = p["roughness"]
        arr[i].metallic = p["metallic"]
        arr[i].emissive = p["emissive"]
        arr[i].index_start = p["index_start"]
        arr[i].index_end = p["index_end"]
    return arr


class OracleScene:
    """Scene::parse_gltf output + SceneBuffers::from_scene (scene.rs:280-305) on the CPU."""

    def __init__(self, vertices, indices, primitives, dedup=False):
        self.vertices = np.ascontiguousarray(vertices, dtype=VERTEX_DTYPE)
        idx = np.ascontiguousarray(indices, dtype=np.uint32)
        self._prims = _primitives_struct(primitives)
        self.h = lib().or_scene_build(_p(self.vertices), self.vertices.size, _p(idx), idx.size,
                                      C.cast(self._prims, C.c_void_p), len(primitives), int(dedup))
        nb, nt, ni, nx = (C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint32())
        lib().or_scene_sizes(self.h, C.byref(nb), C.byref(nt), C.byref(ni), C.byref(nx))
        self.blas = np.zeros(nb.value, NODE_DTYPE)
        self.tlas = np.zeros(nt.value, NODE_DTYPE)
        self.instances = np.zeros(ni.value, INSTANCE_DTYPE)
        self.indices = np.zeros(nx.value, np.uint32)
        lib().or_scene_export(self.h, _p(self.blas), _p(self.tlas), _p(self.instances), _p(self.indices))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.or_scene_free(self.h)
            self.h = None

    def trace(self, rays, any_hit=False, threads=None):
        """rays: (n, 8) float32 (o.xyz, _, d.xyz, _).  Returns (t_uv (n,4) f32, ids (n,4) u32, counters (n,4) u32)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        hf = np.zeros((n, 4), np.float32)
        hu = np.zeros((n, 4), np.uint32)
        cnt = np.zeros((n, 4), np.uint32)
        lib().or_trace(self.h, _p(rays), n, int(any_hit), _p(hf), _p(hu), _p(cnt), threads or default_threads())
        return hf, hu, cnt

    def render(self, clip_to_world, width, height, sobol, first_sample, spp, bounces=8, contribution_factor=4.0,
               env=(0.5, 0.6, 0.8), region=None, out=None, per_sample=False, precision=32, threads=None,
               env_texels=None, rr_start=0, env_cube=None):
        """Running-mean render of samples first_sample..first_sample+spp-1 (1-based) over a pixel region.

        Returns (rgba (h, w, 4) float32, traversal queries, per-sample L (h, w, spp, 4) or None, overflow)."""
        x0, y0, w, h = region if region is not None else (0, 0, width, height)
        c2w = np.ascontiguousarray(np.asarray(clip_to_world, np.float32).ravel(order="F"))
        sob = np.ascontiguousarray(sobol, dtype=np.float32)
        if out is None:
            out = np.zeros((h, w, 4), np.float32)
        ps = np.zeros((h, w, spp, 4), np.float32) if per_sample else None
        e, tex = make_env(env, env_texels, env_cube)
        ovf = C.c_uint32(0)
        self.last_counters = np.zeros(4, np.uint64)
        rays = lib().or_render(self.h, _p(c2w), width, height, _p(sob), sob.size // 4, first_sample, spp, bounces,
                               contribution_factor, C.byref(e), x0, y0, w, h, _p(out), _p(ps), precision,
                               threads or default_threads(), C.byref(ovf), _p(self.last_counters), rr_start)
        return out, int(rays), ps, bool(ovf.value)

    def work_per_ray(self):
        """Mean reference work counters per traversal query of the last render:
        (n_aabb, n_tri, n_inst) as counted at raytracing_sw.wgsl:187,207-208,227,261,280."""
        rays, aabb, tri, inst = (float(x) for x in self.last_counters)
        return aabb / max(rays, 1.0), tri / max(rays, 1.0), inst / max(rays, 1.0)


def primary_rays(clip_to_world, width, height, sobol, sample):
    c2w = np.ascontiguousarray(np.asarray(clip_to_world, np.float32).ravel(order="F"))
    sob = np.ascontiguousarray(sobol, dtype=np.float32)
    out = np.zeros((height * width, 8), np.float32)
    lib().or_primary_rays(_p(c2w), width, height, _p(sob), sob.size // 4, sample, _p(out))
    return out


def bc6h_decode_blocks(blocks, signed=False):
    """Half-float bits (n, 16, 3) of n BC6H blocks ((n, 16) bytes): texels row-major in the
    block, channels RGB (bc6h.cpp)."""
    b = np.ascontiguousarray(blocks).reshape(-1).view(np.uint8).reshape(-1, 16)
    out = np.empty((b.shape[0], 16, 3), np.uint16)
    lib().or_bc6h_decode_blocks(_p(b), C.c_size_t(b.shape[0]), C.c_int(1 if signed else 0), _p(out))
    return out


def bc6h_decode(blocks, width, height, layers=1, signed=False):
    """(layers, height, width, 4) float32 texels (alpha 1) of BC6H blocks in row-major block
    order, (layers, ceil(h/4), ceil(w/4), 16) bytes (bc6h.cpp)."""
    b = np.ascontiguousarray(blocks).reshape(-1).view(np.uint8)
    need = ((width + 3) // 4) * ((height + 3) // 4) * layers * 16
    if b.size != need:
        raise ValueError(f"{b.size} bytes of BC6H blocks, {need} expected")
    out = np.empty((layers, height, width, 4), np.float32)
    lib().or_bc6h_decode(_p(b), C.c_uint32(width), C.c_uint32(height), C.c_uint32(layers),
                         C.c_int(1 if signed else 0), _p(out))
    return out

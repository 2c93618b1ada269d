"""Seeded synthetic scenes for the nBounce benchmark workloads, plus camera math.

A scene here is what ``Scene::parse_gltf`` (reference ``src/pathtracing/scene.rs:108-217``)
produces: one vertex array in the reference's 48-byte layout (``scene.rs:13-21``), one
u32 index buffer whose indices are already rebased to global vertex ids
(``scene.rs:173``), and a list of primitives, each with a local-to-world transform, a
material and a range of the index buffer (``scene.rs:59-67,199-206``).  Meshes used by
several instances share one index range, as glTF nodes that reference the same mesh do.

Camera matrices follow glam's ``Mat4::look_at_rh`` and ``Mat4::perspective_infinite_rh``
as used by ``src/common/camera.rs:121-142``; the pass consumes ``clip_to_world``.

The workloads:
* ``spheres_scene``  - 64 icosphere instances (subdivision 3, 1280 triangles) with centres
  U[-10,10]^3, radius U[0.5,1.5], random materials and a ground quad under a constant
  environment (0.5, 0.6, 0.8); 256x256 pinhole camera, 60 degree field of view.
* ``instanced_scene`` - 16 seeded meshes (noise-displaced icospheres and heightfield grids)
  in 1024 instances with random rotation and scale U[0.2,3], under a procedural
  2048x1024 RGBA32F sky with a 0.5 degree sun disc; 1920x1080 camera.
* ``triangle_soup``  - N random small triangles in [-1,1]^3 for the traversal
  microbenchmark, with coherent (camera grid) and incoherent (random) ray sets.
"""
from dataclasses import dataclass, field

import numpy as np

VERTEX_DTYPE = np.dtype([("pos", "<f4", 3), ("u", "<f4"), ("nrm", "<f4", 3), ("v", "<f4"), ("tan", "<f4", 4)])


# ------------------------------------------------------------------------------------------
# camera (glam conventions, column-major 4x4 in float64 then rounded)
# ------------------------------------------------------------------------------------------
def look_at_rh(eye, target, up):
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def perspective_infinite_rh(fov_y, aspect, z_near):
    f = 1.0 / np.tan(0.5 * fov_y)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = -1.0
    m[3, 2] = -1.0
    m[2, 3] = -z_near
    return m


def camera_matrices(eye, target, width, height, fov_y=np.pi / 3, up=(0.0, 1.0, 0.0), z_near=0.1):
    """Returns (world_to_clip, clip_to_world) as float32 4x4 (row-major numpy, i.e. M @ v)."""
    w2c = perspective_infinite_rh(fov_y, width / height, z_near) @ look_at_rh(eye, target, up)
    return w2c.astype(np.float32), np.linalg.inv(w2c).astype(np.float32)


# ------------------------------------------------------------------------------------------
# meshes
# ------------------------------------------------------------------------------------------
def icosphere(subdiv):
    """Unit icosphere: (positions (n,3) f64, faces (m,3) u32), counter-clockwise from outside."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = np.array(v, np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array(f, np.int64)
    for _ in range(subdiv):
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        mids = verts[uniq[:, 0]] + verts[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        base = len(verts)
        verts = np.concatenate([verts, mids])
        m = inv.reshape(3, -1).T + base  # midpoints of edges (0,1), (1,2), (2,0)
        a, b, c = faces[:, 0], faces[:, 1], faces[:, 2]
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        faces = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                                np.stack([ab, bc, ca], 1)])
    # make the winding counter-clockwise seen from outside: (v1-v0)x(v2-v0) . centroid > 0
    p = verts[faces]
    nrm = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    flip = (nrm * p.mean(axis=1)).sum(1) < 0
    faces[flip] = faces[flip][:, [0, 2, 1]]
    return verts, faces.astype(np.uint32)


def vertex_normals(pos, faces):
    p = pos[faces]
    fn = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])  # area weighted
    n = np.zeros_like(pos)
    for k in range(3):
        np.add.at(n, faces[:, k], fn)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return n


def sphere_tangents(n):
    up = np.where(np.abs(n[:, 1:2]) > 0.99, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    t = np.cross(up, n)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    return np.concatenate([t, np.ones((len(n), 1))], 1)


def pack_vertices(pos, nrm, tan, uv=None):
    out = np.zeros(len(pos), VERTEX_DTYPE)
    out["pos"] = pos
    out["nrm"] = nrm
    out["tan"] = tan
    if uv is not None:
        out["u"], out["v"] = uv[:, 0], uv[:, 1]
    return out


def smooth_noise_3d(p, rng, octaves=4, freq=2.0):
    """Sum of random-phase plane waves: a cheap band-limited noise on points p (n,3)."""
    acc = np.zeros(len(p))
    amp = 1.0
    for _ in range(octaves):
        for _ in range(4):
            k = rng.normal(size=3)
            k *= freq / np.linalg.norm(k)
            acc += amp * np.sin(p @ k + rng.uniform(0, 2 * np.pi))
        amp *= 0.5
        freq *= 2.0
    return acc / 4.0


def displaced_icosphere(subdiv, rng, amount=0.15):
    pos, faces = icosphere(subdiv)
    pos = pos * (1.0 + amount * smooth_noise_3d(pos, rng))[:, None]
    nrm = vertex_normals(pos, faces)
    return pack_vertices(pos, nrm, sphere_tangents(nrm)), faces


def heightfield(n, rng, amount=0.25):
    """n x n vertex grid over [-1,1]^2 in xz, displaced in y; faces counter-clockwise from +y."""
    xs = np.linspace(-1.0, 1.0, n)
    gx, gz = np.meshgrid(xs, xs, indexing="xy")
    gy = amount * smooth_noise_3d(np.stack([gx.ravel(), np.zeros(gx.size), gz.ravel()], 1), rng, freq=3.0)
    pos = np.stack([gx.ravel(), gy, gz.ravel()], 1)
    i = np.arange(n - 1)
    a = (i[None, :] + n * i[:, None]).ravel()
    b, c, d = a + 1, a + n, a + n + 1
    faces = np.concatenate([np.stack([a, c, b], 1), np.stack([b, c, d], 1)]).astype(np.uint32)
    nrm = vertex_normals(pos, faces)
    tan = np.cross(nrm, np.array([0.0, 0.0, 1.0]))  # roughly +x, orthogonal to n
    tan /= np.maximum(np.linalg.norm(tan, axis=1, keepdims=True), 1e-30)
    uv = np.stack([(gx.ravel() + 1) / 2, (gz.ravel() + 1) / 2], 1)
    return pack_vertices(pos, nrm, np.concatenate([tan, np.ones((len(pos), 1))], 1), uv), faces


def ground_quad(y, half):
    pos = np.array([[-half, y, -half], [half, y, -half], [-half, y, half], [half, y, half]], np.float64)
    faces = np.array([[0, 2, 1], [1, 2, 3]], np.uint32)  # (v1-v0)x(v2-v0) = +y
    nrm = np.tile([0.0, 1.0, 0.0], (4, 1))
    tan = np.tile([1.0, 0.0, 0.0, 1.0], (4, 1))
    return pack_vertices(pos, nrm, tan), faces


# ------------------------------------------------------------------------------------------
# transforms and materials
# ------------------------------------------------------------------------------------------
def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def trs(t, r=None, s=1.0):
    m = np.eye(4)
    m[:3, :3] = (np.eye(3) if r is None else r) * s
    m[:3, 3] = t
    return m


def random_material(rng):
    """Base colour U[0,1]^3, roughness U[0.05,1], metallic Bernoulli(0.3); 10% emissive with
    strength U[1,10].  Emission is expressed as in scene.rs:191-197: colour = emissive colour, emissive = 1."""
    color = rng.uniform(0.0, 1.0, 3)
    roughness = rng.uniform(0.05, 1.0)
    metallic = float(rng.uniform() < 0.3)
    emissive = 0.0
    if rng.uniform() < 0.1:
        color = color * rng.uniform(1.0, 10.0)
        emissive = 1.0
    return dict(color=np.array([*color, 1.0], np.float32), roughness=np.float32(roughness),
                metallic=np.float32(metallic), emissive=np.float32(emissive))


# ------------------------------------------------------------------------------------------
# scene container
# ------------------------------------------------------------------------------------------
@dataclass
class SceneDesc:
    vertices: np.ndarray                      # VERTEX_DTYPE
    indices: np.ndarray                       # u32, global vertex ids
    meshes: list                              # [(index_start, index_end)]
    instances: list                           # dicts: mesh, l2w, w2l, color, roughness, metallic, emissive
    width: int = 256
    height: int = 256
    clip_to_world: np.ndarray = None
    world_to_clip: np.ndarray = None
    env_color: tuple = (0.5, 0.6, 0.8)
    env_texels: np.ndarray = None             # (h, w, 4) f32 equirect, or None for a constant
    bounces: int = 8
    spp: int = 16
    extra: dict = field(default_factory=dict)

    def primitives(self):
        """Per-instance primitive records in the order Scene::parse_gltf emits them."""
        out = []
        for inst in self.instances:
            s, e = self.meshes[inst["mesh"]]
            out.append(dict(l2w=inst["l2w"], w2l=inst["w2l"], color=inst["color"], roughness=inst["roughness"],
                            metallic=inst["metallic"], emissive=inst["emissive"], index_start=s, index_end=e))
        return out

    @property
    def n_triangles_unique(self):
        return sum((e - s) // 3 for s, e in self.meshes)

    @property
    def n_triangles_instanced(self):
        return sum((self.meshes[i["mesh"]][1] - self.meshes[i["mesh"]][0]) // 3 for i in self.instances)


class _Builder:
    def __init__(self):
        self.v, self.i, self.meshes, self.nv, self.ni = [], [], [], 0, 0

    def add_mesh(self, verts, faces):
        self.v.append(verts)
        self.i.append(faces.astype(np.uint32).ravel() + np.uint32(self.nv))
        self.meshes.append((self.ni, self.ni + faces.size))
        self.nv += len(verts)
        self.ni += faces.size
        return len(self.meshes) - 1

    def finish(self):
        return np.concatenate(self.v), np.concatenate(self.i).astype(np.uint32), self.meshes


def _instance(mesh, l2w, mat):
    l2w32 = l2w.astype(np.float32)
    w2l32 = np.linalg.inv(l2w).astype(np.float32)
    return dict(mesh=mesh, l2w=l2w32, w2l=w2l32, **mat)


def spheres_scene(seed=0x5EED0, n_spheres=64, subdiv=3, width=256, height=256, spp=16, bounces=6):
    rng = np.random.default_rng(seed)
    b = _Builder()
    pos, faces = icosphere(subdiv)
    sphere = b.add_mesh(pack_vertices(pos, pos, sphere_tangents(pos)), faces)
    gv, gf = ground_quad(-11.0, 60.0)
    ground = b.add_mesh(gv, gf)
    insts = []
    for _ in range(n_spheres):
        c = rng.uniform(-10.0, 10.0, 3)
        r = rng.uniform(0.5, 1.5)
        insts.append(_instance(sphere, trs(c, None, r), random_material(rng)))
    insts.append(_instance(ground, np.eye(4), dict(color=np.array([0.8, 0.8, 0.8, 1.0], np.float32),
                                                  roughness=np.float32(0.9), metallic=np.float32(0.0),
                                                  emissive=np.float32(0.0))))
    v, i, meshes = b.finish()
    w2c, c2w = camera_matrices((0.0, 6.0, 34.0), (0.0, -1.0, 0.0), width, height)
    return SceneDesc(v, i, meshes, insts, width, height, c2w, w2c, (0.5, 0.6, 0.8), None, bounces, spp)


def quad_mesh(center, eu, ev):
    """Two triangles spanning center +- eu +- ev; front face (the side the backface-culled
    intersection test accepts) towards eu x ev."""
    c, eu, ev = (np.asarray(a, np.float64) for a in (center, eu, ev))
    pos = np.array([c - eu - ev, c + eu - ev, c - eu + ev, c + eu + ev])
    n = np.cross(eu, ev)
    n /= np.linalg.norm(n)
    t = eu / np.linalg.norm(eu)
    faces = np.array([[0, 1, 2], [1, 3, 2]], np.uint32)
    return pack_vertices(pos, np.tile(n, (4, 1)), np.tile([*t, 1.0], (4, 1))), faces


def room_scene(width=128, height=128, spp=16, bounces=8, light=(15.0, 15.0, 13.0)):
    """A closed 10 x 10 x 10 room lit only by an emissive ceiling panel: red and green side
    walls, white floor, ceiling and end walls, a diffuse and a rough gold sphere.  Radiance
    reaches most pixels after several diffuse bounces (interreflection-dominated)."""
    b = _Builder()
    walls = [  # (center, eu, ev, colour): front faces point into the room
        ((0, 0, 0), (5, 0, 0), (0, 0, -5), (0.75, 0.75, 0.75)),    # floor
        ((0, 10, 0), (5, 0, 0), (0, 0, 5), (0.75, 0.75, 0.75)),    # ceiling
        ((0, 5, -5), (5, 0, 0), (0, 5, 0), (0.75, 0.75, 0.75)),    # back
        ((0, 5, 5), (0, 5, 0), (5, 0, 0), (0.75, 0.75, 0.75)),     # front
        ((-5, 5, 0), (0, 5, 0), (0, 0, 5), (0.75, 0.12, 0.10)),    # left
        ((5, 5, 0), (0, 0, 5), (0, 5, 0), (0.12, 0.70, 0.12)),     # right
    ]
    insts = []
    for c, eu, ev, col in walls:
        m = b.add_mesh(*quad_mesh(c, eu, ev))
        insts.append(_instance(m, np.eye(4), dict(color=np.array([*col, 1.0], np.float32), roughness=np.float32(0.9),
                                                  metallic=np.float32(0.0), emissive=np.float32(0.0))))
    lm = b.add_mesh(*quad_mesh((0, 9.95, 0), (1.5, 0, 0), (0, 0, 1.5)))
    insts.append(_instance(lm, np.eye(4), dict(color=np.array([*light, 1.0], np.float32), roughness=np.float32(1.0),
                                               metallic=np.float32(0.0), emissive=np.float32(1.0))))
    pos, faces = icosphere(4)
    sph = b.add_mesh(pack_vertices(pos, pos, sphere_tangents(pos)), faces)
    insts.append(_instance(sph, trs((-2.0, 1.8, -1.5), None, 1.8),
                           dict(color=np.array([0.8, 0.8, 0.8, 1.0], np.float32), roughness=np.float32(0.8),
                                metallic=np.float32(0.0), emissive=np.float32(0.0))))
    insts.append(_instance(sph, trs((2.2, 1.5, 1.0), None, 1.5),
                           dict(color=np.array([1.0, 0.78, 0.34, 1.0], np.float32), roughness=np.float32(0.25),
                                metallic=np.float32(1.0), emissive=np.float32(0.0))))
    v, i, meshes = b.finish()
    w2c, c2w = camera_matrices((0.0, 5.0, 4.6), (0.0, 4.0, -5.0), width, height)
    return SceneDesc(v, i, meshes, insts, width, height, c2w, w2c, (0.0, 0.0, 0.0), None, bounces, spp)


def camera_path(n_frames, seed=0x5EEDC, eye=(0.0, 14.0, 62.0), target=(0.0, -2.0, 0.0), eye_spread=(16.0, 5.0, 10.0),
                target_spread=(4.0, 1.5, 4.0), n_keys=6):
    """Seeded camera spline: n_frames (eye, target) pairs on Catmull-Rom curves through n_keys
    random keys around eye / target (clamped end tangents; the last frame sits on the last key)."""
    rng = np.random.default_rng(seed)
    ke = np.asarray(eye, np.float64) + rng.uniform(-1.0, 1.0, (n_keys, 3)) * np.asarray(eye_spread)
    kt = np.asarray(target, np.float64) + rng.uniform(-1.0, 1.0, (n_keys, 3)) * np.asarray(target_spread)

    def catmull_rom(P, u):
        i = min(int(u), n_keys - 2)
        t = u - i
        p0, p1, p2, p3 = P[max(i - 1, 0)], P[i], P[i + 1], P[min(i + 2, n_keys - 1)]
        return 0.5 * (2.0 * p1 + (p2 - p0) * t + (2.0 * p0 - 5.0 * p1 + 4.0 * p2 - p3) * t * t
                      + (3.0 * p1 - p0 - 3.0 * p2 + p3) * t * t * t)

    return [(catmull_rom(ke, u), catmull_rom(kt, u)) for u in np.linspace(0.0, n_keys - 1.0, n_frames)]


def sky_envmap(seed, width=2048, height=1024, sun_dir=(0.3, 0.8, -0.52), sun_radiance=1.0e4,
               sun_diameter_deg=0.5):
    """Equirect RGBA32F sky: lognormal(0, 1.5) radiance field (smooth) + one sun disc."""
    rng = np.random.default_rng(seed)
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    theta = v * np.pi
    phi = (u - 0.5) * 2.0 * np.pi
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    d = np.stack([st * np.sin(phi)[None, :], np.broadcast_to(ct, (height, width)), -st * np.cos(phi)[None, :]], -1)
    g = smooth_noise_3d(d.reshape(-1, 3), rng, octaves=3, freq=1.5).reshape(height, width)
    g = (g - g.mean()) / (g.std() + 1e-12)
    lum = np.exp(1.5 * g)
    tint = np.stack([0.8 + 0.2 * np.clip(ct, -1, 1).repeat(width, 1), np.full((height, width), 0.9),
                     np.full((height, width), 1.0)], -1)
    img = lum[..., None] * tint
    s = np.asarray(sun_dir, np.float64)
    s /= np.linalg.norm(s)
    cosang = d @ s
    img[cosang > np.cos(np.radians(sun_diameter_deg / 2))] = sun_radiance
    out = np.ones((height, width, 4), np.float32)
    out[..., :3] = img
    return out


def cube_directions(n):
    """Unit directions of the texel centres of a cube map with n x n faces: (6, n, n, 3), faces
    +X, -X, +Y, -Y, +Z, -Z with (s, t) in [-1, 1] per the standard cube-map table."""
    c = 2.0 * (np.arange(n) + 0.5) / n - 1.0
    t, s = np.meshgrid(c, c, indexing="ij")
    one = np.ones_like(s)
    faces = [np.stack(f, -1) for f in ((one, -t, -s), (-one, -t, s), (s, one, t), (s, -one, -t), (s, -t, one),
                                       (-s, -t, -one))]
    d = np.stack(faces)
    return d / np.linalg.norm(d, axis=-1, keepdims=True)


def cube_from_equirect(texels, n):
    """Cube-map faces (6, n, n, 4) sampled (nearest texel) from an equirect RGBA32F map with the
    library's equirect mapping u = atan2(x, -z) / 2 pi + 1/2, v = acos(y) / pi."""
    h, w = texels.shape[:2]
    d = cube_directions(n)
    u = np.arctan2(d[..., 0], -d[..., 2]) / (2 * np.pi) + 0.5
    v = np.arccos(np.clip(d[..., 1], -1.0, 1.0)) / np.pi
    x = np.clip((u * w).astype(np.int64), 0, w - 1)
    y = np.clip((v * h).astype(np.int64), 0, h - 1)
    return np.ascontiguousarray(texels[y, x], dtype=np.float32)


def instanced_scene(seed=0x5EED1, n_instances=1024, width=1920, height=1080, spp=64, bounces=8,
                    env_size=(2048, 1024), scale=1.0):
    """16 seeded meshes (50k-1M triangles each, ~4.9M unique) in n_instances instances: one
    terrain (the largest heightfield scaled 45x, 12 below the centre) plus instances with
    random rotation, scale U[0.2,3] and positions in [-30,30] x [-10,15] x [-30,30], meshes
    drawn with probability ~ 1/triangles^2 (~70M instanced triangles).  ``scale`` < 1
    shrinks every mesh's resolution (for CPU-sized tests) keeping the scene's layout."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    sizes = []
    plan = [("hf", 160)] * 4 + [("ico", 6)] * 4 + [("ico", 7)] * 4 + [("hf", 512)] * 2 + [("hf", 708)] * 2
    for kind, p in plan:
        if kind == "ico":
            sub = max(1, p - (0 if scale >= 1 else int(round(np.log2(1 / scale) / 2))))
            v, f = displaced_icosphere(sub, rng)
        else:
            n = max(4, int(p * scale ** 0.5))
            v, f = heightfield(n, rng)
        b.add_mesh(v, f)
        sizes.append(len(f))
    sizes = np.array(sizes, np.float64)
    w = sizes ** -2.0
    w /= w.sum()
    terrain = dict(color=np.array([0.45, 0.42, 0.38, 1.0], np.float32), roughness=np.float32(0.8),
                   metallic=np.float32(0.0), emissive=np.float32(0.0))
    insts = [_instance(len(sizes) - 1, trs((0.0, -12.0, 0.0), None, 45.0), terrain)]
    for _ in range(n_instances - 1):
        m = int(rng.choice(len(sizes), p=w))
        t = rng.uniform(-30.0, 30.0, 3)
        t[1] = rng.uniform(-10.0, 15.0)
        insts.append(_instance(m, trs(t, random_rotation(rng), rng.uniform(0.2, 3.0)), random_material(rng)))
    v, i, meshes = b.finish()
    w2c, c2w = camera_matrices((0.0, 14.0, 62.0), (0.0, -2.0, 0.0), width, height)
    env = sky_envmap(seed + 1, *env_size)
    return SceneDesc(v, i, meshes, insts, width, height, c2w, w2c, (0.5, 0.6, 0.8), env, bounces, spp)


def triangle_soup(n_tris, seed=0x5EED2, edge=0.02):
    """n random triangles: centres U[-1,1]^3, vertices centre + N(0, edge/sqrt(3))^3 offsets."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1.0, 1.0, (n_tris, 1, 3))
    p = (c + rng.normal(0.0, edge / np.sqrt(3.0), (n_tris, 3, 3))).reshape(-1, 3)
    faces = np.arange(3 * n_tris, dtype=np.uint32).reshape(-1, 3)
    v = pack_vertices(p, np.tile([0.0, 1.0, 0.0], (len(p), 1)), np.tile([1.0, 0, 0, 1.0], (len(p), 1)))
    return v, faces


def soup_scene(n_tris, seed=0x5EED2):
    b = _Builder()
    v, f = triangle_soup(n_tris, seed)
    m = b.add_mesh(v, f)
    verts, idx, meshes = b.finish()
    inst = [_instance(m, np.eye(4), dict(color=np.array([0.8, 0.8, 0.8, 1], np.float32), roughness=np.float32(0.5),
                                         metallic=np.float32(0), emissive=np.float32(0)))]
    return SceneDesc(verts, idx, meshes, inst)


def coherent_rays(n_x, n_y, eye=(0.0, 0.0, 3.0), fov_deg=60.0):
    """Pinhole grid of n_x*n_y rays from eye toward -z: (n, 8) float32 (o, 0, d, 0)."""
    xs = (np.arange(n_x) + 0.5) / n_x * 2 - 1
    ys = (np.arange(n_y) + 0.5) / n_y * 2 - 1
    gx, gy = np.meshgrid(xs, ys, indexing="xy")
    tan_h = np.tan(np.radians(fov_deg) / 2)
    aspect = n_x / n_y
    d = np.stack([gx.ravel() * tan_h * aspect, gy.ravel() * tan_h, -np.ones(gx.size)], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.zeros((gx.size, 8), np.float32)
    out[:, :3] = eye
    out[:, 4:7] = d
    return out


def incoherent_rays(n, seed=0x5EED3):
    """Origins U[-1,1]^3, directions uniform on the sphere: (n, 8) float32."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 8), np.float32)
    out[:, :3] = rng.uniform(-1.0, 1.0, (n, 3))
    d = rng.normal(size=(n, 3))
    out[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    return out


def stratified_tiles(width, height, nx=6, ny=4, size=16):
    """nx * ny square tiles of `size` pixels, one centred in each cell of an nx x ny grid over
    the frame: (x0, y0, size, size) row by row.  The relMSE truth images and the CPU timing
    samples use these tiles, so that every part of the frame is weighted alike."""
    out = []
    for j in range(ny):
        for i in range(nx):
            x0 = (2 * i + 1) * width // (2 * nx) - size // 2
            y0 = (2 * j + 1) * height // (2 * ny) - size // 2
            out.append((int(x0), int(y0), int(size), int(size)))
    return out


def scene_fingerprint(desc):
    """A few numbers that change whenever the seeded generator's output changes: triangle and
    instance counts and binary64 sums of the vertex positions and instance transforms."""
    pos = desc.vertices["pos"].astype(np.float64)
    l2w = np.array([i["l2w"] for i in desc.instances], np.float64)
    return {"triangles": int(desc.n_triangles_unique), "instances": len(desc.instances),
            "pos_sum": float(pos.sum()), "l2w_sum": float(l2w.sum())}


def cache_camera(width=1920, height=1080, n_frames=300):
    """(world_to_clip, clip_to_world) of the radiance-cache workload's last camera: the end of
    camera_path, which sits on the spline's last key whatever the frame count."""
    eye, target = camera_path(n_frames)[-1]
    return camera_matrices(eye, target, width, height)

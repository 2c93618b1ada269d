"""Traversal on geometry at the edges of the format: degenerate and flat triangles, exact
duplicates and scene scales from 1e-3 to 1e4 against the oracle; and scenes deep enough to
overflow the 64-entry traversal stack or reach the iteration cap, which must report their
status (NB_ERR_STACK_OVERFLOW / NB_ERR_TIMEOUT) with every access in bounds and the context
usable afterwards."""
import ctypes as C

import numpy as np
import pytest

import nbounce_gb300 as nb
from nbounce_gb300 import _lib as L
from nbounce_gb300 import scenes
from oracle import oracle as O

from test_gpu_trace import NO_HIT, compare_hits

pytestmark = pytest.mark.gpu

MATERIAL = dict(color=np.array([0.8, 0.8, 0.8, 1.0], np.float32), roughness=np.float32(0.5),
                metallic=np.float32(0.0), emissive=np.float32(0.0))


def _pack(pos):
    pos = np.asarray(pos, np.float64)
    return scenes.pack_vertices(pos, np.tile([0.0, 0.0, 1.0], (len(pos), 1)), np.tile([1.0, 0.0, 0.0, 1.0],
                                                                                      (len(pos), 1)))


def _grid(n, axis, offset):
    """An n x n grid of quads (2 n^2 triangles) in the plane coordinate[axis] = offset."""
    g = np.linspace(-1.0, 1.0, n + 1)
    a, b = np.meshgrid(g, g, indexing="xy")
    pos = np.zeros(((n + 1) ** 2, 3))
    others = [k for k in range(3) if k != axis]
    pos[:, others[0]], pos[:, others[1]], pos[:, axis] = a.ravel(), b.ravel(), offset
    f = []
    for j in range(n):
        for i in range(n):
            q = j * (n + 1) + i
            f += [[q, q + 1, q + n + 2], [q, q + n + 2, q + n + 1]]
    return pos, np.array(f, np.uint32)


def degenerate_mesh(seed=17):
    """Flat grids (boxes of zero extent on one axis) in z = 0 and x = 0.3, and a soup with
    zero-area (collinear) triangles, triangles with a repeated vertex, slivers (two vertices
    1e-6 apart) and exact duplicates of other triangles (ties in t)."""
    rng = np.random.default_rng(seed)
    parts_p, parts_f, nv = [], [], 0
    for axis, off in ((2, 0.0), (0, 0.3)):
        p, f = _grid(16, axis, off)
        parts_p.append(p)
        parts_f.append(f + nv)
        nv += len(p)
    v, _ = scenes.triangle_soup(1500, seed=seed, edge=0.08)
    soup = v["pos"].astype(np.float64).reshape(-1, 3, 3)
    k = len(soup) // 5
    soup[:k, 2] = soup[:k, 0] + 0.37 * (soup[:k, 1] - soup[:k, 0])            # collinear
    soup[k:2 * k, 2] = soup[k:2 * k, 1]                                        # repeated vertex
    soup[2 * k:3 * k, 2] = soup[2 * k:3 * k, 1] + 1e-6 * rng.normal(size=(k, 3))  # slivers
    dup = soup[3 * k:3 * k + 200].copy()                                      # exact duplicates
    soup = np.concatenate([soup, dup])
    parts_p.append(soup.reshape(-1, 3))
    parts_f.append(np.arange(soup.size // 3, dtype=np.uint32).reshape(-1, 3) + nv)
    return np.concatenate(parts_p), np.concatenate(parts_f)


def scene_at_scale(s):
    """The degenerate mesh scaled by s in its vertices (identity instance) and, a second time,
    by an instance transform of scale s moved by 2.5 s along x."""
    pos, faces = degenerate_mesh()
    b = scenes._Builder()
    m0 = b.add_mesh(_pack(pos * s), faces)
    m1 = b.add_mesh(_pack(pos), faces)
    l2w = np.diag([s, s, s, 1.0])
    l2w[0, 3] = 2.5 * s
    insts = [scenes._instance(m0, np.eye(4), MATERIAL), scenes._instance(m1, l2w, MATERIAL)]
    v, i, meshes = b.finish()
    return scenes.SceneDesc(v, i, meshes, insts)


def rays_at(s, n, seed):
    """Rays aimed at random points of the scene from random directions, starting 3 s away (so
    the reference's absolute BIAS of 0.1 still lets them hit at every scale but the smallest)."""
    rng = np.random.default_rng(seed)
    target = np.stack([rng.uniform(-1.0, 3.5, n), rng.uniform(-1.0, 1.0, n), rng.uniform(-1.0, 1.0, n)], 1) * s
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.zeros((n, 8), np.float32)
    out[:, :3] = target - 3.0 * max(s, 0.05) * d
    out[:, 4:7] = d
    return out


@pytest.mark.parametrize("scale", [1e-3, 1.0, 1e4])
def test_degenerate_flat_and_duplicate_triangles_match_oracle(scale):
    desc = scene_at_scale(scale)
    gpu = nb.SceneBuffers.from_desc(desc, dedup=True)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    rays = rays_at(scale, 20000, seed=int(scale * 7) % 1000 + 3)
    for any_hit in (False, True):
        hits, inst = gpu.trace_host(rays, any_hit=any_hit)
        rf, ru, _ = orc.trace(rays, any_hit=any_hit)
        if any_hit:
            assert np.array_equal(hits[:, 0] != NO_HIT, rf[:, 0] != NO_HIT)
            continue
        # exact duplicates make exact ties, which either side may resolve its own way
        _, both = compare_hits(hits, inst, gpu.export()["indices"], rf, ru, max_tie_frac=0.05)
        assert both > 2000 if scale >= 1.0 else both > 0


def coincident_scene(n_tris, n_inst):
    """n_inst coincident instances of a mesh of n_tris coincident, tilted triangles (both
    windings, so a ray from either side hits): every box of both trees is the same box, so a
    ray pushes every hit child on the way down and nothing is culled by its closest hit."""
    pos = np.array([[-1.0, -1.0, -0.5], [1.0, -1.0, 0.5], [0.0, 1.0, 0.0]])
    faces = np.tile(np.array([[0, 1, 2], [0, 2, 1]], np.uint32), (n_tris // 2, 1))
    b = scenes._Builder()
    m = b.add_mesh(_pack(pos), faces)
    v, i, meshes = b.finish()
    return scenes.SceneDesc(v, i, meshes, [scenes._instance(m, np.eye(4), MATERIAL) for _ in range(n_inst)])


def _trace_raw(scene, rays, flags):
    n = rays.shape[0]
    hits = np.zeros((n, 4), np.float32)
    inst = np.zeros(n, np.uint32)
    rc = L.lib().nb_trace_rays_host(scene.handle, rays.ctypes.data_as(C.c_void_p), n, flags,
                                    hits.ctypes.data_as(C.c_void_p), inst.ctypes.data_as(C.c_void_p), None)
    word = C.c_uint32()
    L.lib().nb_scene_status(scene.handle, C.byref(word), None)
    return rc, word.value, hits, inst


def test_stack_overflow_and_iteration_cap_are_reported_in_bounds():
    """8192 coincident instances of 2^21 coincident triangles: about 10 wide-node levels of 7
    pushes each on the way to the first leaf, more than the 64-entry stack holds.  Pushes past
    the end are dropped and flagged; a closest-hit query, which visits every node of every
    instance, also stops at the iteration cap.  Hits stay valid, and the next query on the same
    scene reports a clean status."""
    desc = coincident_scene(1 << 21, 8192)
    scene = nb.SceneBuffers.from_desc(desc, dedup=True)
    n_tris = desc.indices.size // 3
    rng = np.random.default_rng(4)
    rays = np.zeros((64, 8), np.float32)
    rays[:, :2] = rng.uniform(-0.2, 0.2, (64, 2))
    rays[:, 2] = 5.0
    rays[:, 6] = -1.0
    rc, word, hits, inst = _trace_raw(scene, rays, L.NB_TRACE_ANY)
    assert rc == L.NB_ERR_STACK_OVERFLOW and word & 1
    assert np.all(hits[:, 0] != NO_HIT) and np.all(hits[:, 3].view(np.uint32) < n_tris) and np.all(inst < 8192)
    rc, word, hits, inst = _trace_raw(scene, rays[:32], 0)
    assert rc == L.NB_ERR_STACK_OVERFLOW and word == 3  # both bits: overflow and iteration cap
    assert np.all(hits[:, 0] != NO_HIT) and np.all(hits[:, 3].view(np.uint32) < n_tris) and np.all(inst < 8192)
    away = rays.copy()
    away[:, 6] = 1.0  # pointing away from everything
    rc, word, hits, _ = _trace_raw(scene, away, 0)
    assert rc == L.NB_OK and word == 0 and np.all(hits[:, 0] == NO_HIT)

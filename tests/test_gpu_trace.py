"""Traversal parity: the CUDA intersect_scene query against the oracle's restatement of
raytracing_sw.wgsl on the same seeded rays and the same trees.

Bar (from the pass's parity spec): hit triangle/instance ids bit-exact except documented
near-ties; t and barycentrics within 1e-5 relative.  A near-tie is a ray whose two answers
lie within 1e-5 relative in t (two triangles the ray meets at the same distance, e.g. on a
shared edge, resolved by a different traversal order).
"""
import numpy as np
import pytest

import nbounce_gb300 as nb
from nbounce_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NO_HIT = np.float32(3.4028234663852886e38)
REL_TOL = 1e-5


def compare_hits(gpu_hits, gpu_inst, perm_indices, ref_f, ref_u, max_tie_frac=1e-3):
    g_t = gpu_hits[:, 0]
    r_t = ref_f[:, 0]
    g_hit = g_t != NO_HIT
    r_hit = r_t != NO_HIT
    tri = gpu_hits[:, 3].view(np.uint32)
    idx3 = perm_indices.reshape(-1, 3)
    g_ids = np.full((len(g_t), 3), 0xFFFFFFFF, np.uint32)
    g_ids[g_hit] = idx3[tri[g_hit]]
    same = (g_hit == r_hit)
    both = g_hit & r_hit
    same[both] = np.all(g_ids[both] == ref_u[both, 1:], axis=1) & (gpu_inst[both] == ref_u[both, 0])
    mism = ~same
    # every mismatch must be a near-tie
    t_a = np.where(g_hit, g_t, np.inf).astype(np.float64)
    t_b = np.where(r_hit, r_t, np.inf).astype(np.float64)
    with np.errstate(invalid="ignore"):
        tie = np.abs(t_a - t_b) <= REL_TOL * np.minimum(t_a, t_b)
    assert np.all(tie[mism]), f"{int(np.sum(mism & ~tie))} non-tie mismatches"
    assert mism.mean() <= max_tie_frac, f"near-tie fraction {mism.mean():.2e}"
    ok = both & same
    np.testing.assert_allclose(g_t[ok], r_t[ok], rtol=REL_TOL)
    np.testing.assert_allclose(gpu_hits[ok, 1:3], ref_f[ok, 1:3], rtol=REL_TOL, atol=REL_TOL)
    return int(mism.sum()), int(both.sum())


@pytest.fixture(scope="module")
def soup():
    desc = scenes.soup_scene(20000, seed=11)
    gpu = nb.SceneBuffers.from_desc(desc, dedup=True)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    return desc, gpu, orc


@pytest.mark.parametrize("kind", ["coherent", "incoherent"])
def test_soup_closest_hit_matches_oracle(soup, kind):
    desc, gpu, orc = soup
    rays = scenes.coherent_rays(128, 96) if kind == "coherent" else scenes.incoherent_rays(20000, seed=5)
    hits, inst = gpu.trace_host(rays)
    rf, ru, cnt = orc.trace(rays)
    assert cnt[:, 3].max() == 0
    ties, both = compare_hits(hits, inst, gpu.export()["indices"], rf, ru)
    assert both > 500


def test_soup_any_hit_agrees_on_occlusion(soup):
    desc, gpu, orc = soup
    rays = scenes.incoherent_rays(20000, seed=6)
    any_hits, _ = gpu.trace_host(rays, any_hit=True)
    closest, _ = gpu.trace_host(rays)
    rf, _, _ = orc.trace(rays, any_hit=True)
    g_occ = any_hits[:, 0] != NO_HIT
    assert np.array_equal(g_occ, closest[:, 0] != NO_HIT)
    assert np.array_equal(g_occ, rf[:, 0] != NO_HIT)
    # an any-hit answer is a real hit: never closer than the closest one
    assert np.all(any_hits[g_occ, 0] >= closest[g_occ, 0])


def test_instanced_scene_primary_rays_match(tmp_path):
    desc = scenes.spheres_scene(width=96, height=96)
    sob = nb.sobol_burley_table()
    for dedup in (True, False):
        gpu = nb.SceneBuffers.from_desc(desc, dedup=dedup)
        orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=dedup)
        rays = O.primary_rays(desc.clip_to_world, desc.width, desc.height, sob, 1)
        hits, inst = gpu.trace_host(rays)
        rf, ru, _ = orc.trace(rays)
        compare_hits(hits, inst, gpu.export()["indices"], rf, ru)


def test_scene_from_reference_buffers_traces_identically():
    desc = scenes.spheres_scene(width=64, height=64)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=False)
    gpu = nb.SceneBuffers.from_bvh(orc.blas, orc.tlas, orc.instances, orc.vertices, orc.indices)
    rays = scenes.incoherent_rays(8000, seed=9) * np.array([12, 12, 12, 0, 1, 1, 1, 0], np.float32)
    hits, inst = gpu.trace_host(rays)
    rf, ru, _ = orc.trace(rays)
    compare_hits(hits, inst, orc.indices, rf, ru)


def test_empty_query_and_miss_everything(soup):
    desc, gpu, orc = soup
    hits, inst = gpu.trace_host(np.zeros((0, 8), np.float32))
    assert hits.shape == (0, 4)
    away = np.zeros((64, 8), np.float32)
    away[:, :3] = [5.0, 5.0, 5.0]
    away[:, 4:7] = [1.0, 0.0, 0.0]
    hits, inst = gpu.trace_host(away)
    assert np.all(hits[:, 0] == NO_HIT) and np.all(inst == 0xFFFFFFFF)


def test_axis_aligned_and_surface_origin_rays_match_oracle(soup):
    """Directions with exactly-zero components (the box test nudges 1/0 to a large finite
    reciprocal, the triangle test uses the true direction) and rays that start on a triangle
    (rejected by BIAS = 0.1, raytracing_sw.wgsl:4,76) against the oracle."""
    desc, gpu, orc = soup
    rng = np.random.default_rng(21)
    n = 6000
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = rng.uniform(-1.2, 1.2, (n, 3))
    axis = rng.integers(0, 3, n)
    sign = np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0)
    rays[np.arange(n), 4 + axis] = sign
    # a third of the rays start at a triangle's centroid, in a random direction
    idx = desc.indices.reshape(-1, 3)
    pos = desc.vertices["pos"]
    k = n // 3
    t = rng.integers(0, len(idx), k)
    rays[:k, :3] = pos[idx[t]].mean(axis=1)
    d = rng.normal(size=(k, 3))
    rays[:k, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    hits, inst = gpu.trace_host(rays)
    rf, ru, cnt = orc.trace(rays)
    assert cnt[:, 3].max() == 0
    ties, both = compare_hits(hits, inst, gpu.export()["indices"], rf, ru)
    assert both > 200
    assert np.all(hits[:, 0][hits[:, 0] != NO_HIT] >= 0.1)


def test_small_large_and_power_of_two_direction_components_match_oracle(soup):
    """The box test takes its reciprocal directions from the hardware's approximate reciprocal
    and covers that rounding by per-axis plane margins; the triangle test divides exactly.
    Directions (not normalised: the query takes any direction) whose components sit around the
    1e-20 nudge, far below the others, at exact powers of two, or spread over 16 decades find
    the oracle's closest hits."""
    desc, gpu, orc = soup
    rng = np.random.default_rng(33)
    n = 8000
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = rng.uniform(-1.2, 1.2, (n, 3))
    d = rng.normal(size=(n, 3))
    rows = np.arange(n)
    small = np.array([1e-21, 9.9e-21, 1e-20, 1.01e-20, 1e-19, 2.0 ** -60, 1e-12, 1e-6])
    which = rng.integers(0, 3, n)
    d[rows, which] = np.where(d[rows, which] < 0, -1.0, 1.0) * small[rng.integers(0, len(small), n)]
    q = n // 4  # exact powers of two, whose reciprocals are exact
    d[:q] = np.where(d[:q] < 0, -1.0, 1.0) * 2.0 ** rng.integers(-10, 11, (q, 3))
    e = n // 8  # components spread over 16 decades
    d[q:q + e] *= 10.0 ** rng.integers(-8, 9, (e, 3))
    rays[:, 4:7] = d
    assert np.all(np.isfinite(rays))
    hits, inst = gpu.trace_host(rays)
    rf, ru, cnt = orc.trace(rays)
    assert cnt[:, 3].max() == 0
    ties, both = compare_hits(hits, inst, gpu.export()["indices"], rf, ru)
    assert both > 300  # 480 of the 8000 rays hit the sparse soup


def test_non_finite_rays_hit_nothing(soup):
    """Rays with a NaN or infinite origin or direction component meet nothing, as in the
    oracle (every slab and triangle comparison of the reference fails on NaN); finite rays
    in the same query are unaffected."""
    desc, gpu, orc = soup
    rng = np.random.default_rng(33)
    n = 512
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = rng.uniform(-0.5, 0.5, (n, 3)) + np.float32([0.0, 0.0, -3.0])
    rays[:, 4:7] = rng.normal(0.0, 0.05, (n, 3)) + np.float32([0.0, 0.0, 1.0])
    bad = np.arange(n) % 2 == 0
    comp = rng.integers(0, 6, n)
    vals = np.array([np.nan, np.inf, -np.inf], np.float32)[rng.integers(0, 3, n)]
    cols = np.where(comp < 3, comp, comp + 1)
    rays[bad, cols[bad]] = vals[bad]
    hits, inst = gpu.trace_host(rays)
    rf, ru, _ = orc.trace(rays)
    assert np.all(hits[bad, 0] == NO_HIT) and np.all(inst[bad] == 0xFFFFFFFF)
    assert np.all(rf[bad, 0] == NO_HIT)
    good = ~bad
    assert np.sum(rf[good, 0] != NO_HIT) > 25  # 51 of the 256 finite rays meet the soup
    compare_hits(hits[good], inst[good], gpu.export()["indices"], rf[good], ru[good])


def test_large_instance_split_into_tlas_entries_traces_like_the_oracle():
    """The terrain of the instanced scene covers most of the scene, so the device TLAS enters
    it once per child of its BLAS root (partial re-braiding) with tight world boxes; rays
    grazing it and rays from above must find the oracle's closest hits (the oracle traverses
    the reference TLAS over the transformed root boxes)."""
    desc = scenes.instanced_scene(scale=1 / 64, n_instances=96, width=64, height=64, env_size=(16, 8))
    gpu = nb.SceneBuffers.from_desc(desc)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    rng = np.random.default_rng(8)
    n = 20000
    rays = np.zeros((n, 8), np.float32)
    half = n // 2
    # from above, toward the terrain and the instances
    rays[:half, :3] = rng.uniform([-40, 20, -40], [40, 30, 40], (half, 3))
    d = rng.normal(size=(half, 3)) * [0.4, 1.0, 0.4]
    d[:, 1] = -np.abs(d[:, 1])
    rays[:half, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    # grazing: just above the terrain's level, nearly horizontal
    rays[half:, :3] = rng.uniform([-40, -11.5, -40], [40, -8.0, 40], (n - half, 3))
    g = rng.normal(size=(n - half, 3)) * [1.0, 0.05, 1.0]
    rays[half:, 4:7] = g / np.linalg.norm(g, axis=1, keepdims=True)
    hits, inst = gpu.trace_host(rays)
    rf, ru, _ = orc.trace(rays)
    assert gpu.info()["n_tlas_entries"] > len(desc.instances)  # the terrain was split
    ties, both = compare_hits(hits, inst, gpu.export()["indices"], rf, ru)
    assert both > n // 4

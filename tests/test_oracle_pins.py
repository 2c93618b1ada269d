"""Pins of the CPU oracle against sources independent of it.

The reference has no tests or golden vectors, so each piece of the oracle is pinned
against something outside it: SciPy's unscrambled Sobol generator (direction numbers),
an independent numpy evaluation of PCG4D / map4f (common.wgsl:7-41), float64 sin/cos
(error bound of the deterministic sin/cos), the (0,m,2)-net structure Owen scrambling
must preserve, and bvh.rs's structural invariants.  The regression fixture in
tests/golden/oracle_golden.npz (made by tests/golden/make_golden.py) pins the oracle's
outputs bit for bit.
"""
import os

import numpy as np
import pytest

from nbounce_gb300 import scenes
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_sobol_direction_numbers_match_committed_fixture():
    ref = np.load(os.path.join(GOLDEN, "sobol_unscrambled_68x256.npy"))
    got = np.array([[O.sobol_u32(i, d) for d in range(68)] for i in range(256)], np.uint32)
    assert np.array_equal(got, ref)


def test_sobol_direction_numbers_match_scipy():
    qmc = pytest.importorskip("scipy.stats").qmc
    n = 1024
    eng = qmc.Sobol(d=68, scramble=False, bits=32)
    ref = (eng.random(n) * 2.0 ** 32).astype(np.uint64).astype(np.uint32)
    gray = np.arange(n) ^ (np.arange(n) >> 1)
    got = np.array([[O.sobol_u32(int(g), d) for d in range(68)] for g in gray], np.uint32)
    assert np.array_equal(got, ref)


def pcg4d_numpy(s):
    v = (np.asarray(s, np.uint64) * 1664525 + 1013904223) & 0xFFFFFFFF
    m = 0xFFFFFFFF

    def mix(v):
        v = v.copy()
        v[0] = (v[0] + v[1] * v[3]) & m
        v[1] = (v[1] + v[2] * v[0]) & m
        v[2] = (v[2] + v[0] * v[1]) & m
        v[3] = (v[3] + v[1] * v[2]) & m
        return v

    v = mix(v)
    v ^= v >> 16
    return mix(v).astype(np.uint32)


@pytest.mark.parametrize("xy", [(0, 0), (1, 2), (255, 255), (1919, 1079), (123456, 7)])
def test_pcg4d_and_map4f_match_independent_numpy(xy):
    s = [xy[0], xy[1], xy[0], xy[1]]
    h = pcg4d_numpy(s)
    assert np.array_equal(O.hash4u(s), h)
    f = ((h >> 9) | np.uint32(0x3F800000)).view(np.float32) - np.float32(1.0)
    assert np.array_equal(O.hash4f(s), f)
    assert np.all((f >= 0) & (f < 1))


def test_sincos_error_bound():
    x = np.linspace(-3.3, 6.5, 400001).astype(np.float32)
    s, c = O.sincos(x)
    xs = x.astype(np.float64)
    assert np.max(np.abs(s - np.sin(xs))) < 1.5e-7
    assert np.max(np.abs(c - np.cos(xs))) < 1.5e-7
    assert np.all(np.abs(s) <= 1.0) and np.all(np.abs(c) <= 1.0)


def test_sobol_table_is_stratified_per_dimension_and_net_in_pairs():
    t = O.sobol_table(1024, 17)
    assert t.dtype == np.float32 and np.all((t >= 0) & (t < 1))
    pts = t.reshape(1024, 68)
    for m in (4, 6, 8, 10):
        n = 1 << m
        for d in range(68):  # every coordinate is a (0,1)-sequence: one point per 1/n interval
            cells = np.floor(pts[:n, d] * n).astype(np.int64)
            assert np.array_equal(np.sort(cells), np.arange(n)), (m, d)
        raw = np.array([[O.sobol_u32(i, d) for d in range(68)] for i in range(n)], np.float64) / 2.0 ** 32
        for d in range(0, 68, 2):
            # nested uniform scrambling maps elementary intervals onto elementary intervals, so
            # each dimension pair keeps the interval counts of the unscrambled points; pair (0,1)
            # is a (0,m,2)-net (one point per interval)
            for k in range(m + 1):
                def counts(p):
                    cx = np.floor(p[:n, d] * (1 << k)).astype(np.int64)
                    cy = np.floor(p[:n, d + 1] * (1 << (m - k))).astype(np.int64)
                    return np.sort(np.bincount(cx * (1 << (m - k)) + cy, minlength=n))
                assert np.array_equal(counts(pts), counts(raw)), (m, d, k)
                if d == 0:
                    assert counts(pts).max() == 1, (m, k)


def test_sobol_table_is_scrambled_and_seeded():
    a = O.sobol_table(64, 17, seed=0)
    b = O.sobol_table(64, 17, seed=1)
    assert not np.array_equal(a, b)
    # Owen scrambling moves the unscrambled origin point away from 0
    assert np.all(a[0] != 0.0)


def check_bvh_invariants(nodes, positions, perm, root=0, n_prims=None):
    tri = positions[perm.reshape(-1, 3)]
    lo, hi = tri.min(axis=1), tri.max(axis=1)
    covered = np.zeros(len(tri), np.int64)
    stack = [(root, 0)]
    max_depth = 0
    while stack:
        i, d = stack.pop()
        max_depth = max(max_depth, d)
        n = nodes[i]
        if n["end"] > 0:
            s, e = int(n["start"]), int(n["end"])
            assert e > s
            covered[s:e] += 1
            assert np.all(lo[s:e] >= n["min"]) and np.all(hi[s:e] <= n["max"])
        else:
            c = int(n["start"])
            for k in (c, c + 1):
                assert np.all(nodes[k]["min"] >= n["min"]) and np.all(nodes[k]["max"] <= n["max"])
                stack.append((k, d + 1))
    assert np.all(covered == 1)
    assert max_depth <= 32
    return max_depth


@pytest.mark.parametrize("n", [1, 2, 3, 5, 11, 12, 13, 100, 3000])
def test_bvh_invariants_random_soup(n):
    v, f = scenes.triangle_soup(n, seed=n)
    nodes, perm = O.bvh_build_triangles(v["pos"], f)
    check_bvh_invariants(nodes, v["pos"], perm)
    assert sorted(map(tuple, perm.reshape(-1, 3))) == sorted(map(tuple, f))


def test_bvh_depth_cap_and_coincident_centroids():
    # identical triangles cannot be split (every split has an empty side): one leaf
    p = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    f = np.tile(np.arange(3, dtype=np.uint32), (40, 1))
    nodes, perm = O.bvh_build_triangles(p, f)
    assert len(nodes) == 1 and nodes[0]["end"] == 40
    # a long chain of nested slivers exercises the MAX_DEPTH = 32 cut-off
    k = 80
    s = (2.0 ** -np.arange(k)).astype(np.float32)
    pos = np.stack([np.stack([s * 0, s * 0, s * 0], 1), np.stack([s, s * 0, s * 0], 1),
                    np.stack([s * 0, s, s * 0], 1)], 1).reshape(-1, 3)
    f = np.arange(3 * k, dtype=np.uint32).reshape(-1, 3)
    nodes, perm = O.bvh_build_triangles(pos, f)
    check_bvh_invariants(nodes, pos, perm)


def test_oracle_matches_committed_golden_outputs():
    g = np.load(os.path.join(GOLDEN, "oracle_golden.npz"))
    t = O.sobol_table(32, 17)
    assert np.array_equal(t.view(np.uint32), g["sobol32"].view(np.uint32))
    desc = scenes.soup_scene(2000, seed=21)
    osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    hf, hu, _ = osc.trace(scenes.incoherent_rays(4000, seed=22))
    assert np.array_equal(hf.view(np.uint32), g["soup_hits_f"].view(np.uint32))
    assert np.array_equal(hu, g["soup_hits_u"])
    sph = scenes.spheres_scene(width=24, height=24)
    osc = O.OracleScene(sph.vertices, sph.indices, sph.primitives(), dedup=True)
    img, rays, _, _ = osc.render(sph.clip_to_world, 24, 24, O.sobol_table(1024, 17), 1, 4, bounces=6,
                                 env=sph.env_color)
    assert np.array_equal(img.view(np.uint32), g["spheres24_4spp"].view(np.uint32))
    assert rays == int(g["spheres24_rays"])

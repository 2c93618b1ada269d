"""The library's host side against the oracle, bit for bit, without a GPU.

nb_bvh_build and nb_scene_create(NB_SCENE_HOST_ONLY) reproduce bvh.rs and
SceneBuffers::from_scene (scene.rs:280-305): node arrays, TLAS-permuted instances and the
triangle-permuted index buffer must equal the oracle's exactly, in both the per-primitive
(reference) mode and the one-BLAS-per-mesh mode.
"""
import numpy as np
import pytest

import nbounce_gb300 as nb
from nbounce_gb300 import scenes
from oracle import oracle as O


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("maker", ["soup1", "soup2", "soup3", "soup11", "soup12", "soup5000", "ico4", "hf48",
                                   "coincident", "grid_ties", "soup300000", "hf256"])
def test_bvh_build_bit_exact(maker):
    """The two large cases split their top levels on several threads and the ranges below
    sequentially into flat arrays spliced into the reference numbering."""
    rng = np.random.default_rng(7)
    if maker.startswith("soup"):
        v, f = scenes.triangle_soup(int(maker[4:]), seed=3)
        pos = v["pos"]
    elif maker == "ico4":
        pos, f = scenes.icosphere(4)
    elif maker in ("hf48", "hf256"):
        v, f = scenes.heightfield(int(maker[2:]), rng)
        pos = v["pos"]
    elif maker == "coincident":
        pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
        f = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]] * 7, np.uint32)
    else:  # a flat regular grid: many equal SAH costs
        v, f = scenes.heightfield(33, rng, amount=0.0)
        pos = v["pos"]
    a_nodes, a_perm = nb.bvh_build(pos, f)
    b_nodes, b_perm = O.bvh_build_triangles(pos, f)
    assert np.array_equal(bits(a_nodes), bits(b_nodes))
    assert np.array_equal(a_perm, b_perm)


@pytest.mark.parametrize("dedup", [False, True])
def test_scene_assembly_bit_exact_spheres(dedup):
    desc = scenes.spheres_scene()
    ours = nb.SceneBuffers.from_desc(desc, dedup=dedup, host_only=True).export()
    ref = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=dedup)
    for k, r in (("blas", ref.blas), ("tlas", ref.tlas), ("instances", ref.instances), ("indices", ref.indices)):
        assert np.array_equal(bits(ours[k]), bits(r)), k


def test_scene_assembly_bit_exact_instanced_small():
    desc = scenes.instanced_scene(n_instances=200, width=64, height=36, env_size=(64, 32), scale=1 / 64)
    ours = nb.SceneBuffers.from_desc(desc, dedup=True, host_only=True)
    ex = ours.export()
    ref = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    for k, r in (("blas", ref.blas), ("tlas", ref.tlas), ("instances", ref.instances), ("indices", ref.indices)):
        assert np.array_equal(bits(ex[k]), bits(r)), k
    info = ours.info()
    used = len({i["mesh"] for i in desc.instances})
    assert info["n_blas_roots"] == used and info["n_instances"] == 200


def test_reference_mode_reproduces_shared_mesh_rebuild():
    """scene.rs:285-299 appends one BLAS per primitive.  Rebuilding a shared range is not
    idempotent (brute-force SAH cost ties pick another split once the triangles are permuted),
    so the first BLAS of a shared mesh goes stale against the final index buffer.  Both sides
    reproduce that, and the one-BLAS-per-mesh mode does not have it."""
    desc = scenes.spheres_scene()
    ref = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=False)
    pos = desc.vertices["pos"]

    def stale_leaves(blas, indices, root):
        tri = pos[indices.reshape(-1, 3)]
        lo, hi = tri.min(axis=1), tri.max(axis=1)
        bad, stack = 0, [root]
        while stack:
            n = blas[stack.pop()]
            if n["end"] > 0:
                s, e = int(n["start"]), int(n["end"])
                bad += int(np.any(lo[s:e] < n["min"] - 1e-6) or np.any(hi[s:e] > n["max"] + 1e-6))
            else:
                stack += [int(n["start"]), int(n["start"]) + 1]
        return bad

    first_root = int(ref.instances["node"].min())
    assert stale_leaves(ref.blas, ref.indices, first_root) > 0
    ded = nb.SceneBuffers.from_desc(desc, dedup=True, host_only=True).export()
    assert all(stale_leaves(ded["blas"], ded["indices"], int(r)) == 0 for r in set(ded["instances"]["node"]))


def test_world_to_local_is_derived_when_absent():
    desc = scenes.spheres_scene()
    prims = desc.primitives()
    for p in prims:
        p["w2l"] = np.zeros((4, 4), np.float32)
    ex = nb.SceneBuffers.from_scene(desc.vertices, desc.indices, prims, host_only=True).export()
    w2l = ex["instances"]["w2l"].reshape(-1, 4, 4).transpose(0, 2, 1)
    l2w = ex["instances"]["l2w"].reshape(-1, 4, 4).transpose(0, 2, 1)
    eye = np.einsum("nij,njk->nik", w2l.astype(np.float64), l2w.astype(np.float64))
    assert np.allclose(eye, np.eye(4), atol=1e-5)


def test_invalid_inputs_are_rejected_with_codes():
    desc = scenes.spheres_scene()
    bad = desc.indices.copy()
    bad[5] = len(desc.vertices) + 3
    with pytest.raises(nb.NbError) as e:
        nb.SceneBuffers.from_scene(desc.vertices, bad, desc.primitives(), host_only=True)
    assert e.value.status == 1 and "out of range" in str(e.value)
    prims = desc.primitives()
    prims[0]["index_end"] = prims[0]["index_start"]
    with pytest.raises(nb.NbError) as e:
        nb.SceneBuffers.from_scene(desc.vertices, desc.indices, prims, host_only=True)
    assert e.value.status == 1
    prims = desc.primitives()
    prims[0]["l2w"] = np.zeros((4, 4), np.float32)
    prims[0]["w2l"] = np.zeros((4, 4), np.float32)
    with pytest.raises(nb.NbError) as e:
        nb.SceneBuffers.from_scene(desc.vertices, desc.indices, prims, host_only=True)
    assert "singular" in str(e.value)


def test_host_only_scene_cannot_render_or_trace():
    desc = scenes.soup_scene(50)
    s = nb.SceneBuffers.from_desc(desc, host_only=True)
    with pytest.raises(nb.NbError) as e:
        s.trace_host(np.zeros((4, 8), np.float32))
    assert e.value.status == 1


def test_sobol_table_product_equals_oracle():
    a = nb.sobol_burley_table(1024, 17, seed=0)
    b = O.sobol_table(1024, 17, seed=0)
    assert np.array_equal(bits(a), bits(b))
    a = nb.sobol_burley_table(16, 17, seed=12345)
    b = O.sobol_table(16, 17, seed=12345)
    assert np.array_equal(bits(a), bits(b))
    with pytest.raises(nb.NbError):
        nb.sobol_burley_table(4, 18)


def test_output_size_rule():
    assert nb.Pathtracer.output_size(1920, 1080, 0.3) == (576, 320)
    assert nb.Pathtracer.output_size(1920, 1080, 1.0) == (1920, 1080)


def test_device_tlas_splits_only_large_instances():
    """Device TLAS entries (host-only build): every instance enters once, except instances whose
    box exceeds 2% of the scene's box area and whose BLAS root has only inner children - the
    instanced scene's 45x terrain - which enter once per child of that root."""
    spheres = scenes.spheres_scene(width=16, height=16)
    s = nb.SceneBuffers.from_desc(spheres, host_only=True).info()
    assert s["n_tlas_entries"] == s["n_instances"]
    desc = scenes.instanced_scene(scale=1 / 64, n_instances=96, width=16, height=16, env_size=(16, 8))
    i = nb.SceneBuffers.from_desc(desc, host_only=True).info()
    assert i["n_instances"] < i["n_tlas_entries"] <= i["n_instances"] + 7 * 4

"""GLB ingest (Scene::parse_gltf, scene.rs:108-217).

The reference's own scenes (assets/spheres.glb, assets/testscene.glb) are parsed when the
directory holding them is named by the NB_REFERENCE_ASSETS environment variable (a CPU test;
it skips without it); a generated scene is
round-tripped through write_glb/parse_glb everywhere, and the MeshError cases are checked.
"""
import json
import os
import struct

import numpy as np
import pytest

import nbounce_gb300 as nb
from nbounce_gb300 import gltf, scenes
from oracle import oracle as O

REF_ASSETS = os.environ.get("NB_REFERENCE_ASSETS", "")


def asset(name):
    p = os.path.join(REF_ASSETS, name) if REF_ASSETS else ""
    if not p or not os.path.exists(p):
        pytest.skip("NB_REFERENCE_ASSETS does not name the reference's assets directory")
    return p


def test_reference_spheres_glb():
    d = gltf.load_glb(asset("spheres.glb"))
    assert len(d.meshes) == 15 and len(d.instances) == 15
    assert all((e - s) // 3 == 1280 for s, e in d.meshes)
    rough = sorted({round(float(i["roughness"]), 2) for i in d.instances})
    metal = sorted({round(float(i["metallic"]), 2) for i in d.instances})
    assert rough == [0.0, 0.25, 0.5, 0.75, 1.0] and metal == [0.0, 0.5, 1.0]
    assert all(np.allclose(i["color"], [1, 0, 0, 1]) for i in d.instances)
    # the library and the oracle assemble identical reference buffers from it
    ours = nb.SceneBuffers.from_desc(d, dedup=False, host_only=True).export()
    ref = O.OracleScene(d.vertices, d.indices, d.primitives(), dedup=False)
    for k, r in (("blas", ref.blas), ("tlas", ref.tlas), ("instances", ref.instances), ("indices", ref.indices)):
        assert np.array_equal(ours[k].view(np.uint32), r.view(np.uint32)), k


def test_reference_testscene_glb_renders_on_the_oracle():
    d = gltf.load_glb(asset("testscene.glb"), width=32, height=32)
    tris = sorted((e - s) // 3 for s, e in d.meshes)
    assert tris == [12, 960, 15744, 15744]
    ref = O.OracleScene(d.vertices, d.indices, d.primitives(), dedup=True)
    img, rays, _, _ = ref.render(d.clip_to_world, 32, 32, O.sobol_table(1024, 17), 1, 1, bounces=4)
    assert np.isfinite(img).all() and rays >= 32 * 32


def test_round_trip_of_a_generated_scene():
    desc = scenes.instanced_scene(n_instances=12, width=32, height=18, env_size=(16, 8), scale=1 / 256)
    # one instance per mesh so that per-primitive materials survive the round trip
    seen, insts = set(), []
    for inst in desc.instances:
        if inst["mesh"] not in seen:
            seen.add(inst["mesh"])
            insts.append(inst)
    desc.instances = insts
    back = gltf.parse_glb(gltf.write_glb(desc))
    assert len(back.instances) == len(insts)
    for a, b in zip(insts, back.instances):
        s0, e0 = desc.meshes[a["mesh"]]
        s1, e1 = back.meshes[b["mesh"]]
        va = desc.vertices[desc.indices[s0:e0]]
        vb = back.vertices[back.indices[s1:e1]]
        assert np.array_equal(va["pos"], vb["pos"]) and np.array_equal(va["tan"], vb["tan"])
        np.testing.assert_allclose(b["l2w"], a["l2w"], rtol=0, atol=0)
        assert float(b["roughness"]) == float(a["roughness"]) and float(b["emissive"]) == float(a["emissive"])


def _minimal_glb(attrs=("POSITION", "NORMAL", "TANGENT"), mode=4, with_indices=True):
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    data = {"POSITION": pos, "NORMAL": np.tile([0, 0, 1.0], (3, 1)).astype(np.float32),
            "TANGENT": np.tile([1.0, 0, 0, 1], (3, 1)).astype(np.float32)}
    bin_ = b""
    views, accs, attr_js = [], [], {}
    for name in attrs:
        a = data[name]
        views.append({"buffer": 0, "byteOffset": len(bin_), "byteLength": a.nbytes})
        accs.append({"bufferView": len(views) - 1, "componentType": 5126, "count": 3,
                     "type": "VEC3" if a.shape[1] == 3 else "VEC4"})
        attr_js[name] = len(accs) - 1
        bin_ += a.tobytes()
    prim = {"attributes": attr_js, "mode": mode}
    if with_indices:
        ind = np.array([0, 1, 2], np.uint32)
        views.append({"buffer": 0, "byteOffset": len(bin_), "byteLength": ind.nbytes})
        accs.append({"bufferView": len(views) - 1, "componentType": 5125, "count": 3, "type": "SCALAR"})
        prim["indices"] = len(accs) - 1
        bin_ += ind.tobytes()
    js = {"asset": {"version": "2.0"}, "buffers": [{"byteLength": len(bin_)}], "bufferViews": views,
          "accessors": accs, "meshes": [{"primitives": [prim]}], "nodes": [{"mesh": 0}]}
    jb = json.dumps(js).encode()
    jb += b" " * ((-len(jb)) % 4)
    body = struct.pack("<II", len(jb), 0x4E4F534A) + jb + struct.pack("<II", len(bin_), 0x004E4942) + bin_
    return struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body


def test_minimal_glb_parses_with_default_texcoords():
    d = gltf.parse_glb(_minimal_glb())
    assert len(d.vertices) == 3 and np.all(d.vertices["u"] == 0) and np.all(d.vertices["v"] == 0)
    assert float(d.instances[0]["metallic"]) == 1.0 and float(d.instances[0]["roughness"]) == 1.0


@pytest.mark.parametrize("kw,kind", [(dict(attrs=("NORMAL", "TANGENT")), "MissingPositions"),
                                     (dict(attrs=("POSITION", "TANGENT")), "MissingNormals"),
                                     (dict(attrs=("POSITION", "NORMAL")), "MissingTangents"),
                                     (dict(mode=1), "NotTriangleList"),
                                     (dict(with_indices=False), "MissingIndices")])
def test_mesh_errors(kw, kind):
    with pytest.raises(gltf.MeshError) as e:
        gltf.parse_glb(_minimal_glb(**kw))
    assert e.value.kind == kind


def test_not_a_glb():
    with pytest.raises(gltf.MeshError):
        gltf.parse_glb(b"not a glb file at all")

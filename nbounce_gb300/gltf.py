"""Binary glTF (.glb) ingest producing the scene the pass consumes.

Restates ``Scene::parse_gltf`` (reference ``src/pathtracing/scene.rs:108-217``) without the
gltf crate: the GLB container (12-byte header, JSON chunk, BIN chunk), accessors and buffer
views are decoded here with numpy.  Rules kept from the reference:

* every mesh primitive must be a triangle list (mode 4), else ``MeshError.NotTriangleList``;
* POSITION and NORMAL are required (``MissingPositions`` / ``MissingNormals``), TANGENT too
  (``MissingTangents``: the reference does not generate tangents), TEXCOORD_0 defaults to 0;
* indices are required (``MissingIndices``) and rebased to global vertex ids (scene.rs:173);
* meshes are processed first, in order, then every node with a mesh adds one primitive per
  mesh primitive with the node's local transform (``node.transform().matrix()``: the node's
  own matrix or TRS, not composed with parents - as the reference does);
* a material with a nonzero emissive factor becomes emissive: colour = (emissive, 1),
  emissive = 1 (scene.rs:190-197); defaults follow glTF (base colour 1, metallic 1,
  roughness 1).

Only embedded BIN-chunk buffers are supported (the reference's assets are self-contained GLBs).
"""
import json
import struct

import numpy as np

from .scenes import VERTEX_DTYPE, SceneDesc


class MeshError(ValueError):
    """Mirrors the reference's MeshError (scene.rs:69-98)."""

    def __init__(self, kind, detail=""):
        super().__init__(f"{kind}{': ' + detail if detail else ''}")
        self.kind = kind


_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}


def read_glb(data):
    """(json dict, bin bytes) of a GLB file's contents."""
    if len(data) < 20:
        raise MeshError("Gltf", "file too short")
    magic, version, length = struct.unpack_from("<III", data, 0)
    if magic != 0x46546C67 or version != 2:
        raise MeshError("Gltf", "not a glTF 2.0 binary")
    off, js, bin_ = 12, None, b""
    while off + 8 <= min(length, len(data)):
        clen, ctype = struct.unpack_from("<II", data, off)
        chunk = data[off + 8: off + 8 + clen]
        if ctype == 0x4E4F534A:
            js = json.loads(chunk.decode("utf-8"))
        elif ctype == 0x004E4942:
            bin_ = bytes(chunk)
        off += 8 + clen
    if js is None:
        raise MeshError("Gltf", "missing JSON chunk")
    return js, bin_


def _accessor(js, bin_, idx):
    acc = js["accessors"][idx]
    view = js["bufferViews"][acc["bufferView"]]
    if view.get("buffer", 0) != 0:
        raise MeshError("Gltf", "only the embedded buffer is supported")
    dtype = np.dtype(_COMPONENT[acc["componentType"]])
    n = _NCOMP[acc["type"]]
    count = acc["count"]
    start = view.get("byteOffset", 0) + acc.get("byteOffset", 0)
    stride = view.get("byteStride", 0) or dtype.itemsize * n
    raw = np.frombuffer(bin_, dtype=np.uint8, count=stride * (count - 1) + dtype.itemsize * n, offset=start)
    rows = np.lib.stride_tricks.as_strided(raw, shape=(count, dtype.itemsize * n), strides=(stride, 1))
    out = np.ascontiguousarray(rows).view(dtype).reshape(count, n)
    if acc.get("normalized") and dtype.kind in "iu":
        out = out.astype(np.float32) / np.float32(np.iinfo(dtype).max)
    return out


def _node_matrix(node):
    if "matrix" in node:
        return np.array(node["matrix"], np.float64).reshape(4, 4).T  # column-major in glTF
    t = np.array(node.get("translation", [0, 0, 0]), np.float64)
    x, y, z, w = node.get("rotation", [0, 0, 0, 1])
    s = np.array(node.get("scale", [1, 1, 1]), np.float64)
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    m = np.eye(4)
    m[:3, :3] = r * s[None, :]
    m[:3, 3] = t
    return m


def parse_glb(data, width=256, height=256, spp=16, bounces=8, camera=None, env_color=(0.5, 0.6, 0.8)):
    """Scene::parse_gltf on GLB bytes -> SceneDesc (one mesh entry per glTF mesh primitive)."""
    js, bin_ = read_glb(data)
    verts, idx, meshes = [], [], []
    prim_range = {}
    nv = ni = 0
    for mi, mesh in enumerate(js.get("meshes", [])):
        for pi, prim in enumerate(mesh["primitives"]):
            if prim.get("mode", 4) != 4:
                raise MeshError("NotTriangleList")
            attr = prim["attributes"]
            if "POSITION" not in attr:
                raise MeshError("MissingPositions")
            if "NORMAL" not in attr:
                raise MeshError("MissingNormals")
            pos = _accessor(js, bin_, attr["POSITION"]).astype(np.float32)
            nrm = _accessor(js, bin_, attr["NORMAL"]).astype(np.float32)
            uv = (_accessor(js, bin_, attr["TEXCOORD_0"]).astype(np.float32) if "TEXCOORD_0" in attr
                  else np.zeros((len(pos), 2), np.float32))
            if "TANGENT" not in attr:
                raise MeshError("MissingTangents", "Tangent generation is not yet supported")
            tan = _accessor(js, bin_, attr["TANGENT"]).astype(np.float32)
            if "indices" not in prim:
                raise MeshError("MissingIndices")
            ind = _accessor(js, bin_, prim["indices"]).astype(np.uint32).ravel()
            v = np.zeros(len(pos), VERTEX_DTYPE)
            v["pos"], v["nrm"], v["tan"] = pos, nrm, tan
            v["u"], v["v"] = uv[:, 0], uv[:, 1]
            verts.append(v)
            idx.append(ind + np.uint32(nv))
            prim_range[(mi, pi)] = len(meshes)
            meshes.append((ni, ni + ind.size))
            nv += len(pos)
            ni += ind.size
    materials = js.get("materials", [])
    insts = []
    for node in js.get("nodes", []):
        if "mesh" not in node:
            continue
        l2w = _node_matrix(node)
        for pi, prim in enumerate(js["meshes"][node["mesh"]]["primitives"]):
            mat = materials[prim["material"]] if "material" in prim else {}
            pbr = mat.get("pbrMetallicRoughness", {})
            emissive = np.array(mat.get("emissiveFactor", [0.0, 0.0, 0.0]), np.float32)
            is_emissive = bool(np.any(emissive != 0))
            color = (np.array([*emissive, 1.0], np.float32) if is_emissive
                     else np.array(pbr.get("baseColorFactor", [1, 1, 1, 1]), np.float32))
            insts.append(dict(mesh=prim_range[(node["mesh"], pi)], l2w=l2w.astype(np.float32),
                              w2l=np.linalg.inv(l2w).astype(np.float32), color=color,
                              roughness=np.float32(pbr.get("roughnessFactor", 1.0)),
                              metallic=np.float32(pbr.get("metallicFactor", 1.0)),
                              emissive=np.float32(1.0 if is_emissive else 0.0)))
    if not verts:
        raise MeshError("Gltf", "no meshes")
    from .scenes import camera_matrices
    eye, target = camera if camera is not None else ((5.0, 0.0, 0.0), (0.0, 0.0, 0.0))  # camera.rs:41-42
    w2c, c2w = camera_matrices(eye, target, width, height)
    return SceneDesc(np.concatenate(verts), np.concatenate(idx).astype(np.uint32), meshes, insts, width, height,
                     c2w, w2c, tuple(env_color), None, bounces, spp)


def load_glb(path, **kw):
    with open(path, "rb") as f:
        return parse_glb(f.read(), **kw)


def write_glb(desc):
    """Serialises a SceneDesc as a GLB (one glTF mesh per mesh range, one node per instance)."""
    bin_parts, views, accessors = [], [], []

    def add(arr, target, comp, typ):
        arr = np.ascontiguousarray(arr)
        off = sum(len(b) for b in bin_parts)
        pad = (-off) % 4
        if pad:
            bin_parts.append(b"\0" * pad)
            off += pad
        bin_parts.append(arr.tobytes())
        views.append({"buffer": 0, "byteOffset": off, "byteLength": arr.nbytes, "target": target})
        accessors.append({"bufferView": len(views) - 1, "componentType": comp, "count": len(arr), "type": typ})
        if typ == "VEC3" and comp == 5126:
            accessors[-1]["min"] = arr.min(axis=0).tolist()
            accessors[-1]["max"] = arr.max(axis=0).tolist()
        return len(accessors) - 1

    meshes_js = []
    v = desc.vertices
    for s, e in desc.meshes:
        ind = desc.indices[s:e]
        used = np.unique(ind)
        remap = np.zeros(int(used.max()) + 1, np.uint32)
        remap[used] = np.arange(len(used), dtype=np.uint32)
        sub = v[used]
        a_pos = add(sub["pos"].astype(np.float32), 34962, 5126, "VEC3")
        a_nrm = add(sub["nrm"].astype(np.float32), 34962, 5126, "VEC3")
        a_tan = add(sub["tan"].astype(np.float32), 34962, 5126, "VEC4")
        a_uv = add(np.stack([sub["u"], sub["v"]], 1).astype(np.float32), 34962, 5126, "VEC2")
        a_idx = add(remap[ind].reshape(-1, 1), 34963, 5125, "SCALAR")
        meshes_js.append({"primitives": [{"attributes": {"POSITION": a_pos, "NORMAL": a_nrm, "TANGENT": a_tan,
                                                         "TEXCOORD_0": a_uv}, "indices": a_idx, "mode": 4}]})
    materials, nodes = [], []
    for k, inst in enumerate(desc.instances):
        c = [float(x) for x in inst["color"]]
        mat = {"pbrMetallicRoughness": {"baseColorFactor": c, "metallicFactor": float(inst["metallic"]),
                                        "roughnessFactor": float(inst["roughness"])}}
        if inst["emissive"] > 0:
            mat["emissiveFactor"] = c[:3]
        materials.append(mat)
        meshes_js[inst["mesh"]]["primitives"][0].setdefault("material", len(materials) - 1)
        m = np.asarray(inst["l2w"], np.float64)
        nodes.append({"mesh": inst["mesh"], "matrix": m.T.ravel().tolist()})
    js = {"asset": {"version": "2.0"}, "buffers": [{"byteLength": sum(len(b) for b in bin_parts)}],
          "bufferViews": views, "accessors": accessors, "meshes": meshes_js, "materials": materials, "nodes": nodes,
          "scenes": [{"nodes": list(range(len(nodes)))}], "scene": 0}
    jb = json.dumps(js).encode()
    jb += b" " * ((-len(jb)) % 4)
    bb = b"".join(bin_parts)
    bb += b"\0" * ((-len(bb)) % 4)
    body = struct.pack("<II", len(jb), 0x4E4F534A) + jb + struct.pack("<II", len(bb), 0x004E4942) + bb
    return struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body

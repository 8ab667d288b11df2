"""Scene ingest: VulkanExp's `.scene` container and glTF 2.0 into the arrays
of include/ddgi.h (a `scenes.Scene`), so that real scenes can replace the
synthetic ones.

The arrays are the ones the reference's renderer derives from a loaded
scene:
  * one offset-table entry per mesh with triangles: (the mesh's default
    material, its first vertex, its first index) (Renderer::
    updateMeshOffsetTable, src/Renderer.cpp:97-126);
  * one instance per entity that renders a mesh, with the entity's global
    transform (parent global x local, src/Scene.cpp:940-955) as its
    row-major 3x4 object-to-world matrix, custom index = the mesh's
    offset-table entry and mask INSTANCE_STATIC (Renderer::createTLAS,
    src/Renderer.cpp:525-550), ordered by (mesh, material) as
    Renderer::sortRenderers orders them (entity order among equals);
  * materials from the glTF-style `pbrMetallicRoughness` objects
    (parseMaterial, src/vulkan/Material.cpp:7-28; defaults: base colour 1,
    metallic 1, roughness 1, emissive 0; texture ids kept, not sampled).
Global transforms are composed in double and rounded to float once.

Formats:
  `.scene` (README.md "Scene Format"; Scene::save / Scene::loadScene,
  src/Scene.cpp:706-935): header {magic "SCEN" 0x4e454353, version,
  total length}, then chunks {length, type} + data; chunk 0 is JSON
  ("JSON" 0x4E4F534A), the rest binary (" BIN" 0x004E4942).  JSON:
  materials, entities {name, transform (16 numbers, column-major), children
  (entity indices), meshRenderer {meshIndex, materialIndex}}, meshes {name,
  material, vertexArray, indexArray (chunk indices, JSON = 0)}, textures.
  Vertex arrays hold the 64-byte Vertex records, index arrays uint32.
  glTF 2.0 (`.gltf` with external or base64 buffers, `.glb`), the subset
  Scene::loadglTF (src/Scene.cpp:115-533) reads for static meshes: one mesh
  per primitive (default material = the primitive's), POSITION / NORMAL /
  TANGENT / TEXCOORD_0 / indices accessors, node matrix or TRS, node
  hierarchy under the scenes' root nodes; a node with several primitives
  gets one child entity per primitive.
"""
import base64
import json
import os
import struct

import numpy as np

from .abi import INSTANCE_DTYPE, MATERIAL_DTYPE, MESH_DTYPE, NO_TEXTURE, OFFSET_DTYPE, VERTEX_DTYPE
from .scenes import Scene, scene_bounds

SCENE_MAGIC = 0x4E454353
CHUNK_JSON = 0x4E4F534A
CHUNK_BIN = 0x004E4942
GLB_MAGIC = 0x46546C67


class IngestError(ValueError):
    pass


# ---------------------------------------------------------------------------
# an intermediate scene: meshes, materials, entity tree
# ---------------------------------------------------------------------------
class SceneData:
    """Meshes (vertex records + uint32 indices + default material),
    materials (dicts in the glTF material form) and entities (local
    column-major 4x4, children, optional (mesh, material) renderer)."""

    def __init__(self):
        self.meshes = []      # dicts: name, vertices (VERTEX_DTYPE), indices (uint32), material
        self.materials = []   # glTF-style material dicts
        self.entities = []    # dicts: name, transform (4x4 float64, math order), children, renderer
        self.roots = []       # entities without a parent, in order

    def global_transforms(self):
        out = [None] * len(self.entities)
        parent = [-1] * len(self.entities)
        for i, e in enumerate(self.entities):
            for c in e["children"]:
                if not 0 <= c < len(self.entities):
                    raise IngestError("entity %d: child %d out of range" % (i, c))
                if parent[c] != -1:
                    raise IngestError("entity %d has two parents" % c)
                parent[c] = i
        order = [i for i in range(len(self.entities)) if parent[i] == -1]
        stack = [(i, np.eye(4)) for i in reversed(order)]
        seen = 0
        while stack:
            i, pm = stack.pop()
            g = pm @ self.entities[i]["transform"]
            out[i] = g
            seen += 1
            for c in reversed(self.entities[i]["children"]):
                stack.append((c, g))
        if seen != len(self.entities):
            raise IngestError("entity hierarchy has a cycle")
        return out


def _material_record(m):
    r = np.zeros((), MATERIAL_DTYPE)
    pbr = m.get("pbrMetallicRoughness", None)
    base = [1.0, 1.0, 1.0, 1.0]
    metal, rough = 1.0, 1.0
    albedo_tex = mr_tex = NO_TEXTURE
    if pbr is not None:
        base = pbr.get("baseColorFactor", base)
        metal = pbr.get("metallicFactor", 1.0)
        rough = pbr.get("roughnessFactor", 1.0)
        if "baseColorTexture" in pbr:
            albedo_tex = int(pbr["baseColorTexture"]["index"]) & 0xFFFFFFFF
        if "metallicRoughnessTexture" in pbr:
            mr_tex = int(pbr["metallicRoughnessTexture"]["index"]) & 0xFFFFFFFF
    r["metallic"] = metal
    r["roughness"] = rough
    r["base_color"] = base[:3]
    r["emissive"] = m.get("emissiveFactor", [0.0, 0.0, 0.0])[:3]
    r["albedo_texture"] = albedo_tex
    r["metallic_roughness_texture"] = mr_tex
    r["normal_texture"] = int(m["normalTexture"]["index"]) & 0xFFFFFFFF if "normalTexture" in m else NO_TEXTURE
    r["emissive_texture"] = int(m["emissiveTexture"]["index"]) & 0xFFFFFFFF if "emissiveTexture" in m else NO_TEXTURE
    return r


def to_scene(data):
    """SceneData -> scenes.Scene (the arrays of include/ddgi.h)."""
    valid = [m for m in range(len(data.meshes)) if len(data.meshes[m]["indices"]) >= 3]
    if not data.materials:
        data.materials = [{}]
    verts, inds = [], []
    meshes = np.zeros(len(data.meshes), MESH_DTYPE)
    offsets = np.zeros(len(valid), OFFSET_DTYPE)
    entry_of_mesh = {}
    vofs = iofs = 0
    for m, mesh in enumerate(data.meshes):
        v, idx = mesh["vertices"], np.asarray(mesh["indices"], np.uint32)
        n = len(idx) - len(idx) % 3
        idx = idx[:n]
        if n and idx.max(initial=0) >= len(v):
            raise IngestError("mesh %d: index out of range" % m)
        meshes[m] = (vofs, len(v), iofs, n)
        if m in valid:
            mat = int(mesh["material"])
            if not 0 <= mat < len(data.materials):
                raise IngestError("mesh %d: material %d out of range" % (m, mat))
            entry_of_mesh[m] = len(entry_of_mesh)
            offsets[entry_of_mesh[m]] = (mat, vofs, iofs)
        verts.append(v)
        inds.append(idx)
        vofs += len(v)
        iofs += n
    g = data.global_transforms()
    renderers = [(e["renderer"][0], e["renderer"][1], i) for i, e in enumerate(data.entities)
                 if e.get("renderer") is not None and e["renderer"][0] in entry_of_mesh]
    renderers.sort(key=lambda r: (r[0], r[1], r[2]))
    inst = np.zeros(len(renderers), INSTANCE_DTYPE)
    for k, (mesh, _mat, ent) in enumerate(renderers):
        inst[k]["transform"] = g[ent][:3, :4].reshape(12).astype(np.float32)
        inst[k]["custom_index"] = entry_of_mesh[mesh]
        inst[k]["mask"] = 1  # INSTANCE_STATIC
        inst[k]["mesh_index"] = mesh
    mats = np.array([_material_record(m) for m in data.materials], MATERIAL_DTYPE)
    v = np.concatenate(verts) if verts else np.zeros(0, VERTEX_DTYPE)
    i = np.concatenate(inds).astype(np.uint32) if inds else np.zeros(0, np.uint32)
    sc = Scene(v, i, meshes, inst, offsets, mats)
    sc.bounds = scene_bounds(sc) if len(inst) else (np.zeros(3), np.ones(3))
    return sc


# ---------------------------------------------------------------------------
# .scene container
# ---------------------------------------------------------------------------
def _mat4_from_columns(a):
    a = [float(x) for x in a]
    if len(a) != 16:
        raise IngestError("transform needs 16 numbers")
    return np.array(a, np.float64).reshape(4, 4).T  # column-major list -> math matrix


def read_scene_file(path):
    """Parses a `.scene` file into SceneData."""
    with open(path, "rb") as f:
        buf = f.read()
    if len(buf) < 20:
        raise IngestError("file too short")
    magic, _version, length = struct.unpack_from("<III", buf, 0)
    if magic != SCENE_MAGIC:
        raise IngestError("not a scene file (magic %#x)" % magic)
    length = min(length, len(buf))
    chunks = []
    off = 12
    while off + 8 <= length:
        clen, ctype = struct.unpack_from("<II", buf, off)
        if off + 8 + clen > length:
            raise IngestError("chunk %d runs past the end of the file" % len(chunks))
        chunks.append((ctype, buf[off + 8:off + 8 + clen]))
        off += 8 + clen
    if not chunks or chunks[0][0] != CHUNK_JSON:
        raise IngestError("the first chunk must be JSON")
    root = json.loads(chunks[0][1].decode("utf-8"))
    data = SceneData()
    data.materials = list(root.get("materials", []))
    for m in root.get("meshes", []):
        vi, ii = int(m["vertexArray"]), int(m["indexArray"])
        if not (0 < vi < len(chunks) and 0 < ii < len(chunks)):
            raise IngestError("mesh '%s': chunk index out of range" % m.get("name", ""))
        vb, ib = chunks[vi][1], chunks[ii][1]
        if len(vb) % VERTEX_DTYPE.itemsize or len(ib) % 4:
            raise IngestError("mesh '%s': chunk sizes are not whole records" % m.get("name", ""))
        data.meshes.append({"name": m.get("name", ""), "vertices": np.frombuffer(vb, VERTEX_DTYPE).copy(),
                            "indices": np.frombuffer(ib, np.uint32).copy(), "material": int(m.get("material", 0))})
    for e in root.get("entities", []):
        r = e.get("meshRenderer")
        data.entities.append({"name": e.get("name", ""), "transform": _mat4_from_columns(e["transform"]),
                              "children": [int(c) for c in e.get("children", [])],
                              "renderer": None if r is None else (int(r["meshIndex"]), int(r["materialIndex"]))})
    return data


def write_scene_file(path, data):
    """Writes SceneData as a `.scene` file (the layout of Scene::save)."""
    chunks = []
    meshes = []
    for m in data.meshes:
        base = 1 + len(chunks)
        meshes.append({"name": m["name"], "material": int(m["material"]), "vertexArray": base, "indexArray": base + 1})
        chunks.append(np.ascontiguousarray(m["vertices"], VERTEX_DTYPE).tobytes())
        chunks.append(np.ascontiguousarray(m["indices"], np.uint32).tobytes())
    ents = []
    for e in data.entities:
        d = {"name": e["name"], "transform": [float(x) for x in np.asarray(e["transform"]).T.reshape(16)],
             "parent": -1, "children": list(e["children"])}
        if e.get("renderer") is not None:
            d["meshRenderer"] = {"meshIndex": int(e["renderer"][0]), "materialIndex": int(e["renderer"][1])}
        ents.append(d)
    js = json.dumps({"materials": data.materials, "entities": ents, "meshes": meshes, "textures": []}).encode()
    total = 12 + sum(8 + len(c) for c in [js] + chunks)
    with open(path, "wb") as f:
        f.write(struct.pack("<III", SCENE_MAGIC, 0, total))
        for ctype, c in [(CHUNK_JSON, js)] + [(CHUNK_BIN, c) for c in chunks]:
            f.write(struct.pack("<II", len(c), ctype))
            f.write(c)


# ---------------------------------------------------------------------------
# glTF 2.0
# ---------------------------------------------------------------------------
_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}


def _accessor(gl, buffers, idx):
    a = gl["accessors"][idx]
    dt = np.dtype(_COMPONENT[a["componentType"]])
    nc = _NCOMP[a["type"]]
    count = int(a["count"])
    if "bufferView" not in a:
        return np.zeros((count, nc), dt)
    bv = gl["bufferViews"][a["bufferView"]]
    data = buffers[bv["buffer"]]
    start = int(bv.get("byteOffset", 0)) + int(a.get("byteOffset", 0))
    stride = int(bv.get("byteStride", 0)) or dt.itemsize * nc
    if count and start + stride * (count - 1) + dt.itemsize * nc > len(data):
        raise IngestError("accessor %d runs past its buffer" % idx)
    raw = np.frombuffer(data, np.uint8, count=stride * (count - 1) + dt.itemsize * nc if count else 0, offset=start)
    out = np.empty((count, nc), dt)
    for k in range(nc):  # strided gather, component by component
        cols = np.lib.stride_tricks.as_strided(raw[k * dt.itemsize:], shape=(count, dt.itemsize),
                                               strides=(stride, 1))
        out[:, k] = np.ascontiguousarray(cols).view(dt).reshape(count)
    if a.get("normalized") and dt.kind in "iu":
        # normalised integers (glTF 2.0 section 3.11): c / max, signed ones
        # clamped at -1; the reference reads float attributes only
        # (src/Scene.cpp:72-88, 229), so this widens what loads
        top = float(np.iinfo(dt).max)
        return np.maximum(out.astype(np.float64) / top, -1.0).astype(np.float32)
    return out


def _quat_to_mat(q):
    x, y, z, w = [float(v) for v in q]
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y), 0],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x), 0],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y), 0],
        [0, 0, 0, 1]])


def _node_matrix(node):
    if "matrix" in node:
        return _mat4_from_columns(node["matrix"])
    t = np.eye(4)
    t[:3, 3] = node.get("translation", [0.0, 0.0, 0.0])
    r = _quat_to_mat(node.get("rotation", [0.0, 0.0, 0.0, 1.0]))
    s = np.diag(list(node.get("scale", [1.0, 1.0, 1.0])) + [1.0])
    return t @ r @ s


def _load_buffers(gl, base_dir, glb_bin):
    out = []
    for k, b in enumerate(gl.get("buffers", [])):
        uri = b.get("uri")
        if uri is None:
            if glb_bin is None:
                raise IngestError("buffer %d has no data" % k)
            out.append(glb_bin)
        elif uri.startswith("data:"):
            if ";base64," not in uri:
                raise IngestError("buffer %d: unsupported data URI" % k)
            out.append(base64.b64decode(uri.split(";base64,", 1)[1]))
        else:
            with open(os.path.join(base_dir, uri), "rb") as f:
                out.append(f.read())
    return out


def read_gltf(path):
    """Parses a `.gltf` or `.glb` file into SceneData."""
    with open(path, "rb") as f:
        raw = f.read()
    glb_bin = None
    if raw[:4] == struct.pack("<I", GLB_MAGIC):
        _m, _v, length = struct.unpack_from("<III", raw, 0)
        off, gl = 12, None
        while off + 8 <= min(length, len(raw)):
            clen, ctype = struct.unpack_from("<II", raw, off)
            body = raw[off + 8:off + 8 + clen]
            if ctype == CHUNK_JSON and gl is None:
                gl = json.loads(body.decode("utf-8"))
            elif ctype == CHUNK_BIN and glb_bin is None:
                glb_bin = body
            off += 8 + clen
        if gl is None:
            raise IngestError("GLB without a JSON chunk")
    else:
        gl = json.loads(raw.decode("utf-8"))
    buffers = _load_buffers(gl, os.path.dirname(os.path.abspath(path)), glb_bin)
    data = SceneData()
    data.materials = list(gl.get("materials", []))
    prims_of_mesh = []
    for m in gl.get("meshes", []):
        ids = []
        for p in m.get("primitives", []):
            if p.get("mode", 4) != 4:
                continue  # triangles only
            at = p["attributes"]
            pos = _accessor(gl, buffers, at["POSITION"]).astype(np.float32)
            v = np.zeros(len(pos), VERTEX_DTYPE)
            v["pos"] = pos[:, :3]
            v["color"] = 1.0
            if "NORMAL" in at:
                v["normal"] = _accessor(gl, buffers, at["NORMAL"])[:, :3]
            if "TANGENT" in at:
                v["tangent"] = _accessor(gl, buffers, at["TANGENT"])[:, :4]
            if "TEXCOORD_0" in at:
                v["uv"] = _accessor(gl, buffers, at["TEXCOORD_0"])[:, :2]
            if "indices" in p:
                idx = _accessor(gl, buffers, p["indices"]).reshape(-1).astype(np.uint32)
            else:
                idx = np.arange(len(pos) - len(pos) % 3, dtype=np.uint32)
            ids.append(len(data.meshes))
            data.meshes.append({"name": m.get("name", ""), "vertices": v, "indices": idx,
                                "material": int(p.get("material", 0))})
        prims_of_mesh.append(ids)
    nodes = gl.get("nodes", [])
    for n in nodes:
        data.entities.append({"name": n.get("name", ""), "transform": _node_matrix(n),
                              "children": [int(c) for c in n.get("children", [])], "renderer": None})
    for ni, n in enumerate(nodes):
        if "mesh" not in n:
            continue
        ids = prims_of_mesh[int(n["mesh"])]
        if len(ids) == 1:
            data.entities[ni]["renderer"] = (ids[0], data.meshes[ids[0]]["material"])
        else:
            for mid in ids:
                data.entities[ni]["children"].append(len(data.entities))
                data.entities.append({"name": "", "transform": np.eye(4), "children": [],
                                      "renderer": (mid, data.meshes[mid]["material"])})
    # nodes outside every scene are not drawn (the reference parents scene
    # roots under its root entity); without scenes, every root node is drawn
    scenes_ = gl.get("scenes")
    if scenes_:
        listed = set()
        for s in scenes_:
            listed.update(int(x) for x in s.get("nodes", []))
        reachable = set()
        stack = list(listed)
        while stack:
            i = stack.pop()
            if i in reachable:
                continue
            reachable.add(i)
            stack.extend(data.entities[i]["children"])
        for i, e in enumerate(data.entities):
            if i not in reachable:
                e["renderer"] = None
    return data


def load(path):
    """A `.scene`, `.gltf` or `.glb` file as a scenes.Scene."""
    ext = os.path.splitext(path)[1].lower()
    if ext == ".scene":
        return to_scene(read_scene_file(path))
    if ext in (".gltf", ".glb"):
        return to_scene(read_gltf(path))
    raise IngestError("unsupported scene file '%s'" % path)


def scene_data_from(scene):
    """SceneData of a scenes.Scene (one entity per instance, under one root):
    the inverse of to_scene, used to write generated scenes as `.scene`."""
    data = SceneData()
    data.materials = []
    for m in scene.materials:
        data.materials.append({"pbrMetallicRoughness": {"baseColorFactor": [float(x) for x in m["base_color"]] + [1.0],
                                                        "metallicFactor": float(m["metallic"]),
                                                        "roughnessFactor": float(m["roughness"])},
                               "emissiveFactor": [float(x) for x in m["emissive"]]})
    # one mesh per (mesh, offset entry) pair the instances use: the default
    # material is the entry's material
    pairs = {}
    for inst in scene.instances:
        pairs.setdefault((int(inst["mesh_index"]), int(inst["custom_index"])), None)
    for k, (mi, ci) in enumerate(sorted(pairs)):
        me = scene.meshes[mi]
        oe = scene.offsets[ci]
        idx = scene.indices[oe["index_offset"]:oe["index_offset"] + me["index_count"]]
        v = scene.vertices[oe["vertex_offset"]:oe["vertex_offset"] + me["vertex_count"]]
        data.meshes.append({"name": "mesh%d_%d" % (mi, ci), "vertices": v.copy(), "indices": idx.copy(),
                            "material": int(oe["material_index"])})
        pairs[(mi, ci)] = k
    data.entities.append({"name": "root", "transform": np.eye(4), "children": [], "renderer": None})
    for inst in scene.instances:
        m = np.eye(4)
        m[:3, :4] = inst["transform"].reshape(3, 4).astype(np.float64)
        k = pairs[(int(inst["mesh_index"]), int(inst["custom_index"]))]
        data.entities[0]["children"].append(len(data.entities))
        data.entities.append({"name": "", "transform": m, "children": [], "renderer": (k, data.meshes[k]["material"])})
    return data

"""Writes tests/golden/editor_room.scene, a small scene file laid out byte
for byte as VulkanExp's editor saves one (Scene::save, src/Scene.cpp:
710-817), independently of the package's own writer:

* header {magic 0x4e454353 "SCEN", version 0, total length} (GLBHeader,
  src/Scene.cpp:51-55; README.md "Scene Format");
* chunk 0: JSON, then per mesh two BIN chunks (vertex array, index array),
  each chunk {uint32 length, uint32 type} + data, no padding
  (GLBChunkType JSON 0x4E4F534A, BIN 0x004E4942, src/Scene.cpp:57-60;
  the loop at src/Scene.cpp:806-811);
* the JSON text as the reference's JSON class prints it (src/JSON.hpp:
  27-32, 178-186, 590-614): objects "{"key": value, ...}" with keys in
  std::map order, arrays "[a, b]", reals by std::to_string (six decimals),
  integers by std::to_string, strings quoted;
* the root object's keys as Scene::save fills them: "materials" (toJSON of
  Material, src/vulkan/Material.cpp:30-53: name, pbrMetallicRoughness
  {baseColorFactor as a vec4 with w = 1, metallicFactor, roughnessFactor,
  baseColorTexture {index}, metallicRoughnessTexture {index}}, normalTexture
  {index}, emissiveFactor, emissiveTexture {index}; an unset texture is
  InvalidTextureIndex, uint32 -1 printed through int as -1), "entities"
  (name, transform as 16 column-major reals (Serialization.hpp:25-29),
  parent -1, children, meshRenderer {meshIndex, materialIndex}), "meshes"
  (name, material, vertexArray, indexArray: chunk numbers, the JSON chunk
  being 0), "textures";
* vertex records of 64 bytes: pos vec3, color vec3, normal vec3, tangent
  vec4, texCoord vec2, uint32 padding (src/vulkan/Vertex.hpp:8-15); indices
  uint32.

The scene: a floor quad, a box mesh used by three entities (two under a
rotated group, one scaled into a pillar), a wall quad, and a mesh with no
triangles (skipped by the renderer).  Run:
    python tests/golden/make_scene_fixture.py
"""
import math
import os
import struct

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "editor_room.scene")


def jreal(x):
    return "%f" % x  # std::to_string(float): %f


def jvalue(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, int):
        return "%d" % v
    if isinstance(v, float):
        return jreal(v)
    if isinstance(v, str):
        return '"' + v.replace("\\", "\\\\").replace('"', '\\"') + '"'
    if isinstance(v, list):
        return "[" + ", ".join(jvalue(x) for x in v) + "]"
    if isinstance(v, dict):
        return "{" + ", ".join('"%s": %s' % (k, jvalue(v[k])) for k in sorted(v)) + "}"
    raise TypeError(type(v))


INVALID = -1  # InvalidTextureIndex through static_cast<int>


def material(name, base, metal, rough, emissive=(0.0, 0.0, 0.0)):
    return {"name": name,
            "pbrMetallicRoughness": {"baseColorFactor": [float(base[0]), float(base[1]), float(base[2]), 1.0],
                                     "metallicFactor": float(metal), "roughnessFactor": float(rough),
                                     "baseColorTexture": {"index": INVALID},
                                     "metallicRoughnessTexture": {"index": INVALID}},
            "normalTexture": {"index": INVALID}, "emissiveFactor": [float(e) for e in emissive],
            "emissiveTexture": {"index": INVALID}}


def vertex(p, n, uv=(0.0, 0.0)):
    # pos, color (1), normal, tangent, texCoord, padding
    return struct.pack("<3f3f3f4f2fI", *p, 1.0, 1.0, 1.0, *n, 1.0, 0.0, 0.0, 1.0, *uv, 0)


def quad(size_x, size_z):
    v = b"".join(vertex((sx * size_x / 2, 0.0, sz * size_z / 2), (0.0, 1.0, 0.0), ((sx + 1) / 2, (sz + 1) / 2))
                 for sx, sz in ((-1, -1), (1, -1), (1, 1), (-1, 1)))
    idx = [0, 2, 1, 0, 3, 2]  # counter-clockwise seen from +y
    return v, struct.pack("<%dI" % len(idx), *idx)


def box():
    faces = [((1, 0, 0), (0, 1, 0), (0, 0, 1)), ((-1, 0, 0), (0, 0, 1), (0, 1, 0)),
             ((0, 1, 0), (0, 0, 1), (1, 0, 0)), ((0, -1, 0), (1, 0, 0), (0, 0, 1)),
             ((0, 0, 1), (1, 0, 0), (0, 1, 0)), ((0, 0, -1), (0, 1, 0), (1, 0, 0))]
    verts, idx = b"", []
    for k, (n, a, b) in enumerate(faces):
        c = [0.5 * x for x in n]
        for sa, sb in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
            p = tuple(c[i] + 0.5 * sa * a[i] + 0.5 * sb * b[i] for i in range(3))
            verts += vertex(p, n)
        idx += [4 * k, 4 * k + 1, 4 * k + 2, 4 * k, 4 * k + 2, 4 * k + 3]
    return verts, struct.pack("<%dI" % len(idx), *idx)


def trs(t=(0.0, 0.0, 0.0), yaw=0.0, pitch=0.0, s=(1.0, 1.0, 1.0)):
    """Column-major 4x4 (glm layout) of T * Ry(yaw) * Rx(pitch) * S."""
    cy, sy, cp, sp = math.cos(yaw), math.sin(yaw), math.cos(pitch), math.sin(pitch)
    ry = [[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]]
    rx = [[1, 0, 0], [0, cp, -sp], [0, sp, cp]]
    r = [[sum(ry[i][k] * rx[k][j] for k in range(3)) for j in range(3)] for i in range(3)]
    m = [[r[i][j] * s[j] for j in range(3)] + [t[i]] for i in range(3)] + [[0.0, 0.0, 0.0, 1.0]]
    return [float(m[row][col]) for col in range(4) for row in range(4)]


def main():
    materials = [material("Floor", (0.7, 0.7, 0.7), 0.0, 1.0), material("Red", (0.8, 0.2, 0.1), 0.0, 0.6),
                 material("Glow", (0.3, 0.6, 0.9), 0.2, 0.4, (0.5, 0.4, 0.1))]
    floor_v, floor_i = quad(20.0, 20.0)
    box_v, box_i = box()
    wall_v, wall_i = quad(6.0, 3.0)
    mesh_data = [("Floor", 0, floor_v, floor_i), ("Box", 1, box_v, box_i), ("Wall", 2, wall_v, wall_i),
                 ("Empty", 0, vertex((0.0, 0.0, 0.0), (0.0, 1.0, 0.0)), b"")]
    entities = [
        {"name": "Root", "transform": trs(), "parent": -1, "children": [1, 2, 5, 6]},
        {"name": "Floor", "transform": trs(), "parent": -1, "children": [], "meshRenderer": {"meshIndex": 0,
                                                                                           "materialIndex": 0}},
        {"name": "Group", "transform": trs((2.0, 0.0, 1.0), yaw=math.radians(30.0)), "parent": -1,
         "children": [3, 4]},
        {"name": "Box A", "transform": trs((0.0, 0.75, 0.0), s=(1.5, 1.5, 1.5)), "parent": -1, "children": [],
         "meshRenderer": {"meshIndex": 1, "materialIndex": 1}},
        {"name": "Box B", "transform": trs((-3.0, 1.0, 2.0), pitch=math.radians(20.0)), "parent": -1,
         "children": [], "meshRenderer": {"meshIndex": 1, "materialIndex": 2}},
        {"name": "Pillar", "transform": trs((5.0, 2.0, -4.0), s=(0.5, 4.0, 0.5)), "parent": -1, "children": [],
         "meshRenderer": {"meshIndex": 1, "materialIndex": 0}},
        {"name": "Wall", "transform": trs((0.0, 1.5, -6.0), pitch=math.radians(90.0)), "parent": -1,
         "children": [], "meshRenderer": {"meshIndex": 2, "materialIndex": 2}},
    ]
    meshes, chunks = [], []
    for name, mat, v, i in mesh_data:
        offset = 1 + len(chunks)
        meshes.append({"name": name, "material": mat, "vertexArray": offset, "indexArray": offset + 1})
        chunks += [v, i]
    root = {"materials": materials, "entities": entities, "meshes": meshes,
            "textures": [{"source": "data/blank.png", "format": 43, "sampler": {}}]}
    js = jvalue(root).encode()
    bufs = [(0x4E4F534A, js)] + [(0x004E4942, c) for c in chunks]
    total = 12 + sum(8 + len(c) for _, c in bufs)
    with open(OUT, "wb") as f:
        f.write(struct.pack("<III", 0x4E454353, 0, total))
        for t, c in bufs:
            f.write(struct.pack("<II", len(c), t))
            f.write(c)
    print(OUT, total, "bytes")


if __name__ == "__main__":
    main()

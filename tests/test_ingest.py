"""Scene ingest (`.scene` container and glTF 2.0) on the CPU: a generated
scene written as `.scene` and read back traces and shades identically (the
oracle gives the same hits and the same atlas, bit for bit); a hand-built
glTF yields the instances, global transforms and materials its node tree
describes, the same from `.gltf` and `.glb`."""
import base64
import json
import struct

import numpy as np
import pytest

from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, ingest, scenes


def test_scene_file_round_trip(tmp_path):
    w = scenes.room_workload(21, n_boxes=60, resolution=(4, 4, 4), rays=64)
    path = tmp_path / "room.scene"
    ingest.write_scene_file(str(path), ingest.scene_data_from(w.scene))
    head = path.read_bytes()[:12]
    assert struct.unpack("<III", head)[0] == 0x4E454353
    assert struct.unpack("<III", head)[2] == path.stat().st_size
    sc = ingest.load(str(path))
    assert len(sc.instances) == len(w.scene.instances)
    assert (sc.instances["transform"] == w.scene.instances["transform"]).all()
    assert sc.triangle_count == w.scene.triangle_count
    rng = np.random.default_rng(2)
    o = rng.uniform(-1, 11, size=(5000, 3)).astype(np.float32)
    d = rng.normal(size=(5000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    a, _ = Oracle(w.scene).trace(o, d, 0.01, 100.0)
    b, _ = Oracle(sc).trace(o, d, 0.01, 100.0)
    assert (a == b).all()
    outs = []
    for s in (w.scene, sc):
        c, dd = zero_atlas(w.grid)
        st = np.ones(w.grid.probe_count(), np.uint32)
        Oracle(s).update(w.grid, w.light, w.orientation(0), c, dd, st)
        outs.append((c, dd))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_scene_file_rejects_bad_files(tmp_path):
    p = tmp_path / "bad.scene"
    p.write_bytes(b"GLTF" + bytes(20))
    with pytest.raises(ingest.IngestError):
        ingest.load(str(p))
    p.write_bytes(struct.pack("<III", 0x4E454353, 0, 1000) + struct.pack("<II", 5000, 0x4E4F534A) + b"{}")
    with pytest.raises(ingest.IngestError):
        ingest.load(str(p))


def _box():
    p, n, t = scenes.box_geometry((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    return p.astype(np.float32), n.astype(np.float32), t.reshape(-1).astype(np.uint16)


def make_gltf():
    p, n, t = _box()
    blob = p.tobytes() + n.tobytes() + t.tobytes()
    views = [{"buffer": 0, "byteOffset": 0, "byteLength": p.nbytes},
             {"buffer": 0, "byteOffset": p.nbytes, "byteLength": n.nbytes},
             {"buffer": 0, "byteOffset": p.nbytes + n.nbytes, "byteLength": t.nbytes}]
    acc = [{"bufferView": 0, "componentType": 5126, "count": len(p), "type": "VEC3"},
           {"bufferView": 1, "componentType": 5126, "count": len(n), "type": "VEC3"},
           {"bufferView": 2, "componentType": 5123, "count": len(t), "type": "SCALAR"}]
    prim = lambda mat: {"attributes": {"POSITION": 0, "NORMAL": 1}, "indices": 2, "material": mat}
    q = [0.0, np.sin(0.3), 0.0, np.cos(0.3)]  # rotation about y by 0.6 rad
    gl = {
        "asset": {"version": "2.0"},
        "scenes": [{"nodes": [0]}], "scene": 0,
        "nodes": [
            {"translation": [1.0, 2.0, 3.0], "rotation": q, "scale": [2.0, 2.0, 2.0], "children": [1, 2]},
            {"matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 4.0, 0.0, -1.0, 1], "mesh": 0},
            {"translation": [0.0, 1.5, 0.0], "mesh": 1},
            {"mesh": 0},  # not in any scene: not drawn
        ],
        "meshes": [{"primitives": [prim(0)]}, {"primitives": [prim(1), prim(0)]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 1.0], "metallicFactor": 0.0,
                                                "roughnessFactor": 0.7}},
                      {"emissiveFactor": [1.0, 0.5, 0.0]}],
        "buffers": [{"byteLength": len(blob)}],
        "bufferViews": views, "accessors": acc,
    }
    return gl, blob


def expected_globals():
    c, s = np.cos(0.6), np.sin(0.6)
    root = np.eye(4)
    root[:3, :3] = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]]) * 2.0
    root[:3, 3] = [1, 2, 3]
    a = np.eye(4)
    a[:3, 3] = [4, 0, -1]
    b = np.eye(4)
    b[:3, 3] = [0, 1.5, 0]
    return root @ a, root @ b


def check_loaded(sc):
    assert len(sc.instances) == 3  # node 1 (mesh 0) + node 2's two primitives
    ga, gb = expected_globals()
    # ordered by (mesh, material): mesh 0 (node 1), then the two primitives of mesh 1
    assert list(sc.instances["mesh_index"]) == [0, 1, 2]
    np.testing.assert_allclose(sc.instances["transform"][0].reshape(3, 4), ga[:3], rtol=1e-6, atol=1e-6)
    for k in (1, 2):
        np.testing.assert_allclose(sc.instances["transform"][k].reshape(3, 4), gb[:3], rtol=1e-6, atol=1e-6)
    assert (sc.instances["mask"] == 1).all()
    # offset entries carry each mesh's default material
    assert [int(sc.offsets[ci]["material_index"]) for ci in sc.instances["custom_index"]] == [0, 1, 0]
    m0, m1 = sc.materials
    assert np.allclose(m0["base_color"], [0.2, 0.4, 0.6]) and m0["metallic"] == 0.0 and np.isclose(m0["roughness"], 0.7)
    assert np.allclose(m1["base_color"], 1.0) and m1["metallic"] == 1.0 and np.allclose(m1["emissive"], [1.0, 0.5, 0.0])
    assert m0["albedo_texture"] == abi.NO_TEXTURE
    # geometry: a ray through instance 0's box centre hits it
    o = Oracle(sc)
    centre = ga[:3, 3].astype(np.float32)
    h, _ = o.trace(np.array([centre + [0, 0, 10]], np.float32), np.array([[0, 0, -1]], np.float32), 0.01, 100.0)
    assert h["instance"][0] != abi.MISS


def test_gltf_and_glb(tmp_path):
    gl, blob = make_gltf()
    g1 = dict(gl)
    g1["buffers"] = [{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                      base64.b64encode(blob).decode()}]
    p1 = tmp_path / "s.gltf"
    p1.write_text(json.dumps(g1))
    check_loaded(ingest.load(str(p1)))
    # external buffer file
    (tmp_path / "s.bin").write_bytes(blob)
    g2 = dict(gl)
    g2["buffers"] = [{"byteLength": len(blob), "uri": "s.bin"}]
    p2 = tmp_path / "s2.gltf"
    p2.write_text(json.dumps(g2))
    check_loaded(ingest.load(str(p2)))
    # binary container
    js = json.dumps(gl).encode()
    js += b" " * (-len(js) % 4)
    bb = blob + b"\0" * (-len(blob) % 4)
    glb = struct.pack("<III", 0x46546C67, 2, 12 + 8 + len(js) + 8 + len(bb))
    glb += struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bb), 0x004E4942) + bb
    p3 = tmp_path / "s.glb"
    p3.write_bytes(glb)
    check_loaded(ingest.load(str(p3)))


def test_gltf_cycle_rejected(tmp_path):
    gl, blob = make_gltf()
    gl["nodes"][1]["children"] = [0]
    gl["buffers"] = [{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                      base64.b64encode(blob).decode()}]
    p = tmp_path / "c.gltf"
    p.write_text(json.dumps(gl))
    with pytest.raises(ingest.IngestError):
        ingest.load(str(p))


FIXTURE = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "editor_room.scene")


def test_editor_saved_scene_fixture():
    """tests/golden/editor_room.scene is laid out as the editor's
    Scene::save writes a file (src/Scene.cpp:710-817, made by
    tests/golden/make_scene_fixture.py, not by this package's writer): the
    reference's JSON printing (six-decimal reals, "-1" for unset textures,
    std::map key order), unpadded chunks, 64-byte vertices.  It loads into
    the renderer's arrays: one offset entry per mesh with triangles (the
    empty mesh has none), instances ordered by (mesh, material, entity) with
    global transforms parent x local, materials with unset textures."""
    data = ingest.read_scene_file(FIXTURE)
    assert [m["name"] for m in data.meshes] == ["Floor", "Box", "Wall", "Empty"]
    sc = ingest.to_scene(data)
    assert len(sc.vertices) == 33 and len(sc.indices) == 48
    assert sc.offsets.tolist() == [(0, 0, 0), (1, 4, 6), (2, 28, 42)]
    assert sc.instances["mesh_index"].tolist() == [0, 1, 1, 1, 2]
    assert sc.instances["custom_index"].tolist() == [0, 1, 1, 1, 2]
    assert (sc.instances["mask"] == 1).all()
    # Pillar (mesh 1, material 0) sorts before Box A (material 1), Box B (2)
    np.testing.assert_array_equal(sc.instances["transform"][1], np.float32([0.5, 0, 0, 5, 0, 4, 0, 2, 0, 0, 0.5, -4]))
    # Box A: Group (yaw 30 deg, printed as 0.866025 / 0.5) x (scale 1.5, lift 0.75)
    c, s = 0.866025, 0.5
    group = np.array([[c, 0, s, 2], [0, 1, 0, 0], [-s, 0, c, 1], [0, 0, 0, 1]])
    box_a = np.array([[1.5, 0, 0, 0], [0, 1.5, 0, 0.75], [0, 0, 1.5, 0], [0, 0, 0, 1]])
    np.testing.assert_array_equal(sc.instances["transform"][2], (group @ box_a)[:3].reshape(12).astype(np.float32))
    assert sc.materials["base_color"][2].tolist() == pytest.approx([0.3, 0.6, 0.9])
    assert sc.materials["emissive"][2].tolist() == pytest.approx([0.5, 0.4, 0.1])
    assert (sc.materials["albedo_texture"] == abi.NO_TEXTURE).all()
    assert (sc.materials["normal_texture"] == abi.NO_TEXTURE).all()
    # the oracle traces it: rays from above hit the floor or the boxes
    o = Oracle(sc)
    rng = np.random.default_rng(4)
    org = np.column_stack([rng.uniform(-9, 9, 2000), np.full(2000, 8.0), rng.uniform(-9, 9, 2000)]).astype(np.float32)
    dirs = np.tile(np.float32([0, -1, 0]), (2000, 1))
    hits, _ = o.trace(org, dirs, 0.01, 100.0)
    assert (hits["instance"] != abi.MISS).all()
    assert set(hits["instance"].tolist()) >= {0, 2}
    o.close()


def test_gltf_accessors_strided_and_normalised():
    """Accessor reads: interleaved views (byteStride), byte offsets, and
    normalised integer components (glTF 2.0: unsigned c / max, signed
    max(c / max, -1)); plain integers stay integers."""
    from vulkanexp_gb300.ingest import _accessor

    # interleaved (u16 u, u16 v, pad, f32 x) records of 12 bytes, at offset 4
    rec = np.zeros(3, dtype=[("u", "<u2"), ("v", "<u2"), ("pad", "<u4"), ("x", "<f4")])
    rec["u"] = [0, 32767, 65535]
    rec["v"] = [65535, 0, 1]
    rec["x"] = [1.5, -2.0, 3.25]
    blob = b"\0" * 4 + rec.tobytes()
    s8 = np.array([-128, -127, 0, 127], np.int8).tobytes()
    gl = {"bufferViews": [{"buffer": 0, "byteOffset": 4, "byteLength": rec.nbytes, "byteStride": 12},
                          {"buffer": 1, "byteOffset": 0, "byteLength": 4}],
          "accessors": [{"bufferView": 0, "componentType": 5123, "count": 3, "type": "VEC2", "normalized": True},
                        {"bufferView": 0, "byteOffset": 8, "componentType": 5126, "count": 3, "type": "SCALAR"},
                        {"bufferView": 0, "componentType": 5123, "count": 3, "type": "VEC2"},
                        {"bufferView": 1, "componentType": 5120, "count": 4, "type": "SCALAR", "normalized": True}]}
    bufs = [blob, s8]
    uv = _accessor(gl, bufs, 0)
    assert uv.dtype == np.float32
    np.testing.assert_allclose(uv, [[0.0, 1.0], [32767 / 65535, 0.0], [1.0, 1 / 65535]], rtol=1e-7)
    np.testing.assert_array_equal(_accessor(gl, bufs, 1)[:, 0], [1.5, -2.0, 3.25])
    raw = _accessor(gl, bufs, 2)
    assert raw.dtype == np.uint16 and raw.tolist() == [[0, 65535], [32767, 0], [65535, 1]]
    np.testing.assert_allclose(_accessor(gl, bufs, 3)[:, 0], [-1.0, -1.0, 0.0, 1.0], rtol=1e-7)

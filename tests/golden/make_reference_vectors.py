"""Writes tests/golden/reference_shaders.npz: input/output vectors of the
reference's own shader code, run on the host by oracle/_ref/libref_glsl.so
(the files of src/shaders compiled as C++, oracle/build_ref_glsl.py), so that
tests can pin the oracle and the CUDA path to the reference without its
sources present.

Cases (inputs seeded, numpy's legacy RandomState, whose streams are fixed):
* helper functions: sphericalFibonacci (irradiance.glsl:52-64) for
  N = 7, 64, 192, 256; octDecode and spherePointToOctohedralUV on points
  that include the octahedron's edges and corners;
  probeIndexToWorldPosition on two grids; pbrMetallicRoughness
  (pbrMetallicRoughness.glsl); sky (sky.glsl) from ground level to above the
  atmosphere, looking at and away from the sun; sampleProbes
  (irradiance.glsl:145-230) on a 3x2x3 grid with disabled probes, inside and
  outside the grid;
* the update passes (probesUpdate.glsl as probesUpdateIrradiance.comp and
  probesUpdateDepth.comp, then probesCopyBorders.comp) on given ray records:
  32 rays (all 12 listed probes), and 192 rays, where the irradiance pass
  loads only its 36 invocations' directions (probesUpdate.glsl:63-68), so
  only depth is kept;
* the probe trace (traceProbes.rgen, closesthit_noreflection.rchit,
  miss.rmiss, shadow.rmiss; hits found by the oracle's traversal) followed
  by the update passes, on two scenes: a closed room with 20 boxes (stored
  here), from a previous atlas of random texels and probe states, and
  tests/golden/editor_room.scene from a cleared atlas; 32 rays, every probe
  listed (the trace writes direction row i from the launch of list
  position i).

* the probe classification (probesInit.rgen with probeInitMiss.rmiss and
  backfaceTest.rchit): the room at 4x3x4 probes and 64 rays, the editor
  scene at 6x3x6 and 96 rays (512 rays per probe, directions past
  raysPerProbe degenerate, as the shader has them);
* the final gather (FinalGather.frag) of a 16 x 16 G-buffer against the
  room's updated atlas: random surface points, a quarter of the pixels sky,
  a camera at an exact position (so inverse(view) is exact) and a
  perspective projection.

* the probe selection (IrradianceProbes::selectProbesToUpdate, the
  reference's own C++ compiled from its source): 16 successive selections
  over 108 probes with random states (0 to 8) and caps 0 (none) to 100.

* genBasis (src/IrradianceProbes.cpp:347-355, compiled from its source
  over the reference's vendored GLM): 300 random unit vectors and the
  branch's edge (n.x at and around 0.9, the axes).

* the hysteresis ramp (the block of IrradianceProbes::update at
  src/IrradianceProbes.cpp:462-476, compiled from its source): 80 updates
  of 0 to 48 probes on a 48-probe grid from hysteresis 0 towards 0.98.

Atlases are reference-format (R11G11B10F colour, RG16F depth) and stored as
float16, which holds every value of both formats exactly.

Run with the root of a checkout of the reference sources as its argument:
    python tests/golden/make_reference_vectors.py <reference checkout>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "reference_shaders.npz")


def grid_words(g):
    import ctypes as C
    return np.frombuffer(C.string_at(C.addressof(g), C.sizeof(g)), np.uint32).copy()


def light_words(L):
    import ctypes as C
    return np.frombuffer(C.string_at(C.addressof(L), C.sizeof(L)), np.float32).copy()


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def reference_atlas(rng, grid):
    """A previous atlas of reference-format values (colour rgb + 1, depth)."""
    from oracle.oracle import Oracle, zero_atlas
    c, d = zero_atlas(grid)
    c[..., 0] = Oracle.round_store(0, rng.uniform(0, 1.5, c.shape[:2]).astype(np.float32))
    c[..., 1] = Oracle.round_store(0, rng.uniform(0, 1.5, c.shape[:2]).astype(np.float32))
    c[..., 2] = Oracle.round_store(1, rng.uniform(0, 1.5, c.shape[:2]).astype(np.float32))
    c[..., 3] = 1.0
    d[...] = Oracle.round_store(2, rng.uniform(0, 4, d.shape).astype(np.float32)).reshape(d.shape)
    return c, d


def helpers(rng, out):
    from oracle import ref_glsl as ref
    from vulkanexp_gb300 import abi
    for n in (7, 64, 192, 256):
        out["fib_%d" % n] = np.stack([ref.spherical_fibonacci(i, n) for i in range(n)])
    q = rng.uniform(-1, 1, size=(400, 2)).astype(np.float32)
    edges = np.array([[1, 0], [0, 1], [-1, 0], [0, -1], [0.5, 0.5], [-0.5, 0.5], [0.5, -0.5], [-0.5, -0.5],
                      [1, 1], [-1, -1], [1, -1], [-1, 1], [0, 0], [0.25, -0.75], [-0.75, 0.25]], np.float32)
    out["oct_decode_in"] = np.concatenate([q, edges])
    out["oct_decode_out"] = np.stack([ref.oct_decode(x, y) for x, y in out["oct_decode_in"]])
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    diag = np.array([[1, 1, 0], [1, 0, -1], [0, -1, 1], [-1, -1, -1], [1, 1, 1]], np.float32)
    diag = diag / np.linalg.norm(diag, axis=1, keepdims=True)
    out["oct_uv_in"] = np.concatenate([unit(rng, 400), axes, diag.astype(np.float32)])
    out["oct_uv_out"] = np.stack([ref.sphere_to_oct_uv(d) for d in out["oct_uv_in"]])
    for name, (lo, hi, res) in {"a": ((0, 0, 0), (10, 6, 10), (8, 4, 8)),
                                "b": ((-3.7, 0.25, -12.0), (41.3, 7.75, 5.5), (7, 3, 5))}.items():
        g = abi.make_grid(lo, hi, res, 64)
        out["pos_grid_" + name] = grid_words(g)
        out["pos_out_" + name] = np.stack([ref.probe_world_position(g, i) for i in range(g.probe_count())])
    m = 300
    n, v, ldir = unit(rng, m), unit(rng, m), unit(rng, m)
    lc = rng.uniform(0, 4, (m, 3)).astype(np.float32)
    alb = np.concatenate([rng.uniform(0, 1, (m, 3)), np.ones((m, 1))], 1).astype(np.float32)
    mr = rng.uniform(0, 1, (m, 2)).astype(np.float32)
    mr[:20, 0] = 0.0
    mr[20:40, 0] = 1.0
    mr[40:60, 1] = 1.0
    mr[60:70, 1] = 0.02
    out["pbr_in"] = np.concatenate([n, v, lc, ldir, alb, mr], 1)
    out["pbr_out"] = np.stack([ref.pbr(r[0:3], r[3:6], r[6:9], r[9:12], r[12:16], r[16], r[17])
                               for r in out["pbr_in"]])
    m = 160
    org = np.stack([rng.uniform(-50, 50, m), rng.choice([0.0, 1.0, 30.0, 500.0, 4000.0], m),
                    rng.uniform(-50, 50, m)], 1).astype(np.float32)
    sun = unit(rng, m)
    sun[:, 1] = np.abs(sun[:, 1])
    d = unit(rng, m)
    d[:20] = sun[:20]  # looking at the sun
    col = rng.uniform(0.5, 3, (m, 3)).astype(np.float32)
    br = rng.uniform(0.5, 2, (m, 1)).astype(np.float32)
    out["sky_in"] = np.concatenate([org, d, sun, col, br], 1)
    out["sky_out"] = np.stack([ref.sky(r[0:3], r[3:6], r[6:9], r[9:12], r[12]) for r in out["sky_in"]])
    g = abi.make_grid((0, 0, 0), (6, 3, 8), (3, 2, 3), 64)
    c, d = reference_atlas(rng, g)
    st = rng.randint(0, 9, g.probe_count()).astype(np.uint32)
    st[:3] = 0
    st[3:] = np.maximum(st[3:], 1)
    m = 300
    pos = rng.uniform(-1, 9, size=(m, 3)).astype(np.float32)
    q = np.concatenate([pos, unit(rng, m), unit(rng, m)], 1)
    out["sp_grid"] = grid_words(g)
    out["sp_states"] = st
    out["sp_color"] = c[..., :3].astype(np.float16)
    out["sp_depth"] = d.astype(np.float16)
    out["sp_in"] = q
    out["sp_out"] = np.stack([ref.sample_probes(g, st, c, d, r[0:3], r[3:6], r[6:9]) for r in q])


def update_passes(rng, out):
    from oracle import ref_glsl as ref
    from oracle.oracle import Oracle
    from vulkanexp_gb300 import abi, scenes
    for R, nlist in ((32, 12), (192, 12)):
        g = abi.make_grid((0, 0, 0), (6, 3, 8), (3, 2, 3), R, precision=abi.PRECISION_REFERENCE_FORMAT)
        P = g.probe_count()
        lst = rng.permutation(P)[:nlist].astype(np.uint32)
        cell = float(np.linalg.norm([3.0, 3.0, 4.0]))
        rays = np.zeros((nlist, R, 4), np.float32)
        rays[..., :3] = rng.uniform(0, 2, (nlist, R, 3))
        kind = rng.randint(0, 4, (nlist, R))
        rays[..., 3] = np.where(kind == 0, -rng.uniform(0, 2, (nlist, R)),
                                np.where(kind == 1, rng.uniform(0, cell, (nlist, R)),
                                         np.where(kind == 2, rng.uniform(cell, 3 * cell, (nlist, R)), 1e27)))
        c, d = reference_atlas(rng, g)
        st = rng.randint(1, 9, P).astype(np.uint32)
        orient = scenes.random_orientation(int(rng.randint(0, 1 << 30)), 0).astype(np.float32)
        dirs = Oracle.direction_table(orient, R)
        k = "upd%d_" % R
        out[k + "grid"] = grid_words(g)
        out[k + "list"] = lst
        out[k + "rays"] = rays
        out[k + "orientation"] = orient.reshape(9)
        out[k + "dirs"] = dirs
        out[k + "states_in"] = st.copy()
        out[k + "color_in"] = c[..., :3].astype(np.float16)
        out[k + "depth_in"] = d.astype(np.float16)
        ref.probes_update(g, lst, rays, dirs, st, c, d)
        out[k + "states_out"] = st
        out[k + "color_out"] = c[..., :3].astype(np.float16)
        out[k + "depth_out"] = d.astype(np.float16)


def trace(rng, out):
    from oracle import ref_glsl as ref
    from oracle.oracle import Oracle, zero_atlas
    from vulkanexp_gb300 import abi, ingest, scenes
    room = scenes.room_with_boxes(int(rng.randint(0, 1 << 30)), 20)
    room.bounds = (np.zeros(3), np.array([10.0, 6.0, 10.0]))
    cases = {"room": (room, (3, 3, 4)),
             "editor": (ingest.load(os.path.join(HERE, "editor_room.scene")), (4, 3, 3))}
    Oracle.set_sky_mode(abi.SKY_ATMOSPHERE)
    for name, (sc, res) in cases.items():
        g = scenes.fit_grid(sc, res, 32, abi.PRECISION_REFERENCE_FORMAT)
        P = g.probe_count()
        L = scenes.default_light()
        lst = rng.permutation(P).astype(np.uint32)
        if name == "room":  # a previous atlas of random texels and states
            c, d = reference_atlas(rng, g)
            st = rng.randint(1, 9, P).astype(np.uint32)
        else:  # the first update: cleared atlas, every probe on
            c, d = zero_atlas(g)
            st = np.ones(P, np.uint32)
        orient = scenes.random_orientation(int(rng.randint(0, 1 << 30)), 0).astype(np.float32)
        k = "trace_%s_" % name
        if name == "room":
            for f in ("vertices", "indices", "meshes", "instances", "offsets", "materials"):
                out[k + f] = getattr(sc, f)
        out[k + "grid"] = grid_words(g)
        out[k + "light"] = light_words(L)
        out[k + "list"] = lst
        out[k + "orientation"] = orient.reshape(9)
        out[k + "states_in"] = st.copy()
        if name == "room":
            out[k + "color_in"] = c[..., :3].astype(np.float16)
            out[k + "depth_in"] = d.astype(np.float16)
        o = Oracle(sc)
        rays, rec, dirs = ref.trace_probes(o, sc, g, L, orient, lst, st, c, d)
        o.close()
        ref.probes_update(g, lst, rays, dirs, st, c, d)
        out[k + "rays"] = rays
        out[k + "trace_args"] = rec
        out[k + "dirs"] = dirs
        out[k + "states_out"] = st
        out[k + "color_out"] = c[..., :3].astype(np.float16)
        out[k + "depth_out"] = d.astype(np.float16)
    Oracle.set_sky_mode(abi.SKY_CONSTANT)


def probe_init(rng, out):
    from oracle import ref_glsl as ref
    from oracle.oracle import Oracle
    from vulkanexp_gb300 import ingest, scenes
    room = scenes.Scene(*[out["trace_room_" + f] for f in ("vertices", "indices", "meshes", "instances", "offsets",
                                                           "materials")])
    room.bounds = (np.zeros(3), np.array([10.0, 6.0, 10.0]))
    editor = ingest.load(os.path.join(HERE, "editor_room.scene"))
    for name, sc, res, R in (("room", room, (4, 3, 4), 64), ("editor", editor, (6, 3, 6), 96)):
        g = scenes.fit_grid(sc, res, R)
        orient = scenes.random_orientation(int(rng.randint(0, 1 << 30)), 0).astype(np.float32)
        o = Oracle(sc)
        out["init_%s_grid" % name] = grid_words(g)
        out["init_%s_orientation" % name] = orient.reshape(9)
        out["init_%s_states" % name] = ref.init_probes(o, sc, g, orient)
        o.close()


def gather_camera():
    """World-to-view (a translation to an exact camera position) and a
    perspective projection, row-major."""
    cam = np.array([4.25, 3.5, 2.0], np.float32)
    view = np.eye(4, dtype=np.float32)
    view[:3, 3] = -cam
    proj = np.zeros((4, 4), np.float32)
    proj[0, 0], proj[1, 1] = 1.0 / np.tan(0.5), 1.0 / np.tan(0.5)
    proj[2, 2], proj[2, 3], proj[3, 2] = 100.0 / (0.1 - 100.0), 10.0 / (0.1 - 100.0), -1.0
    return cam, view, proj


def final_gather(rng, out):
    from oracle import ref_glsl as ref
    W = H = 16
    N = W * H
    g = grid_from_words(out["trace_room_grid"])
    L = light_from_words(out["trace_room_light"])
    color = np.zeros(out["trace_room_color_out"].shape[:2] + (4,), np.float32)
    color[..., :3] = out["trace_room_color_out"].astype(np.float32)
    color[..., 3] = 1.0
    depth = out["trace_room_depth_out"].astype(np.float32)
    states = out["trace_room_states_out"]
    pos = rng.uniform([0.2, 0.2, 0.2], [9.8, 5.8, 9.8], (N, 3))
    dist = rng.uniform(0.5, 10, N)
    dist[rng.uniform(size=N) < 0.25] = 0.0  # sky
    gb = {"position_depth": np.concatenate([pos, dist[:, None]], 1),
          "normal_metalness": np.concatenate([rng.normal(size=(N, 3)), rng.uniform(0, 1, (N, 1))], 1),
          "albedo_roughness": np.concatenate([rng.uniform(0, 1, (N, 3)), rng.uniform(0.05, 1, (N, 1))], 1),
          "emissive": np.concatenate([rng.uniform(0, 0.2, (N, 3)), np.zeros((N, 1))], 1),
          "direct_light": np.concatenate([(rng.uniform(size=(N, 1)) > 0.3), np.zeros((N, 3))], 1),
          "reflection": np.concatenate([rng.uniform(0, 1, (N, 3)), np.ones((N, 1))], 1)}
    gb = {k: v.astype(np.float32).reshape(H, W, 4) for k, v in gb.items()}
    cam, view, proj = gather_camera()
    for k, v in gb.items():
        out["gather_" + k] = v
    out["gather_out"] = ref.final_gather(g, L, states, color, depth, gb, view, proj)


def grid_from_words(words):
    from vulkanexp_gb300 import abi
    return abi.GridDesc.from_buffer_copy(np.ascontiguousarray(words, np.uint32).tobytes())


def light_from_words(words):
    from vulkanexp_gb300 import abi
    return abi.Light.from_buffer_copy(np.ascontiguousarray(words, np.float32).tobytes())


def selection(rng, out):
    from oracle import ref_glsl as ref
    K, n = 16, 108
    states = rng.randint(0, 9, (K, n)).astype(np.uint32)
    caps = np.array([0, 40, 17, 0, 5, 60, 0, 1, 30, 0, 100, 7, 0, 25, 0, 50], np.uint32)
    lists, offsets = ref.select_sequence(states, caps)
    padded = np.full((K, n), 0xFFFFFFFF, np.uint32)
    for k, l in enumerate(lists):
        padded[k, :len(l)] = l
    out["sel_states"] = states
    out["sel_caps"] = caps
    out["sel_lists"] = padded
    out["sel_counts"] = np.array([len(l) for l in lists], np.uint32)
    out["sel_offsets"] = offsets


def basis(rng, out):
    from oracle import ref_glsl as ref
    n = unit(rng, 300)
    edge = []
    for x in (0.9, np.nextafter(np.float32(0.9), np.float32(1)), np.nextafter(np.float32(0.9), np.float32(0)), 0.95,
              -0.9):
        r = np.sqrt(1 - np.float64(x) ** 2)
        edge.append([x, r * 0.6, r * 0.8])
    edge += [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]]
    n = np.concatenate([n, np.asarray(edge, np.float32)]).astype(np.float32)
    out["basis_in"] = n
    out["basis_out"] = np.stack([np.concatenate(ref.gen_basis(v)) for v in n])


def ramp(rng, out):
    from oracle import ref_glsl as ref
    counts = rng.randint(0, 49, 80).astype(np.uint32)
    counts[:10] = 48
    u, p = ref.ramp_sequence(0.0, 0.98, 48, counts)
    out["ramp_counts"] = counts
    out["ramp_uniform"] = u
    out["ramp_param"] = p


def main(reference_root):
    from oracle import build_ref_glsl
    from oracle.oracle import build_oracle
    build_oracle()
    if build_ref_glsl.build(reference_root) is None:
        sys.exit("reference shaders not found under %s" % reference_root)
    rng = np.random.RandomState(20241204)
    out = {}
    helpers(rng, out)
    update_passes(rng, out)
    trace(rng, out)
    probe_init(rng, out)
    final_gather(rng, out)
    selection(rng, out)
    basis(rng, out)
    ramp(rng, out)
    np.savez_compressed(OUT, **out)
    print(OUT, "%d arrays, %d bytes" % (len(out), os.path.getsize(OUT)))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_reference_vectors.py <reference checkout>")
    main(sys.argv[1])

"""The oracle pinned to the reference's own shader code.

tests/golden/reference_shaders.npz holds input/output vectors of the
reference's src/shaders files compiled as C++ and run on the host
(oracle/build_ref_glsl.py; made by tests/golden/make_reference_vectors.py).
The oracle is checked against them here, on CPU:

* helper functions: octDecode, spherePointToOctohedralUV and
  probeIndexToWorldPosition bit for bit; the ray-direction table within one
  float step of sphericalFibonacci (the table's cos and sin are correctly
  rounded, the reference build's are the C library's float ones);
  pbrMetallicRoughness and sampleProbes within 2e-6 relative (the oracle
  writes pow(x, 3) and pow(x, 5) as products); sky within 1e-5 relative;
* the update passes (probesUpdateIrradiance/Depth + probesCopyBorders) on
  the same ray records: reference-format atlases and probe states bit for
  bit (at 192 rays the depth pass only: the reference's irradiance pass
  loads 36 directions, probesUpdate.glsl:63-68);
* the probe classification (probesInit.rgen + its miss and back-face
  stages): every state equal;
* the probe selection (IrradianceProbes::selectProbesToUpdate, the
  reference's C++ compiled from its source): every list and offset of a
  16-call sequence; genBasis (the reference's over its vendored GLM) against
  the C++ facade's, bit for bit; the hysteresis ramp of update() against
  the restatement that the GPU ramp tests use, bit for bit;
* the final gather (FinalGather.frag): surface pixels within 2e-6
  relative, sky pixels within 2e-5 (the view direction is the fixture's
  camera ray computed in double, the shader's in float);
* the probe trace (traceProbes.rgen + closest-hit + miss stages) on the
  same rays: hit distance bit for bit, radiance within 2e-6 relative; then
  the whole update (the oracle's own rays) against the reference's trace +
  passes: every texel within one step of its format (rounding maps values a
  few float ulps apart to neighbouring format values), at most 0.5 % of
  texels not bit-identical, probe states equal.

With the reference build present (oracle/_ref/libref_glsl.so), the same
comparisons run again on fresh random inputs."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, ingest, scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def vec():
    return np.load(os.path.join(GOLDEN, "reference_shaders.npz"))


def grid_from(words):
    return abi.GridDesc.from_buffer_copy(np.ascontiguousarray(words, np.uint32).tobytes())


def light_from(words):
    return abi.Light.from_buffer_copy(np.ascontiguousarray(words, np.float32).tobytes())


def atlas_from(v, key, grid):
    c, d = zero_atlas(grid)
    if key + "color_in" in v:
        c[..., :3] = v[key + "color_in"].astype(np.float32)
        c[..., 3] = 1.0
        d[...] = v[key + "depth_in"].astype(np.float32)
    return c, d


def rel(a, b, floor):
    return np.abs(a.astype(np.float64) - b) / np.maximum(np.abs(b.astype(np.float64)), floor)


def format_steps(a, b, mbits):
    """|a - b| in steps of a 5-bit-exponent float format at |b|."""
    step = 2.0 ** (np.floor(np.log2(np.maximum(np.abs(b.astype(np.float64)), 2.0 ** -14))) - mbits)
    return np.abs(a.astype(np.float64) - b) / step


def room_scene(v):
    sc = scenes.Scene(*[v["trace_room_" + f] for f in ("vertices", "indices", "meshes", "instances", "offsets",
                                                       "materials")])
    sc.bounds = (np.zeros(3), np.array([10.0, 6.0, 10.0]))
    return sc


# ---------------------------------------------------------------------------
# helper functions
# ---------------------------------------------------------------------------
def test_fibonacci_directions(vec):
    for n in (7, 64, 192, 256):
        t = Oracle.direction_table(np.eye(3, dtype=np.float32).reshape(9), n)[:, :3]
        ref = vec["fib_%d" % n]
        assert np.abs(t - ref).max() <= 2.4e-7, n
        assert (t == ref).all(axis=1).mean() >= 0.9, n


def test_octahedral_mapping_and_probe_positions(vec):
    out = np.stack([Oracle.oct_decode(x, y) for x, y in vec["oct_decode_in"]])
    assert (out.view(np.uint32) == vec["oct_decode_out"].view(np.uint32)).all()
    uv = np.stack([Oracle.sphere_to_oct_uv(d) for d in vec["oct_uv_in"]])
    assert (uv.view(np.uint32) == vec["oct_uv_out"].view(np.uint32)).all()
    for name in ("a", "b"):
        g = grid_from(vec["pos_grid_" + name])
        p = np.stack([Oracle.probe_world_position(g, i) for i in range(g.probe_count())])
        assert (p.view(np.uint32) == vec["pos_out_" + name].view(np.uint32)).all()


def test_pbr_and_sky(vec):
    out = np.stack([Oracle.pbr(r[0:3], r[3:6], r[6:9], r[9:12], r[12:15], r[16], r[17]) for r in vec["pbr_in"]])
    assert rel(out, vec["pbr_out"][:, :3], 1e-4).max() <= 2e-6
    sky = np.stack([Oracle.sky(r[0:3], r[3:6], r[6:9], r[9:12], r[12]) for r in vec["sky_in"]])
    assert rel(sky, vec["sky_out"], 1e-4).max() <= 1e-5
    assert (vec["sky_out"] > 0).any(axis=1).mean() > 0.5


def test_sample_probes(vec):
    g = grid_from(vec["sp_grid"])
    c, d = zero_atlas(g)
    c[..., :3] = vec["sp_color"].astype(np.float32)
    c[..., 3] = 1.0
    d[...] = vec["sp_depth"].astype(np.float32)
    out = np.stack([Oracle.sample_probes(g, vec["sp_states"], c, d, r[0:3], r[3:6], r[6:9]) for r in vec["sp_in"]])
    assert rel(out, vec["sp_out"], 1e-4).max() <= 2e-6


# ---------------------------------------------------------------------------
# update passes on given records
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("R", [32, 192])
def test_update_passes(vec, R):
    k = "upd%d_" % R
    g = grid_from(vec[k + "grid"])
    c, d = atlas_from(vec, k, g)
    st = vec[k + "states_in"].copy()
    assert (Oracle.direction_table(vec[k + "orientation"], R) == vec[k + "dirs"]).all()
    Oracle.blend(g, vec[k + "orientation"], vec[k + "rays"], c, d, st, probe_list=vec[k + "list"])
    assert (d.astype(np.float16).view(np.uint16) == vec[k + "depth_out"].view(np.uint16)).all()
    if R <= 36:
        assert (c[..., :3].astype(np.float16).view(np.uint16) == vec[k + "color_out"].view(np.uint16)).all()
        assert (st == vec[k + "states_out"]).all()


# ---------------------------------------------------------------------------
# probe trace, then the whole update
# ---------------------------------------------------------------------------
def trace_case(v, name):
    sc = room_scene(v) if name == "room" else ingest.load(os.path.join(GOLDEN, "editor_room.scene"))
    k = "trace_%s_" % name
    return sc, k, grid_from(v[k + "grid"]), light_from(v[k + "light"])


@pytest.mark.parametrize("name", ["room", "editor"])
def test_trace_stages(vec, name):
    sc, k, g, L = trace_case(vec, name)
    c, d = atlas_from(vec, k, g)
    st = vec[k + "states_in"].copy()
    args = vec[k + "trace_args"]
    o = Oracle(sc)
    Oracle.set_sky_mode(abi.SKY_ATMOSPHERE)
    try:
        out = o.shade_rays(g, L, st, c, d, args.reshape(-1, 8)).reshape(vec[k + "rays"].shape)
    finally:
        Oracle.set_sky_mode(abi.SKY_CONSTANT)
        o.close()
    ref = vec[k + "rays"]
    assert (out[..., 3].view(np.uint32) == ref[..., 3].view(np.uint32)).all()
    assert rel(out[..., :3], ref[..., :3], 1e-3).max() <= 2e-6
    # the trace's rays are the oracle's: origins, directions, [0.01, |extent|]
    R = g.rays_per_probe
    table = Oracle.direction_table(vec[k + "orientation"], R)
    assert np.abs(args[..., 3:6] - table[None, :, :3]).max() <= 2.4e-7
    assert np.abs(vec[k + "dirs"] - table).max() <= 2.4e-7
    for s, p in enumerate(vec[k + "list"]):
        assert (args[s, :, 0:3] == Oracle.probe_world_position(g, int(p))[None]).all()
    assert (args[..., 6] == np.float32(0.01)).all()
    hit = ref[..., 3] > 0
    assert 0.05 < hit.mean() < 0.999


@pytest.mark.parametrize("name", ["room", "editor"])
def test_whole_update(vec, name):
    sc, k, g, L = trace_case(vec, name)
    c, d = atlas_from(vec, k, g)
    st = vec[k + "states_in"].copy()
    o = Oracle(sc)
    Oracle.set_sky_mode(abi.SKY_ATMOSPHERE)
    try:
        o.update(g, L, vec[k + "orientation"], c, d, st, probe_list=vec[k + "list"])
    finally:
        Oracle.set_sky_mode(abi.SKY_CONSTANT)
        o.close()
    rc, rd = vec[k + "color_out"].astype(np.float32), vec[k + "depth_out"].astype(np.float32)
    for ch, mb in enumerate((6, 6, 5)):
        assert format_steps(c[..., ch], rc[..., ch], mb).max() <= 1.0 + 1e-9
    for ch in range(2):
        assert format_steps(d[..., ch], rd[..., ch], 10).max() <= 1.0 + 1e-9
    assert (c[..., :3] != rc).any(axis=-1).mean() <= 0.005
    assert (d != rd).any(axis=-1).mean() <= 0.005
    assert (st == vec[k + "states_out"]).all()


@pytest.mark.parametrize("name", ["room", "editor"])
def test_probe_classification(vec, name):
    sc = room_scene(vec) if name == "room" else ingest.load(os.path.join(GOLDEN, "editor_room.scene"))
    g = grid_from(vec["init_%s_grid" % name])
    o = Oracle(sc)
    st = o.init_probes(g, vec["init_%s_orientation" % name])
    o.close()
    ref = vec["init_%s_states" % name]
    assert (st == ref).all(), "%d of %d probe states differ" % ((st != ref).sum(), len(st))
    assert len(np.unique(ref)) >= 2


def gather_inputs(v):
    """The final-gather case: grid, light, the room's updated atlas and
    states, the G-buffer as N x 4 arrays (direct light N), and for sky pixels
    the view direction in position.xyz (the C ABI's convention), computed in
    double from the fixture's camera."""
    from golden.make_reference_vectors import gather_camera
    g, L = grid_from(v["trace_room_grid"]), light_from(v["trace_room_light"])
    c, d = zero_atlas(g)
    c[..., :3] = v["trace_room_color_out"].astype(np.float32)
    c[..., 3] = 1.0
    d[...] = v["trace_room_depth_out"].astype(np.float32)
    H, W = v["gather_out"].shape[:2]
    gb = {k: v["gather_" + k].reshape(-1, 4).copy() for k in ("position_depth", "normal_metalness",
                                                              "albedo_roughness", "emissive", "reflection")}
    gb["direct_light"] = v["gather_direct_light"].reshape(-1, 4)[:, 0].copy()
    cam, view, proj = gather_camera()
    p = np.arange(H * W)
    u, w = ((p % W) + 0.5) / W, ((p // W) + 0.5) / H
    q = (np.linalg.inv(proj.astype(np.float64)) @ np.stack([2 * u - 1, 2 * w - 1, np.zeros_like(u),
                                                            np.ones_like(u)])).T[:, :3]
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    sky = gb["position_depth"][:, 3] <= 0
    gb["position_depth"][sky, :3] = (np.linalg.inv(view.astype(np.float64))[:3, :3] @ q.T).T[sky]
    return g, L, c, d, v["trace_room_states_out"], gb, cam, sky


def test_final_gather(vec):
    g, L, c, d, st, gb, cam, sky = gather_inputs(vec)
    Oracle.set_sky_mode(abi.SKY_ATMOSPHERE)
    try:
        out = Oracle.final_gather(g, L, st, c, d, gb, cam)
    finally:
        Oracle.set_sky_mode(abi.SKY_CONSTANT)
    ref = vec["gather_out"].reshape(-1, 4)
    r = rel(out[:, :3], ref[:, :3], 1e-3)
    assert r[~sky].max() <= 2e-6 and r[sky].max() <= 2e-5
    assert 0.1 < sky.mean() < 0.5


def test_probe_selection(vec):
    """IrradianceProbes::selectProbesToUpdate, the reference's C++ compiled
    from its source: 16 successive selections with changing states and caps
    equal the restatement's, list and offset."""
    from oracle.oracle import select_probes
    off, loop = 0, 0
    for k in range(len(vec["sel_caps"])):
        picked, off, loop = select_probes(vec["sel_states"][k], off, loop, int(vec["sel_caps"][k]))
        assert np.array_equal(picked, vec["sel_lists"][k, :vec["sel_counts"][k]]), k
        assert off == vec["sel_offsets"][k], k


def test_gen_basis(vec, tmp_path):
    """The facade's genBasis (include/irradiance_probes.hpp) compiled here
    equals the reference's genBasis over its vendored GLM, bit for bit."""
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "gen_basis")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "native", "gen_basis.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], input=np.ascontiguousarray(vec["basis_in"], np.float32).tobytes(), capture_output=True,
                       check=True)
    got = np.frombuffer(r.stdout, np.float32).reshape(-1, 6)
    assert (got.view(np.uint32) == vec["basis_out"].view(np.uint32)).all()


def test_hysteresis_ramp(vec):
    """The hysteresis ramp restatement that holds the C ABI's device ramp
    (ReferenceRamp of test_gpu_hysteresis.py) equals the reference's own
    block of update(), uploaded value and GridParameters.hysteresis after
    each of 80 updates, bit for bit."""
    from test_gpu_hysteresis import ReferenceRamp
    r = ReferenceRamp(0.0, 0.98)
    for k, n in enumerate(vec["ramp_counts"]):
        u = r.update(int(n), 48)
        assert u == vec["ramp_uniform"][k] and r.param == vec["ramp_param"][k], k
    assert len(set(vec["ramp_uniform"].tolist())) > 10


def test_fixture_scene_is_current(vec):
    """The stored room is what the trace saw (its arrays are in the
    fixture), and the editor scene file still loads to the same arrays."""
    sc = ingest.load(os.path.join(GOLDEN, "editor_room.scene"))
    g = scenes.fit_grid(sc, (4, 3, 3), 32, abi.PRECISION_REFERENCE_FORMAT)
    assert bytes(g) == bytes(grid_from(vec["trace_editor_grid"]))


# ---------------------------------------------------------------------------
# the reference build itself, on fresh inputs
# ---------------------------------------------------------------------------
def _ref():
    from oracle import ref_glsl
    if not ref_glsl.available():
        pytest.skip("reference shader build absent (oracle/_ref/libref_glsl.so)")
    return ref_glsl


def test_live_helpers():
    ref = _ref()
    rng = np.random.default_rng(11)
    for _ in range(2000):
        d = rng.normal(size=3).astype(np.float32)
        d /= np.linalg.norm(d)
        assert (Oracle.sphere_to_oct_uv(d) == ref.sphere_to_oct_uv(d)).all()
        x, y = rng.uniform(-1, 1, 2)
        assert (Oracle.oct_decode(x, y) == ref.oct_decode(x, y)).all()
    for n in (32, 100, 512):
        t = Oracle.direction_table(np.eye(3, dtype=np.float32).reshape(9), n)[:, :3]
        r = np.stack([ref.spherical_fibonacci(i, n) for i in range(n)])
        assert np.abs(t - r).max() <= 2.4e-7


def test_live_update_passes():
    ref = _ref()
    rng = np.random.default_rng(12)
    for R, res in ((16, (4, 3, 5)), (36, (3, 3, 3))):
        g = abi.make_grid((0, 0, 0), (6, 4, 8), res, R, precision=abi.PRECISION_REFERENCE_FORMAT, hysteresis=0.9)
        P = g.probe_count()
        lst = rng.permutation(P)[: P // 2 + 1].astype(np.uint32)
        rays = np.zeros((len(lst), R, 4), np.float32)
        rays[..., :3] = rng.uniform(0, 3, rays[..., :3].shape)
        rays[..., 3] = np.where(rng.uniform(size=(len(lst), R)) < 0.3, -1.0, rng.uniform(-1, 8, (len(lst), R)))
        c, d = zero_atlas(g)
        c[..., :3] = Oracle.round_store(0, rng.uniform(0, 2, c[..., :3].shape).astype(np.float32)).reshape(
            c[..., :3].shape)
        c[..., 2] = Oracle.round_store(1, c[..., 2].copy())
        d[...] = Oracle.round_store(2, rng.uniform(0, 4, d.shape).astype(np.float32)).reshape(d.shape)
        st = rng.integers(1, 9, P).astype(np.uint32)
        orient = scenes.random_orientation(5, R)
        c2, d2, st2 = c.copy(), d.copy(), st.copy()
        Oracle.blend(g, orient, rays, c, d, st, probe_list=lst)
        ref.probes_update(g, lst, rays, Oracle.direction_table(orient, R), st2, c2, d2)
        assert (c[..., :3] == c2[..., :3]).all() and (d == d2).all() and (st == st2).all()


def test_live_trace_and_update():
    ref = _ref()
    w = scenes.room_workload(21, n_boxes=40, resolution=(4, 3, 4), rays=32,
                             precision=abi.PRECISION_REFERENCE_FORMAT)
    g, sc, L = w.grid, w.scene, w.light
    P = g.probe_count()
    rng = np.random.default_rng(13)
    lst = rng.permutation(P).astype(np.uint32)
    c, d = zero_atlas(g)
    st = np.ones(P, np.uint32)
    o = Oracle(sc)
    Oracle.set_sky_mode(abi.SKY_ATMOSPHERE)
    try:
        c2, d2, st2 = c.copy(), d.copy(), st.copy()
        for k in range(2):  # the second update reads the first one's atlas
            orient = w.orientation(k)
            rays, args, dirs = ref.trace_probes(o, sc, g, L, orient, lst, st2, c2, d2)
            ref.probes_update(g, lst, rays, dirs, st2, c2, d2)
            out = o.shade_rays(g, L, st, c, d, args.reshape(-1, 8)).reshape(rays.shape)
            assert (out[..., 3] == rays[..., 3]).all()
            assert rel(out[..., :3], rays[..., :3], 1e-3).max() <= 2e-6
            o.update(g, L, orient, c, d, st, probe_list=lst)
            for ch, mb in enumerate((6, 6, 5)):
                assert format_steps(c[..., ch], c2[..., ch], mb).max() <= 1.0 + 1e-9
            assert (c[..., :3] != c2[..., :3]).any(axis=-1).mean() <= 0.005
            assert (st == st2).all()
    finally:
        Oracle.set_sky_mode(abi.SKY_CONSTANT)
        o.close()


def test_live_probe_classification():
    ref = _ref()
    w = scenes.terrain_workload(3, resolution=(8, 4, 8), rays=128, n_instances=60, boxes_per_cluster=200, cells=64)
    o = Oracle(w.scene)
    for k in range(2):
        a = ref.init_probes(o, w.scene, w.grid, w.orientation(k))
        assert (a == o.init_probes(w.grid, w.orientation(k))).all()
    o.close()

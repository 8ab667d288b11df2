"""CPU checks of the oracle: pins against the reference's own tables and
known-answer tests derived from the shader math (no GPU)."""
import ctypes
import json
import os

import numpy as np
import pytest

from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_border_tables_match_reference():
    """The generalised border copy reproduces probesCopyBorders.comp's
    tables (8x8 colour, 16x16 depth) entry for entry, in order."""
    ref = json.load(open(os.path.join(GOLDEN, "border_tables.json")))
    for n, dst, src in ((8, "irradianceCopiesDst", "irradianceCopiesSrc"), (16, "depthCopiesDst", "depthCopiesSrc")):
        t = Oracle.border_table(n)
        ref_pairs = sorted(zip(map(tuple, ref[dst]), map(tuple, ref[src])))
        ours = sorted((tuple(r[:2]), tuple(r[2:])) for r in t)
        assert ours == ref_pairs
        # every border texel written exactly once, every source interior
        dsts = [tuple(r[:2]) for r in t]
        assert len(set(dsts)) == len(dsts) == 4 * (n - 1)
        assert all(1 <= r[2] <= n - 2 and 1 <= r[3] <= n - 2 for r in t)


def test_truncated_texel_constants():
    # probesUpdate.glsl:37,40 use 0.33333 and 0.142857, not 1/3 and 1/7
    assert Oracle.texel_scale(6) == np.float32(0.33333)
    assert Oracle.texel_scale(14) == np.float32(0.142857)
    assert Oracle.texel_scale(4) == np.float32(0.5)


def test_oct_decode_unit_and_roundtrip():
    for n in (6, 14):
        s = Oracle.texel_scale(n)
        for ty in range(n):
            for tx in range(n):
                x, y = s * (tx - 0.5 * (n - 1)), s * (ty - 0.5 * (n - 1))
                d = Oracle.oct_decode(x, y)
                assert abs(np.linalg.norm(d) - 1.0) < 1e-6
                u, v = Oracle.sphere_to_oct_uv(d)
                # spherePointToOctohedralUV o octDecode is the identity on texel centres
                assert abs((2 * u - 1) - x) < 2e-5 and abs((2 * v - 1) - y) < 2e-5


def fibonacci_float32(n):
    """irradiance.glsl:52-64 in float32, operation by operation (cos and sin
    of the float angle in float64, then rounded)."""
    f = np.float32
    i = np.arange(n, dtype=np.float32)
    phi_golden = f(np.sqrt(f(5.0))) * f(0.5) + f(0.5)
    a = i * (phi_golden - f(1.0))
    phi = (f(2.0) * f(3.1415926538)) * (a - np.floor(a))
    cos_t = f(1.0) - (f(2.0) * i + f(1.0)) * (f(1.0) / f(n))
    sin_t = np.sqrt(np.clip(f(1.0) - cos_t * cos_t, f(0.0), f(1.0)))
    x = np.cos(phi.astype(np.float64)).astype(np.float32) * sin_t
    y = np.sin(phi.astype(np.float64)).astype(np.float32) * sin_t
    return np.stack([x, y, cos_t], 1)


def test_spherical_fibonacci_table():
    """The unrotated table is the shader's float formula bit for bit
    (irradiance.glsl:52-64), and within the float rounding of i (PHI - 1)
    (2 pi i 2^-23 radians) of the real-number golden-angle spiral with
    z_i = 1 - (2i+1)/N; a rotation is mat3 * vec3 (traceProbes.rgen:36),
    column by column in float."""
    n = 256
    t = Oracle.direction_table(np.eye(3, dtype=np.float32).reshape(9), n)
    v32 = fibonacci_float32(n)
    assert (t[:, :3] == v32).all()
    assert (t[:, 3] == 1.0).all()
    i = np.arange(n)
    z = 1.0 - (2 * i + 1) / n
    phi = 2 * np.pi * np.mod(i * 0.6180339887498949, 1.0)
    s = np.sqrt(np.clip(1 - z * z, 0, 1))
    v = np.stack([np.cos(phi) * s, np.sin(phi) * s, z], 1)
    bound = 2 * np.pi * np.maximum(i, 1) * 2.0 ** -23 + 1e-6
    assert (np.abs(t[:, :3] - v).max(axis=1) <= bound).all()
    M = scenes.random_orientation(4, 2).reshape(3, 3).astype(np.float32)
    np.testing.assert_allclose(M @ M.T, np.eye(3), atol=1e-6)
    tr = Oracle.direction_table(M.reshape(9), n)
    rot = (M[:, 0][None, :] * v32[:, 0:1] + M[:, 1][None, :] * v32[:, 1:2]) + M[:, 2][None, :] * v32[:, 2:3]
    assert (tr[:, :3] == rot).all()


def _empty_scene():
    sc = scenes.room_with_boxes(5, n_boxes=0)
    sc.instances = sc.instances[:0]
    sc.offsets = sc.offsets[:1]
    return sc


def test_empty_scene_known_answer():
    """No geometry: every ray misses, so after one update from zero every
    interior colour texel is (1-h)*sky and every depth texel (1-h)*(c, c^2)
    with c = |cell| (misses count as depth c, probesUpdate.glsl:78-79)."""
    sc = _empty_scene()
    g = abi.make_grid((0, 0, 0), (4, 3, 5), (3, 3, 3), 64, hysteresis=0.9)
    L = scenes.default_light()
    o = Oracle(sc, threads=2)
    c, d = zero_atlas(g)
    st = np.ones(g.probe_count(), np.uint32)
    o.update(g, L, scenes.random_orientation(3, 0), c, d, st)
    sky = np.array(L.sky[:3], np.float32)
    h = 0.9
    cell = np.linalg.norm(np.array([4 / 2, 3 / 2, 5 / 2]))
    for p in range(g.probe_count()):
        x, y, z = p % 3, (p // 3) % 3, p // 9
        tile = y * 3 + x
        col = c[8 * z + 1:8 * z + 7, 8 * tile + 1:8 * tile + 7, :3]
        np.testing.assert_allclose(col, np.broadcast_to((1 - h) * sky, col.shape), rtol=2e-6)
        dep = d[16 * z + 1:16 * z + 15, 16 * tile + 1:16 * tile + 15]
        np.testing.assert_allclose(dep[..., 0], (1 - h) * cell, rtol=2e-6)
        np.testing.assert_allclose(dep[..., 1], (1 - h) * cell * cell, rtol=2e-6)
    # all rays out of range -> state 8 (probesUpdate.glsl:111-112)
    assert (st == 8).all()


def test_hysteresis_recurrence():
    """K updates of a constant scene from zero give (1 - h^K) * x."""
    sc = _empty_scene()
    g = abi.make_grid((0, 0, 0), (2, 2, 2), (2, 2, 2), 32, hysteresis=0.8)
    L = scenes.default_light()
    o = Oracle(sc, threads=2)
    c, d = zero_atlas(g)
    st = np.ones(g.probe_count(), np.uint32)
    K = 5
    for k in range(K):
        o.update(g, L, scenes.random_orientation(9, k), c, d, st)
    sky = np.array(L.sky[:3])
    np.testing.assert_allclose(c[1:7, 1:7, :3], np.broadcast_to((1 - 0.8 ** K) * sky, (6, 6, 3)), rtol=1e-5)


def test_single_triangle_exact_t_and_facing():
    """A triangle in the plane z = 2 seen along +z from the origin: t = 2;
    front-facing exactly when its normal points back at the ray."""
    from vulkanexp_gb300.abi import INSTANCE_DTYPE, MATERIAL_DTYPE, MESH_DTYPE, OFFSET_DTYPE

    for flip in (False, True):
        pos = np.array([[-1, -1, 2], [2, -1, 2], [-1, 2, 2]], np.float64)
        tri = np.array([0, 2, 1] if flip else [0, 1, 2], np.uint32)
        verts = scenes.make_vertices(pos, np.tile([0, 0, -1.0], (3, 1)))
        meshes = np.array([(0, 3, 0, 3)], MESH_DTYPE)
        inst = np.zeros(1, INSTANCE_DTYPE)
        inst[0]["transform"] = scenes.affine_3x4(np.eye(3), np.zeros(3))
        inst[0]["mask"] = 1
        sc = scenes.Scene(verts, tri, meshes, inst, np.zeros(1, OFFSET_DTYPE), np.zeros(1, MATERIAL_DTYPE))
        o = Oracle(sc, threads=1)
        hits, bary = o.trace(np.zeros((1, 3)), np.array([[0, 0, 1.0]]), 0.01, 100.0)
        assert hits[0]["instance"] == 0 and hits[0]["t"] == np.float32(2.0)
        n = np.cross(pos[tri[1]] - pos[tri[0]], pos[tri[2]] - pos[tri[0]])
        front = np.dot([0, 0, 1.0], n) < 0
        assert bool(hits[0]["backface"]) == (not front)
        # tmin/tmax are inclusive; beyond tmax is a miss
        assert o.trace(np.zeros((1, 3)), np.array([[0, 0, 1.0]]), 0.01, 2.0)[0][0]["t"] == np.float32(2.0)
        assert o.trace(np.zeros((1, 3)), np.array([[0, 0, 1.0]]), 0.01, 1.999)[0][0]["instance"] == abi.MISS


def test_tie_breaks_to_lowest_instance_and_primitive():
    """Two coincident instances of a box, hit through the centre of a face
    (on the diagonal shared by its two triangles): equal t everywhere, so the
    hit goes to the lowest instance, then the lowest primitive."""
    sc = scenes.room_with_boxes(11, n_boxes=2)
    sc.instances = sc.instances[1:3].copy()
    sc.instances[1]["transform"] = sc.instances[0]["transform"]
    o = Oracle(sc, threads=1)
    M = sc.instances[0]["transform"].reshape(3, 4).astype(np.float64)
    centre = M[:, 3]
    # face centre of the local +x face, approached along the face normal
    face = centre + M[:, 0] * 0.5
    normal = M[:, 0] / np.linalg.norm(M[:, 0])
    origin = face + 2.0 * normal
    hits, _ = o.trace(origin[None].astype(np.float32), (-normal)[None].astype(np.float32), 0.01, 100.0)
    assert hits[0]["instance"] == 0
    assert hits[0]["primitive"] == 0  # +x face = triangles 0, 1
    assert hits[0]["backface"] == 0


def test_fp32_matches_fp64_room():
    """The FP32 restatement stays within 1e-4 of the FP64 one on the small
    room workload (one update from zero)."""
    w = scenes.workload(0)
    o = Oracle(w.scene)
    c, d = zero_atlas(w.grid)
    st = np.ones(w.grid.probe_count(), np.uint32)
    o.update(w.grid, w.light, w.orientation(0), c, d, st)
    c64, d64 = zero_atlas(w.grid, fp64=True)
    st64 = np.ones(w.grid.probe_count(), np.uint32)
    o.update(w.grid, w.light, w.orientation(0), c64, d64, st64, fp64=True)
    from conftest import rel_err

    assert rel_err(c, c64, 1e-3).max() < 1e-4
    assert rel_err(d, d64, 1e-3).max() < 1e-4
    assert (st == st64).all()


def test_scene_generators_sizes():
    sc = scenes.room_with_boxes(1234)
    assert sc.triangle_count == 2412
    big = scenes.terrain_with_clusters(1235, n_instances=64, boxes_per_cluster=100, cells=64)
    assert big.unique_triangle_count == 64 * 64 * 2 + 8 * 100 * 12
    assert len(big.instances) == 65


@pytest.mark.parametrize("res", [(8, 16), (6, 14)])
def test_blend_entry_point_normalises(res):
    """Equal-radiance rays blend to that radiance times (1-h)."""
    g = abi.make_grid((0, 0, 0), (1, 1, 1), (2, 2, 2), 64, color_res=res[0], depth_res=res[1], hysteresis=0.5)
    rays = np.zeros((8, 64, 4), np.float32)
    rays[..., :3] = (0.25, 0.5, 1.0)
    rays[..., 3] = 0.1
    c, d = zero_atlas(g)
    st = np.ones(8, np.uint32)
    Oracle.blend(g, scenes.random_orientation(1, 0), rays, c, d, st)
    n = res[0]
    np.testing.assert_allclose(c[1:n - 1, 1:n - 1, :3], np.broadcast_to([0.125, 0.25, 0.5], (n - 2, n - 2, 3)),
                               rtol=1e-5)


def test_final_gather_known_answers():
    """FinalGather.frag with a zero atlas, no direct light and no
    reflection leaves the emissive term; misses return the sky radiance;
    with only direct light it is the GGX sun term."""
    from oracle.oracle import Oracle, zero_atlas
    from vulkanexp_gb300 import abi, scenes

    g = abi.make_grid((0, 0, 0), (4, 4, 4), (3, 3, 3), 32)
    L = scenes.default_light()
    c, d = zero_atlas(g)
    st = np.ones(g.probe_count(), np.uint32)
    n = 6
    rng = np.random.default_rng(1)
    gb = {"position_depth": np.column_stack([rng.uniform(0, 4, (n, 3)), [1, 1, 1, 0, -1, 1]]),
          "normal_metalness": np.column_stack([rng.normal(size=(n, 3)), rng.uniform(0, 1, n)]),
          "albedo_roughness": np.column_stack([rng.uniform(0, 1, (n, 3)), rng.uniform(0.1, 1, n)]),
          "emissive": np.column_stack([rng.uniform(0, 1, (n, 3)), np.zeros(n)]),
          "direct_light": np.zeros(n), "reflection": None}
    gb = {k: None if v is None else v.astype(np.float32) for k, v in gb.items()}
    out = Oracle.final_gather(g, L, st, c, d, gb, (2, 2, 9))
    hit = gb["position_depth"][:, 3] > 0
    assert np.array_equal(out[hit, :3], gb["emissive"][hit, :3])
    assert np.allclose(out[~hit, :3], np.asarray(L.sky[:3], np.float32), rtol=0, atol=0)
    gb["emissive"][:] = 0
    gb["direct_light"][:] = 1
    out = Oracle.final_gather(g, L, st, c, d, gb, (2, 2, 9))
    for i in np.flatnonzero(hit):
        p = gb["position_depth"][i, :3].astype(np.float64)
        nrm = gb["normal_metalness"][i, :3].astype(np.float64)
        nrm /= np.linalg.norm(nrm)
        v = np.array([2, 2, 9.0]) - p
        v /= np.linalg.norm(v)
        ref = np.zeros(3, np.float32)
        Oracle.lib().oracle_pbr(*[np.ascontiguousarray(x, np.float32).ctypes.data_as(ctypes.c_void_p) for x in
                                  (nrm, v, L.color[:3], L.direction[:3], gb["albedo_roughness"][i, :3])],
                                float(gb["normal_metalness"][i, 3]), float(gb["albedo_roughness"][i, 3]),
                                ref.ctypes.data_as(ctypes.c_void_p))
        assert np.allclose(out[i, :3], ref, rtol=1e-5, atol=1e-7)


def _small_float_values(mbits):
    """Every finite non-negative value of an unsigned float with a 5-bit
    exponent (bias 15) and `mbits` mantissa bits, ascending."""
    vals = [m / 2.0 ** mbits * 2.0 ** -14 for m in range(2 ** mbits)]
    for e in range(1, 31):
        vals += [(1 + m / 2.0 ** mbits) * 2.0 ** (e - 15) for m in range(2 ** mbits)]
    return np.array(vals, np.float64)


@pytest.mark.parametrize("kind,mbits", [(0, 6), (1, 5)])
def test_reference_format_rounding_r11_b10(kind, mbits):
    """ddgi_round_r11 / ddgi_round_b10 (the reference's B10G11R11_UFLOAT
    irradiance image) against a brute-force nearest-value search: round to
    nearest, ties to the even mantissa, negative values to 0, above the
    largest finite value (and its half-step) to infinity."""
    vals = _small_float_values(mbits)
    rng = np.random.default_rng(kind)
    x = np.concatenate([
        rng.uniform(0, 4, 20000), 10.0 ** rng.uniform(-8, 4.8, 20000), vals, (vals[1:] + vals[:-1]) / 2,
        -rng.uniform(0, 5, 100), [0.0, -0.0, 1e-30, 6.5e4, 7e4, np.inf, -np.inf]]).astype(np.float32)
    got = Oracle.round_store(kind, x)
    top = vals[-1] + (vals[-1] - vals[-2]) / 2  # at or above: infinity
    for xi, gi in zip(x.astype(np.float64), got.astype(np.float64)):
        if not xi > 0:
            want = 0.0 if xi <= 0 or xi == -np.inf else xi
        elif xi >= top:
            want = np.inf
        else:
            j = np.searchsorted(vals, xi)
            lo, hi = vals[max(j - 1, 0)], vals[min(j, len(vals) - 1)]
            if xi - lo < hi - xi:
                want = lo
            elif hi - xi < xi - lo:
                want = hi
            else:  # a tie: the value with the even mantissa (its index in the table)
                want = lo if (max(j - 1, 0) % 2 == 0) else hi
        assert gi == want, (xi, gi, want)
    assert np.isnan(Oracle.round_store(kind, np.array([np.nan], np.float32))).all()


def test_reference_format_rounding_half():
    """ddgi_round_half (the reference's RG16F depth image) equals IEEE
    float32 -> binary16 round-to-nearest-even conversion."""
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(0, 3, 50000), 10.0 ** rng.uniform(-9, 5, 50000) * rng.choice([-1, 1], 50000),
                        [0.0, -0.0, 65504.0, 65519.0, 65520.0, 1e6, -1e6, 5.96e-8, 2.98e-8, np.inf]]).astype(np.float32)
    got = Oracle.round_store(2, x)
    with np.errstate(over="ignore"):
        want = x.astype(np.float16).astype(np.float32)
    assert (got.view(np.uint32) == want.view(np.uint32)).all()


def test_atmospheric_sky_known_answers():
    """The restatement of sky.glsl (oracle sky mode 1) through the final
    gather's sky pixels (brightness 1, view direction in position.xyz):
    looking straight down from 10 m hits the planet 110 m below the
    atmosphere's reference, which returns max(0.1, sun.y) x 0.05 grey;
    looking up gives a blue sky (Rayleigh scattering: blue > green > red);
    the constant mode returns the light's sky radiance."""
    from vulkanexp_gb300 import scenes

    g = abi.make_grid((0, 0, 0), (1, 1, 1), (2, 2, 2), 8)
    L = scenes.default_light()
    states = np.ones(8, np.uint32)
    color = np.zeros((16, 32, 4), np.float32)
    depth = np.zeros((32, 64, 2), np.float32)
    dirs = np.array([[0, -1, 0], [0, 1, 0], [0.3, 0.2, 0.9]], np.float32)
    gb = {"position_depth": np.column_stack([dirs, np.zeros(3)]).astype(np.float32),
          "normal_metalness": np.zeros((3, 4), np.float32), "albedo_roughness": np.zeros((3, 4), np.float32),
          "emissive": np.zeros((3, 4), np.float32), "direct_light": np.zeros(3, np.float32)}
    origin = np.array([0.0, 10.0, 0.0], np.float32)
    try:
        Oracle.set_sky_mode(1)
        out = Oracle.final_gather(g, L, states, color, depth, gb, origin)
    finally:
        Oracle.set_sky_mode(0)
    sun = np.asarray(L.direction[:3], np.float64)
    sun /= np.linalg.norm(sun)
    np.testing.assert_allclose(out[0, :3], max(0.1, sun[1]) * 0.05, rtol=1e-5)
    assert out[1, 2] > out[1, 1] > out[1, 0] > 0.0
    assert np.isfinite(out).all() and (out[2, :3] > 0).all()
    const = Oracle.final_gather(g, L, states, color, depth, gb, origin)
    assert (const[:, :3] == np.asarray(L.sky[:3], np.float32)).all()

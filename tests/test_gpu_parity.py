"""Parity of the CUDA path against the CPU oracle (GPU tests).

Bar: closest-hit instance/primitive IDs, hit distance and facing are
bit-identical; ray records and atlas texels agree within 1e-4 relative
(|gpu - oracle| <= 1e-4 * max(|oracle|, FLOOR) with FLOOR = 1e-2, the
magnitude below which a texel is compared absolutely)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context, DDGIError

pytestmark = pytest.mark.gpu

TOL = 1e-4
FLOOR = 1e-2


PIPELINES = [abi.PIPELINE_FUSED, abi.PIPELINE_WAVEFRONT]


def make_ctx(w, record_hits=True, pipeline=abi.PIPELINE_WAVEFRONT):
    ctx = Context(w.grid)
    ctx.set_pipeline(pipeline)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    if record_hits:
        ctx.record_hits(True)
    return ctx


def assert_hits_equal(gh, oh):
    assert gh.shape == oh.shape
    mism = (gh["instance"] != oh["instance"]) | (gh["primitive"] != oh["primitive"])
    assert not mism.any(), "hit-ID mismatch on %d of %d rays" % (mism.sum(), mism.size)
    hit = oh["instance"] != abi.MISS
    assert (gh["t"][hit].view(np.uint32) == oh["t"][hit].view(np.uint32)).all(), "t not bit-identical"
    assert (gh["backface"][hit] == oh["backface"][hit]).all()


def random_rays(rng, lo, hi, n):
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def test_trace_rays_bit_exact_room(gpu_lib, room_workload, room_oracle):
    w = room_workload
    ctx = make_ctx(w, record_hits=False)
    rng = np.random.default_rng(7)
    o, d = random_rays(rng, (-1, -1, -1), (11, 7, 11), 20000)
    for any_hit in (False, True):
        gh, gb = ctx.trace_rays(o, d, 0.01, 100.0, 0xFF, any_hit)
        oh, ob = room_oracle.trace(o, d, 0.01, 100.0, 0xFF, any_hit)
        if any_hit:
            assert ((gh["instance"] == abi.MISS) == (oh["instance"] == abi.MISS)).all()
        else:
            assert_hits_equal(gh, oh)
            hit = oh["instance"] != abi.MISS
            assert (gb[hit].view(np.uint32) == ob[hit].view(np.uint32)).all()
    ctx.close()


def test_trace_rays_masks_and_tmin(gpu_lib, room_workload, room_oracle):
    w = room_workload
    ctx = make_ctx(w, record_hits=False)
    rng = np.random.default_rng(8)
    o, d = random_rays(rng, (0, 0, 0), (10, 6, 10), 4000)
    for mask, tmin, tmax in ((0x2, 0.01, 50.0), (0x1, 0.5, 3.0), (0xFF, 0.0, 1e4)):
        gh, _ = ctx.trace_rays(o, d, tmin, tmax, mask)
        oh, _ = room_oracle.trace(o, d, tmin, tmax, mask)
        assert_hits_equal(gh, oh)
    ctx.close()


def run_updates(w, k_updates, probe_list=None, pipeline=abi.PIPELINE_WAVEFRONT):
    ctx = make_ctx(w, pipeline=pipeline)
    o = Oracle(w.scene)
    c, d = zero_atlas(w.grid)
    st = np.ones(w.grid.probe_count(), np.uint32)
    n = w.grid.probe_count() if probe_list is None else len(probe_list)
    for k in range(k_updates):
        ctx.update(w.orientation(k), probe_list)
        ctx.synchronize()
        rays, hits = o.update(w.grid, w.light, w.orientation(k), c, d, st, probe_list, want_rays=True,
                              want_hits=True)
        gh = ctx.get_hits(n)
        assert_hits_equal(gh, hits)
        gr = ctx.get_ray_records(n)
        assert rel_err(gr, rays, FLOOR).max() <= TOL, "ray records, update %d" % k
    gc = ctx.get_atlas(abi.ATLAS_COLOR)
    gd = ctx.get_atlas(abi.ATLAS_DEPTH)
    gs = ctx.get_probe_states()
    ctx.close()
    return gc, gd, gs, c, d, st


@pytest.mark.parametrize("pipeline", PIPELINES)
def test_update_room_one_step_from_zero(gpu_lib, room_workload, pipeline):
    gc, gd, gs, c, d, st = run_updates(room_workload, 1, pipeline=pipeline)
    assert rel_err(gc, c, FLOOR).max() <= TOL
    assert rel_err(gd, d, FLOOR).max() <= TOL
    assert (gs == st).all()


@pytest.mark.parametrize("pipeline", PIPELINES)
def test_update_room_three_steps_bounce(gpu_lib, pipeline):
    """Later updates read the previous atlas through sampleProbes."""
    w = scenes.room_workload(99, n_boxes=60, resolution=(6, 5, 6), rays=96)
    gc, gd, gs, c, d, st = run_updates(w, 3, pipeline=pipeline)
    assert rel_err(gc, c, FLOOR).max() <= TOL
    assert rel_err(gd, d, FLOOR).max() <= TOL
    assert (gs == st).all()


def test_update_probe_subset(gpu_lib):
    w = scenes.room_workload(5, n_boxes=80, resolution=(5, 4, 5), rays=64)
    rng = np.random.default_rng(3)
    plist = rng.permutation(w.grid.probe_count())[:37].astype(np.uint32)
    gc, gd, gs, c, d, st = run_updates(w, 2, plist)
    assert rel_err(gc, c, FLOOR).max() <= TOL
    assert rel_err(gd, d, FLOOR).max() <= TOL
    assert (gs == st).all()


@pytest.mark.parametrize("color_res,depth_res,rays", [(6, 14, 256), (8, 16, 1), (10, 18, 1024)])
def test_update_resolutions_and_ray_counts(gpu_lib, color_res, depth_res, rays):
    w = scenes.room_workload(21, n_boxes=40, resolution=(3, 3, 3), rays=rays, color_res=color_res,
                             depth_res=depth_res)
    gc, gd, gs, c, d, st = run_updates(w, 2)
    assert rel_err(gc, c, FLOOR).max() <= TOL
    assert rel_err(gd, d, FLOOR).max() <= TOL


@pytest.mark.parametrize("pipeline", PIPELINES)
def test_empty_scene_is_sky(gpu_lib, pipeline):
    sc = scenes.room_with_boxes(5, n_boxes=0)
    sc.instances = sc.instances[:0]
    g = abi.make_grid((0, 0, 0), (4, 3, 5), (3, 3, 3), 64, hysteresis=0.9)
    L = scenes.default_light()
    ctx = Context(g)
    ctx.set_pipeline(pipeline)
    ctx.build_scene(sc)
    ctx.set_light(L)
    ctx.update(scenes.random_orientation(3, 0))
    ctx.synchronize()
    c = ctx.get_atlas(abi.ATLAS_COLOR)
    np.testing.assert_allclose(c[1:7, 1:7, :3], np.broadcast_to(0.1 * np.array(L.sky[:3]), (6, 6, 3)), rtol=2e-6)
    ctx.close()


@pytest.mark.parametrize("pipeline", PIPELINES)
def test_terrain_subset_bit_exact_hits(gpu_lib, pipeline):
    """At-scale scene (terrain + 4096 box-cluster instances, ~1M unique
    triangles): one update from zero on a random subset of 256 probes."""
    w = scenes.workload(1)
    rng = np.random.default_rng(11)
    plist = np.sort(rng.permutation(w.grid.probe_count())[:256]).astype(np.uint32)
    gc, gd, gs, c, d, st = run_updates(w, 1, plist, pipeline=pipeline)
    assert rel_err(gc, c, FLOOR).max() <= TOL
    assert rel_err(gd, d, FLOOR).max() <= TOL


def test_errors_are_reported(gpu_lib, room_workload):
    ctx = Context(room_workload.grid)
    with pytest.raises(DDGIError) as e:
        ctx.update(np.eye(3, dtype=np.float32))
    assert e.value.status == 4  # no scene
    ctx.build_scene(room_workload.scene)
    with pytest.raises(DDGIError):
        ctx.update(np.eye(3, dtype=np.float32), np.array([0, 0], np.uint32))  # duplicate probe
    with pytest.raises(DDGIError):
        ctx.update(np.eye(3, dtype=np.float32), np.array([10 ** 6], np.uint32))
    bad = room_workload.scene
    idx = bad.indices.copy()
    idx[5] = 10 ** 7
    broken = scenes.Scene(bad.vertices, idx, bad.meshes, bad.instances, bad.offsets, bad.materials)
    with pytest.raises(DDGIError):
        ctx.build_scene(broken)
    ctx.synchronize(timeout_ms=10000)
    ctx.close()


@pytest.mark.parametrize("tuning", [
    dict(node_width=2), dict(node_width=2, rays_per_warp=8, smem_stack=16),
    dict(rays_per_warp=32), dict(rays_per_warp=8, refill_lanes=16), dict(rays_per_warp=1, smem_stack=16),
    dict(rays_per_warp=4, refill_lanes=1, ctas_per_sm=3, smem_stack=24),
    dict(straggler_lanes=0), dict(straggler_lanes=31), dict(straggler_lanes=3, node_width=8),
    dict(straggler_lanes=16, rays_per_warp=8, smem_stack=16),
])
def test_trace_tunings_do_not_change_results(gpu_lib, room_workload, tuning):
    """Work order, refill, stack placement and occupancy change only the
    schedule: hits, records and atlases stay bit-identical."""
    w = room_workload
    ref = make_ctx(w)
    ref.update(w.orientation(0))
    ctx = make_ctx(w)
    ctx.set_trace_tuning(**tuning)
    assert ctx.trace_tuning() == {**ctx.trace_tuning(), **tuning}
    ctx.update(w.orientation(0))
    n = w.grid.probe_count()
    assert (ctx.get_hits(n) == ref.get_hits(n)).all()
    assert (ctx.get_ray_records(n).view(np.uint32) == ref.get_ray_records(n).view(np.uint32)).all()
    for kind in (abi.ATLAS_COLOR, abi.ATLAS_DEPTH):
        assert (ctx.get_atlas(kind).view(np.uint32) == ref.get_atlas(kind).view(np.uint32)).all()
    ref.close()
    ctx.close()


def test_autotune_restores_state(gpu_lib, room_workload):
    w = room_workload
    ctx = make_ctx(w)
    ctx.update(w.orientation(0))
    before = [ctx.get_atlas(k) for k in (abi.ATLAS_COLOR, abi.ATLAS_DEPTH)] + [ctx.get_probe_states()]
    chosen = ctx.autotune(w.orientation(1), reps=1)
    assert ctx.trace_tuning() == chosen
    after = [ctx.get_atlas(k) for k in (abi.ATLAS_COLOR, abi.ATLAS_DEPTH)] + [ctx.get_probe_states()]
    for a, b in zip(before, after):
        assert (a == b).all()
    with pytest.raises(DDGIError):
        ctx.set_trace_tuning(rays_per_warp=3)
    with pytest.raises(DDGIError):
        ctx.set_trace_tuning(node_width=4)
    with pytest.raises(DDGIError):
        ctx.set_trace_tuning(straggler_lanes=32)
    ctx.close()

"""Batched update of many probe volumes (ddgi_batch_*), GPU tests.

A batch update must give every volume the atlases and probe states that
ddgi_update of that volume alone gives (same kernels' arithmetic on the same
hits): compared here texel by texel, bit for bit, for graph replay and plain
launches, for several launch tunings, across two successive updates (the
second one reads the bounce lighting of the first), on volumes mixing both
generators, FP32 and BF16 forms, 8/16 and 6/14 tiles and 64..512 rays.  One
FP32 volume is also checked directly against the CPU oracle (1e-4 relative,
as the single-volume parity tests)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Batch, Context, DDGIError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def volumes():
    ws = scenes.batch_workloads(seed=4242, count=7, tri_range=(2000, 40000))
    # one small FP32 room that the oracle checks directly
    ws.append(scenes.room_workload(77, n_boxes=120, resolution=(5, 4, 5), rays=64))
    return ws


def make_ctx(w):
    ctx = Context(w.grid)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    return ctx


def orientations(ws, k):
    return np.stack([scenes.random_orientation(w.seed, k) for w in ws])


def atlases(ctx):
    return (ctx.get_atlas(abi.ATLAS_COLOR), ctx.get_atlas(abi.ATLAS_DEPTH), ctx.get_probe_states())


def run_single(ws, K):
    out = []
    for w in ws:
        ctx = make_ctx(w)
        for k in range(K):
            ctx.update(orientations([w], k)[0])
        ctx.synchronize()
        out.append(atlases(ctx))
        ctx.close()
    return out


def assert_same(a, b, what):
    for x, y, name in zip(a, b, ("colour", "depth", "states")):
        assert x.shape == y.shape
        bad = x.view(np.uint32) != y.view(np.uint32) if x.dtype == np.float32 else x != y
        assert not bad.any(), "%s: %s differs on %d of %d values" % (what, name, bad.sum(), bad.size)


@pytest.fixture(scope="module")
def single_results(gpu_lib, volumes):
    return run_single(volumes, 2)


def test_forms_are_mixed(volumes):
    assert {w.grid.precision for w in volumes} == {abi.PRECISION_FP32, abi.PRECISION_BF16}
    assert {w.grid.color_res for w in volumes} == {6, 8}


@pytest.mark.parametrize("graph", [True, False])
def test_batch_equals_single_updates(gpu_lib, volumes, single_results, graph):
    ctxs = [make_ctx(w) for w in volumes]
    b = Batch(ctxs)
    b.use_graph(graph)
    assert b.ray_count == sum(w.grid.probe_count() * w.grid.rays_per_probe for w in volumes)
    for k in range(2):
        b.update(orientations(volumes, k))
    b.synchronize()
    for v, (ctx, ref) in enumerate(zip(ctxs, single_results)):
        assert_same(atlases(ctx), ref, "volume %d (%s)" % (v, volumes[v].name))
    ms = b.completion_ms()
    assert (ms > 0).all() and np.isfinite(ms).all()
    b.close()
    for c in ctxs:
        c.close()


@pytest.mark.parametrize("tuning", [
    dict(smem_stack=16, refill_lanes=4, trace_ctas_per_sm=4, blend_threads=64),
    dict(smem_stack=24, refill_lanes=32, trace_ctas_per_sm=0, blend_threads=128),
    dict(smem_stack=0, refill_lanes=1, trace_ctas_per_sm=2, blend_threads=256),
    dict(node_width=2, rays_per_warp=8, smem_stack=16),
    dict(straggler_lanes=0), dict(straggler_lanes=20, node_width=8),
    dict(blend_threads=0, refill_lanes=12), dict(blend_threads=32),
])
def test_tunings_do_not_change_results(gpu_lib, volumes, single_results, tuning):
    ctxs = [make_ctx(w) for w in volumes]
    b = Batch(ctxs)
    b.set_tuning(**tuning)
    assert b.tuning() == {**b.tuning(), **tuning}
    for k in range(2):
        b.update(orientations(volumes, k))
    b.synchronize()
    for v, (ctx, ref) in enumerate(zip(ctxs, single_results)):
        assert_same(atlases(ctx), ref, "volume %d with %s" % (v, tuning))
    b.close()
    for c in ctxs:
        c.close()


def test_autotune_restores_volumes_and_keeps_results(gpu_lib, volumes, single_results):
    ctxs = [make_ctx(w) for w in volumes]
    b = Batch(ctxs)
    b.update(orientations(volumes, 0))
    b.synchronize()
    before = [atlases(c) for c in ctxs]
    chosen = b.autotune(orientations(volumes, 5), reps=2)
    assert 1 <= chosen["refill_lanes"] <= 32 and chosen["blend_threads"] in (0, 64, 128, 256)
    assert b.tuning() == chosen
    for v, c in enumerate(ctxs):
        assert_same(atlases(c), before[v], "volume %d after autotune" % v)
    b.update(orientations(volumes, 1))
    b.synchronize()
    for v, (ctx, ref) in enumerate(zip(ctxs, single_results)):
        assert_same(atlases(ctx), ref, "volume %d after tuned update" % v)
    b.close()
    for c in ctxs:
        c.close()


def test_batch_volume_matches_oracle(gpu_lib, volumes):
    w = volumes[-1]
    ctxs = [make_ctx(x) for x in volumes]
    b = Batch(ctxs)
    b.update(orientations(volumes, 0))
    b.synchronize()
    o = Oracle(w.scene)
    c, d = zero_atlas(w.grid)
    st = np.ones(w.grid.probe_count(), np.uint32)
    o.update(w.grid, w.light, orientations([w], 0)[0], c, d, st)
    gc, gd, gs = atlases(ctxs[-1])
    assert rel_err(gc, c, 1e-2).max() <= 1e-4
    assert rel_err(gd, d, 1e-2).max() <= 1e-4
    assert (gs == st).all()
    b.close()
    for x in ctxs:
        x.close()


def test_rebuilt_scene_is_rejected(gpu_lib, volumes):
    ws = volumes[:2]
    ctxs = [make_ctx(w) for w in ws]
    b = Batch(ctxs)
    ctxs[1].build_scene(ws[1].scene)  # new device buffers: the arena copy is stale
    with pytest.raises(DDGIError) as e:
        b.update(orientations(ws, 0))
    assert e.value.status == 1
    b.close()
    for c in ctxs:
        c.close()


def test_invalid_tuning_rejected(gpu_lib, volumes):
    ctxs = [make_ctx(volumes[0])]
    b = Batch(ctxs)
    for bad in (dict(refill_lanes=0), dict(refill_lanes=33), dict(blend_threads=48), dict(smem_stack=200)):
        with pytest.raises(DDGIError):
            b.set_tuning(**bad)
    b.close()
    ctxs[0].close()


def test_ramping_volume_is_refused_until_the_ramp_is_off(gpu_lib, volumes, single_results):
    """The batch blends with each grid's hysteresis, so a volume with a
    hysteresis ramp (ddgi_set_target_hysteresis) is refused
    (DDGI_ERR_UNSUPPORTED) instead of drifting from its own ddgi_update;
    with the ramp off again the batch's result equals the single update."""
    w = volumes[-1]
    ctx = make_ctx(w)
    b = Batch([ctx])
    ctx.set_target_hysteresis(0.9)
    with pytest.raises(DDGIError) as e:
        b.update(orientations([w], 0))
    assert e.value.status == 7
    ctx.set_target_hysteresis(-1.0)
    for k in range(2):
        b.update(orientations([w], k))
    b.synchronize()
    assert_same(atlases(ctx), single_results[-1], "volume after its ramp was turned off")
    b.close()
    ctx.close()


def test_reference_format_volumes_in_a_batch(gpu_lib):
    """Volumes whose atlases are stored in the reference's image formats
    (R11G11B10F colour, RG16F depth) next to FP32 and BF16 volumes: each
    equal, bit for bit, to its own context updated alone."""
    ws = [scenes.room_workload(81, n_boxes=60, resolution=(4, 3, 4), rays=64,
                               precision=abi.PRECISION_REFERENCE_FORMAT),
          scenes.room_workload(82, n_boxes=40, resolution=(3, 3, 3), rays=128,
                               precision=abi.PRECISION_REFERENCE_FORMAT, color_res=6, depth_res=14),
          scenes.room_workload(83, n_boxes=50, resolution=(3, 4, 3), rays=64, precision=abi.PRECISION_BF16),
          scenes.room_workload(84, n_boxes=50, resolution=(4, 4, 3), rays=32)]
    single = run_single(ws, 2)
    ctxs = [make_ctx(w) for w in ws]
    b = Batch(ctxs)
    for k in range(2):
        b.update(orientations(ws, k))
    b.synchronize()
    for v, (ctx, ref) in enumerate(zip(ctxs, single)):
        assert_same(atlases(ctx), ref, "volume %d (%s)" % (v, ws[v].name))
    b.close()
    for c in ctxs:
        c.close()

"""Moving instances (ddgi_update_instances): after a top-level refit or
rebuild, closest hits are bit-identical to the oracle built from the moved
scene and to a fresh GPU build of it, and an update stays within 1e-4 of the
oracle."""
import copy

import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Batch, Context, DDGIError

pytestmark = pytest.mark.gpu


def moved(scene, rng, ids, shift=1.5):
    sc = copy.deepcopy(scene)
    for i in ids:
        m = sc.instances["transform"][i].reshape(3, 4).astype(np.float64)
        yaw = scenes.yaw_matrix(rng.uniform(0, 2 * np.pi))
        m[:, :3] = yaw @ m[:, :3]
        m[:, 3] += rng.uniform(-shift, shift, 3)
        sc.instances["transform"][i] = m.reshape(12).astype(np.float32)
    return sc


def make_ctx(w, scene):
    ctx = Context(w.grid)
    ctx.build_scene(scene)
    ctx.set_light(w.light)
    ctx.record_hits(True)
    return ctx


def hits_equal(a, b):
    same = (a["instance"] == b["instance"]) & (a["primitive"] == b["primitive"])
    hit = b["instance"] != abi.MISS
    same &= ~hit | ((a["t"].view(np.uint32) == b["t"].view(np.uint32)) & (a["backface"] == b["backface"]))
    return same


@pytest.mark.parametrize("rebuild", [False, True])
@pytest.mark.parametrize("which", ["room", "terrain"])
def test_moved_instances_match_oracle(gpu_lib, rebuild, which):
    if which == "room":
        w = scenes.room_workload(31, n_boxes=300, resolution=(6, 4, 6), rays=64)
    else:
        w = scenes.terrain_workload(1235, resolution=(6, 3, 6), rays=64, n_instances=400, boxes_per_cluster=300,
                                    cells=96)
    rng = np.random.default_rng(8)
    ni = len(w.scene.instances)
    ids = rng.choice(np.arange(1, ni), size=min(60, ni - 1), replace=False)
    sc2 = moved(w.scene, rng, ids)
    ctx = make_ctx(w, w.scene)
    ctx.update_instances(sc2.instances["transform"][ids], ids=ids, rebuild=rebuild)
    fresh = make_ctx(w, sc2)
    o = Oracle(sc2)
    lo, hi = sc2.bounds if which == "terrain" else (np.zeros(3), np.array([10.0, 6.0, 10.0]))
    orig = rng.uniform(lo - 1, hi + 1, size=(20000, 3)).astype(np.float32)
    d = rng.normal(size=(20000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    for any_hit in (False, True):
        g, _ = ctx.trace_rays(orig, d, 0.01, 500.0, 0xFF, any_hit)
        f, _ = fresh.trace_rays(orig, d, 0.01, 500.0, 0xFF, any_hit)
        r, _ = o.trace(orig, d, 0.01, 500.0, 0xFF, any_hit)
        if any_hit:
            assert ((g["instance"] == abi.MISS) == (r["instance"] == abi.MISS)).all()
        else:
            assert hits_equal(g, r).all(), "%d rays differ from the oracle" % (~hits_equal(g, r)).sum()
            assert hits_equal(g, f).all()
    # one probe update on the moved scene
    ctx.update(w.orientation(0))
    c, dd = zero_atlas(w.grid)
    st = np.ones(w.grid.probe_count(), np.uint32)
    o.update(w.grid, w.light, w.orientation(0), c, dd, st)
    assert rel_err(ctx.get_atlas(abi.ATLAS_COLOR), c, 1e-2).max() <= 1e-4
    assert rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), dd, 1e-2).max() <= 1e-4
    ctx.close()
    fresh.close()


def test_instance_update_errors_and_batch_invalidation(gpu_lib):
    w = scenes.room_workload(31, n_boxes=50, resolution=(4, 4, 4), rays=64)
    ctx = make_ctx(w, w.scene)
    t = w.scene.instances["transform"][[1, 2]].copy()
    with pytest.raises(DDGIError):
        ctx.update_instances(t, ids=[1, 1])
    with pytest.raises(DDGIError):
        ctx.update_instances(t, ids=[1, 999])
    bad = t.copy()
    bad[0, :] = 0.0  # singular
    with pytest.raises(DDGIError):
        ctx.update_instances(bad, ids=[1, 2])
    b = Batch([ctx])
    ctx.update_instances(t, ids=[1, 2])  # valid: the batch is now stale
    with pytest.raises(DDGIError):
        b.update(np.stack([w.orientation(0)]))
    b.close()
    ctx.close()


@pytest.mark.parametrize("build_mode", ["fast_trace", "fast_build"])
def test_mirrored_and_sheared_instances_match_oracle(gpu_lib, build_mode):
    """Instance transforms with a negative determinant (mirrors), uneven
    scales, shears and a nearly flat scale (1e-3): the world-to-object
    inverse is the host's double inverse rounded to float on both sides,
    and facing is decided in object space, where a mirroring instance
    transform does not change a triangle's winding (as in Vulkan ray
    tracing, whose instance transform leaves facing alone).  Closest hits
    bit-identical to the oracle's (instance, primitive, t, facing), any-hit
    agreement, and two probe updates within 1e-4."""
    w = scenes.room_workload(37, n_boxes=120, resolution=(5, 4, 5), rays=64)
    sc = copy.deepcopy(w.scene)
    rng = np.random.default_rng(12)
    forms = [np.diag([-1.0, 1.0, 1.0]), np.diag([1.0, -1.0, -1.0]) @ np.diag([1.0, 2.5, 0.3]),
             np.array([[1.0, 0.4, 0.0], [0.0, 1.0, 0.0], [0.3, 0.0, 1.0]]),
             np.array([[-0.7, 0.2, 0.1], [0.0, 1.3, -0.5], [0.2, 0.0, 0.9]]), np.diag([1.0, 1e-3, 1.0])]
    for i in range(1, len(sc.instances)):
        m = sc.instances["transform"][i].reshape(3, 4).astype(np.float64)
        m[:, :3] = m[:, :3] @ forms[i % len(forms)]
        sc.instances["transform"][i] = m.reshape(12).astype(np.float32)
    ctx = Context(w.grid)
    ctx.set_build_mode(build_mode)
    ctx.build_scene(sc)
    ctx.set_light(w.light)
    o = Oracle(sc)
    orig = rng.uniform(-1.0, 11.0, size=(20000, 3)).astype(np.float32)
    d = rng.normal(size=(20000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    for any_hit in (False, True):
        g, _ = ctx.trace_rays(orig, d, 0.01, 500.0, 0xFF, any_hit)
        r, _ = o.trace(orig, d, 0.01, 500.0, 0xFF, any_hit)
        if any_hit:
            assert ((g["instance"] == abi.MISS) == (r["instance"] == abi.MISS)).all()
        else:
            assert hits_equal(g, r).all(), "%d rays differ from the oracle" % (~hits_equal(g, r)).sum()
            mirrored = np.isin(r["instance"], [i for i in range(1, len(sc.instances))
                                               if np.linalg.det(forms[i % len(forms)]) < 0])
            assert (mirrored & (r["backface"] != 0)).any() and (mirrored & (r["backface"] == 0)).any()
    c, dd = zero_atlas(w.grid)
    st = np.ones(w.grid.probe_count(), np.uint32)
    for k in range(2):
        ctx.update(w.orientation(k))
        o.update(w.grid, w.light, w.orientation(k), c, dd, st)
    assert rel_err(ctx.get_atlas(abi.ATLAS_COLOR), c, 1e-2).max() <= 1e-4
    assert rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), dd, 1e-2).max() <= 1e-4
    assert (ctx.get_probe_states() == st).all()
    ctx.close()

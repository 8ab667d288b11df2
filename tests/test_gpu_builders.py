"""Tree builders (ddgi_set_build_mode): host SAH trees ("fast_trace") and GPU
linear BVHs ("fast_build") give closest hits bit-identical to the oracle and
to each other, for every leaf size, node width and after instance updates."""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from test_gpu_instances import hits_equal, moved
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context, DDGIError

pytestmark = pytest.mark.gpu


def workload(which):
    if which == "room":
        return scenes.room_workload(31, n_boxes=300, resolution=(6, 4, 6), rays=64)
    return scenes.terrain_workload(1235, resolution=(6, 3, 6), rays=64, n_instances=400, boxes_per_cluster=300,
                                   cells=96)


def context(w, scene, mode, leaf=2):
    ctx = Context(w.grid)
    ctx.set_build_mode(mode)
    ctx.set_leaf_size(leaf)
    ctx.build_scene(scene)
    ctx.set_light(w.light)
    ctx.record_hits(True)
    return ctx


def random_rays(w, which, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = w.scene.bounds if which == "terrain" else (np.zeros(3), np.array([10.0, 6.0, 10.0]))
    orig = rng.uniform(lo - 1, hi + 1, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    return orig, (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)


@pytest.mark.parametrize("leaf", [1, 2, 4])
@pytest.mark.parametrize("which", ["room", "terrain"])
def test_sah_trees_bit_exact(gpu_lib, which, leaf):
    w = workload(which)
    o = Oracle(w.scene)
    sah = context(w, w.scene, "fast_trace", leaf)
    lbvh = context(w, w.scene, "fast_build", leaf)
    orig, d = random_rays(w, which, 20000, 5)
    for any_hit in (False, True):
        r, _ = o.trace(orig, d, 0.01, 500.0, 0xFF, any_hit)
        for width in (2, 8):
            sah.set_trace_tuning(node_width=width)
            g, _ = sah.trace_rays(orig, d, 0.01, 500.0, 0xFF, any_hit)
            f, _ = lbvh.trace_rays(orig, d, 0.01, 500.0, 0xFF, any_hit)
            if any_hit:
                assert ((g["instance"] == abi.MISS) == (r["instance"] == abi.MISS)).all()
            else:
                assert hits_equal(g, r).all(), "%d rays differ from the oracle" % (~hits_equal(g, r)).sum()
                assert hits_equal(g, f).all()
    sah.set_trace_tuning(node_width=2)
    sah.update(w.orientation(0))
    c, dd = zero_atlas(w.grid)
    st = np.ones(w.grid.probe_count(), np.uint32)
    o.update(w.grid, w.light, w.orientation(0), c, dd, st)
    assert rel_err(sah.get_atlas(abi.ATLAS_COLOR), c, 1e-2).max() <= 1e-4
    assert rel_err(sah.get_atlas(abi.ATLAS_DEPTH), dd, 1e-2).max() <= 1e-4
    sah.close()
    lbvh.close()


@pytest.mark.parametrize("rebuild", [False, True])
def test_sah_top_level_after_instance_updates(gpu_lib, rebuild):
    w = workload("terrain")
    rng = np.random.default_rng(9)
    ni = len(w.scene.instances)
    ids = rng.choice(np.arange(1, ni), size=60, replace=False)
    sc2 = moved(w.scene, rng, ids)
    ctx = context(w, w.scene, "fast_trace")
    ctx.update_instances(sc2.instances["transform"][ids], ids=ids, rebuild=rebuild)
    o = Oracle(sc2)
    orig, d = random_rays(w, "terrain", 20000, 6)
    g, _ = ctx.trace_rays(orig, d, 0.01, 500.0, 0xFF, False)
    r, _ = o.trace(orig, d, 0.01, 500.0, 0xFF, False)
    assert hits_equal(g, r).all()
    ctx.close()


@pytest.mark.parametrize("overlap", [0.0, 1e-2, 1e-5])
@pytest.mark.parametrize("which", ["room", "terrain"])
def test_spatial_split_trees_bit_exact(gpu_lib, which, overlap):
    """Fast-trace mesh trees with spatial splits (triangles referenced from
    several leaves) give the oracle's closest and any hits bit for bit."""
    w = workload(which)
    o = Oracle(w.scene)
    ctx = Context(w.grid)
    ctx.set_spatial_splits(overlap)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    orig, d = random_rays(w, which, 20000, 12)
    for any_hit in (False, True):
        r, _ = o.trace(orig, d, 0.01, 500.0, 0xFF, any_hit)
        for width in (2, 8):
            ctx.set_trace_tuning(node_width=width)
            g, _ = ctx.trace_rays(orig, d, 0.01, 500.0, 0xFF, any_hit)
            if any_hit:
                assert ((g["instance"] == abi.MISS) == (r["instance"] == abi.MISS)).all()
            else:
                assert hits_equal(g, r).all(), "%d rays differ from the oracle" % (~hits_equal(g, r)).sum()
    with pytest.raises(DDGIError):
        ctx.set_spatial_splits(-1.0)
    ctx.close()


def test_build_mode_rejects_unknown(gpu_lib):
    w = workload("room")
    ctx = Context(w.grid)
    with pytest.raises(ValueError):
        ctx.set_build_mode("fastest")
    ctx.close()

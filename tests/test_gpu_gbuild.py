"""Fast-trace trees built on the GPU (gbuild.cu, build mode "fast_trace")
equal the host builders' trees (sah.cu / sbvh.cu, "fast_trace_host") node for
node: the same child boxes bit for bit, the same references, the same
triangles in the same leaf order, the same depths.  The GPU passes make every
decision with the host's arithmetic, so any difference is a bug.  Covered:
both scene generators (overlapping box clusters, where spatial splits are
taken, and a height field), leaf sizes 1/2/4, spatial splits off / default /
finer, and the full 1M-triangle terrain with 4,097 instances (whose top level
has a binned root above the sweep size)."""
import numpy as np
import pytest

from vulkanexp_gb300 import scenes
from vulkanexp_gb300.ddgi import Context

pytestmark = pytest.mark.gpu


def workload(which):
    if which == "room":
        return scenes.room_workload(31, n_boxes=300, resolution=(6, 4, 6), rays=64)
    if which == "terrain":
        return scenes.terrain_workload(1235, resolution=(6, 3, 6), rays=64, n_instances=400, boxes_per_cluster=300,
                                       cells=96)
    return scenes.workload(1)


def built(w, mode, leaf=2, alpha=1e-3):
    ctx = Context(w.grid)
    ctx.set_build_mode(mode)
    ctx.set_leaf_size(leaf)
    ctx.set_spatial_splits(alpha)
    ctx.build_scene(w.scene)
    out = ctx.read_trees(), ctx.scene_info()
    ctx.close()
    return out


def assert_same_trees(w, leaf, alpha):
    (gn, gt), gi = built(w, "fast_trace", leaf, alpha)
    (hn, ht), hi = built(w, "fast_trace_host", leaf, alpha)
    for k in ("nodes", "tri_refs", "depth_blas", "depth_tlas"):
        assert gi[k] == hi[k], "%s: GPU %d, host %d" % (k, gi[k], hi[k])
    bad = (gn != hn).any(axis=1)
    assert not bad.any(), "%d of %d nodes differ, first at %d" % (bad.sum(), len(bad), int(np.argmax(bad)))
    badt = (gt != ht).any(axis=1)
    assert not badt.any(), "%d of %d leaf triangles differ" % (badt.sum(), len(badt))
    assert gi["tree_build_ms"] > 0.0 and hi["tree_build_ms"] == 0.0
    return gi


@pytest.mark.parametrize("leaf", [1, 2, 4])
@pytest.mark.parametrize("which", ["room", "terrain"])
def test_gpu_trees_equal_host_trees(gpu_lib, which, leaf):
    assert_same_trees(workload(which), leaf, 1e-3)


@pytest.mark.parametrize("alpha", [0.0, 1e-4])
def test_gpu_trees_equal_host_trees_split_settings(gpu_lib, alpha):
    assert_same_trees(workload("terrain"), 2, alpha)


def test_gpu_trees_equal_host_trees_full_terrain(gpu_lib):
    info = assert_same_trees(workload("full"), 2, 1e-3)
    print("full terrain: %d nodes, %d triangle references, GPU mesh-tree build %.1f ms"
          % (info["nodes"], info["tri_refs"], info["tree_build_ms"]))

"""Fast-trace trees built on the GPU (gbuild.cu, build mode "fast_trace")
equal the host builders' trees (sah.cu / sbvh.cu, "fast_trace_host") node for
node: the same child boxes bit for bit, the same references, the same
triangles in the same leaf order, the same depths.  The GPU passes make every
decision with the host's arithmetic, so any difference is a bug.  Covered:
both scene generators (overlapping box clusters, where spatial splits are
taken, and a height field), leaf sizes 1/2/4, spatial splits off / default /
finer, the full 1M-triangle terrain with 4,097 instances (whose top level
has a binned root above the sweep size), and edge cases: meshes of one to
three triangles, fifty coincident triangles (no split plane: halved),
a flat grid (zero extent along an axis), crossing slivers, coordinates
near 1e5, and 4,600 instances a third of which coincide; hits through the
GPU-built trees of the edge cases equal the oracle's."""
import numpy as np
import pytest

from vulkanexp_gb300 import abi, scenes
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


# ---------------------------------------------------------------------------
# edge cases: tiny meshes, coincident and flat geometry, large coordinates, a
# top level above the sweep size with coincident instances
# ---------------------------------------------------------------------------
def custom_scene(meshes, instances, seed=5):
    """Scene of (positions n x 3, triangles m x 3) meshes and (mesh, 3x4
    transform) instances."""
    from vulkanexp_gb300.abi import INSTANCE_DTYPE, MESH_DTYPE, OFFSET_DTYPE
    rng = np.random.default_rng(seed)
    pos, idx, mrec = [], [], np.zeros(len(meshes), MESH_DTYPE)
    vo = io = 0
    for k, (p, t) in enumerate(meshes):
        p = np.asarray(p, np.float32)
        t = np.asarray(t, np.uint32).reshape(-1)
        mrec[k] = (vo, len(p), io, t.size)
        pos.append(p)
        idx.append(t)
        vo += len(p)
        io += t.size
    P = np.concatenate(pos)
    nrm = np.tile(np.array([[0.0, 1.0, 0.0]], np.float32), (len(P), 1))
    inst = np.zeros(len(instances), INSTANCE_DTYPE)
    offs = np.zeros(len(instances), OFFSET_DTYPE)
    for i, (m, tr) in enumerate(instances):
        inst[i]["transform"] = tr
        inst[i]["custom_index"] = i
        inst[i]["mask"] = 1
        inst[i]["mesh_index"] = m
        offs[i] = (i % 4, mrec[m]["vertex_offset"], mrec[m]["index_offset"])
    sc = scenes.Scene(scenes.make_vertices(P, nrm), np.concatenate(idx), mrec, inst, offs,
                      scenes.make_materials(rng, 4, 0.2, 0.8))
    sc.bounds = scenes.scene_bounds(sc)
    return sc


def soup(rng, n, lo, hi, size):
    c = rng.uniform(lo, hi, size=(n, 1, 3))
    p = (c + rng.uniform(-size, size, size=(n, 3, 3))).reshape(-1, 3)
    return p, np.arange(3 * n).reshape(-1, 3)


def edge_case_scene():
    rng = np.random.default_rng(99)
    one = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]]), [[0, 1, 2]])
    two = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.5]]), [[0, 1, 2], [1, 3, 2]])
    three = soup(rng, 3, -1, 1, 0.5)
    same = (np.array([[0, 0, 0], [2, 0, 0], [0, 2, 1]] * 50), np.arange(150).reshape(-1, 3))  # coincident
    g = np.stack(np.meshgrid(np.arange(11.0), np.arange(11.0), indexing="ij"), -1).reshape(-1, 2)
    flat_p = np.concatenate([g, np.zeros((len(g), 1))], 1)  # zero extent along z
    q = np.arange(100).reshape(10, 10)
    flat_t = np.concatenate([np.stack([q[:-1, :-1], q[1:, :-1], q[:-1, 1:]], -1).reshape(-1, 3),
                             np.stack([q[1:, :-1], q[1:, 1:], q[:-1, 1:]], -1).reshape(-1, 3)])
    flat_t = np.where(flat_t >= 0, flat_t + (flat_t // 10), flat_t)  # rows of 11 vertices
    slivers_p = []
    for k in range(120):  # long thin triangles crossing each other
        a = rng.uniform(-5, 5, 3)
        b = rng.uniform(-5, 5, 3)
        slivers_p += [a, b, a + rng.normal(0, 1e-3, 3)]
    slivers = (np.array(slivers_p), np.arange(360).reshape(-1, 3))
    far = soup(rng, 400, 1e5, 1e5 + 4.0, 0.6)  # large coordinates
    meshes = [one, two, three, same, (flat_p, flat_t), slivers, far]
    eye = scenes.affine_3x4(np.eye(3), np.zeros(3))
    instances = [(m, scenes.affine_3x4(scenes.yaw_matrix(0.3 * m), np.array([3.0 * m, 0.0, 0.0])))
                 for m in range(6)]
    instances.append((6, eye))
    return custom_scene(meshes, instances)


def many_instances_scene():
    """4,600 instances (a binned top-level root above the 4,096-instance
    sweep), a third of them at coincident positions."""
    rng = np.random.default_rng(7)
    box = soup(rng, 20, -0.5, 0.5, 0.3)
    instances = []
    for i in range(4600):
        t = rng.uniform(-40, 40, 3) if i % 3 else np.array([1.0, 2.0, 3.0])
        instances.append((0, scenes.affine_3x4(scenes.yaw_matrix(rng.uniform(0, 6.3)), t)))
    return custom_scene([box], instances)


@pytest.mark.parametrize("which", ["edge_cases", "many_instances"])
@pytest.mark.parametrize("leaf", [1, 2])
def test_gpu_trees_equal_host_trees_edge_cases(gpu_lib, which, leaf):
    from oracle.oracle import Oracle
    from test_gpu_instances import hits_equal
    sc = edge_case_scene() if which == "edge_cases" else many_instances_scene()
    g = scenes.fit_grid(sc, (3, 3, 3), 64)

    class W:
        pass
    w = W()
    w.grid, w.scene = g, sc
    assert_same_trees(w, leaf, 1e-3)
    # hits through the GPU-built trees against the oracle
    ctx = Context(g)
    ctx.set_leaf_size(leaf)
    ctx.build_scene(sc)
    rng = np.random.default_rng(3)
    if which == "edge_cases":  # around the meshes near the origin and around the far one
        orig = np.concatenate([rng.uniform(-6, 20, size=(14000, 3)), rng.uniform(1e5 - 2, 1e5 + 6, size=(6000, 3))])
    else:
        orig = rng.uniform(-42, 42, size=(20000, 3))
    orig = orig.astype(np.float32)
    d = rng.normal(size=(20000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    o = Oracle(sc)
    for any_hit in (False, True):
        r, _ = o.trace(orig, d, 0.0, 1e6, 0xFF, any_hit)
        h, _ = ctx.trace_rays(orig, d, 0.0, 1e6, 0xFF, any_hit)
        if any_hit:
            assert ((h["instance"] == abi.MISS) == (r["instance"] == abi.MISS)).all()
        else:
            assert hits_equal(h, r).all(), "%d rays differ from the oracle" % (~hits_equal(h, r)).sum()
            assert (r["instance"] != abi.MISS).mean() > 0.01
    ctx.close()
    o.close()

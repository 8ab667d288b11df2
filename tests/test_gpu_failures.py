"""Failure detection and checkpoints, without a GPU fault:

* a tensor-core completion wait that nothing ends (the one-shot test hook
  issues no MMA) gives up within its time limit, the host reads
  DDGI_ERR_DEVICE ("device wait timed out"), the failed update leaves the
  atlas untouched and the context keeps working;
* atlas checkpoints (ddgi_atlas_save / ddgi_atlas_load) restore a context
  bit for bit and refuse files that do not fit;
* scene input the reference would pass to the driver unchecked: triangles
  with a non-finite vertex are refused, degenerate triangles never hit."""
import copy
import os
import time

import numpy as np
import pytest

from oracle.oracle import Oracle
from test_gpu_instances import hits_equal
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context, DDGIError

pytestmark = pytest.mark.gpu


def small_room(precision):
    return scenes.room_workload(51, n_boxes=60, resolution=(4, 4, 4), rays=64, precision=precision)


def context(w):
    ctx = Context(w.grid)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    return ctx


def atlases(ctx):
    return ctx.get_atlas(abi.ATLAS_COLOR), ctx.get_atlas(abi.ATLAS_DEPTH), ctx.get_probe_states()


def test_stalled_tensor_wait_times_out_and_context_recovers(gpu_lib):
    w = small_room(abi.PRECISION_BF16)
    ctx, ref = context(w), context(w)
    ctx.update(w.orientation(0))
    ref.update(w.orientation(0))
    before = atlases(ctx)
    ctx.inject_fault(abi.FAULT_STALL_TENSOR_WAIT)
    t0 = time.perf_counter()
    ctx.update(w.orientation(1))
    with pytest.raises(DDGIError) as e:
        ctx.synchronize(timeout_ms=20000)
    elapsed = time.perf_counter() - t0
    assert e.value.status == abi.ERR_DEVICE and "timed out" in str(e.value)
    assert elapsed < 10.0
    after = atlases(ctx)
    for a, b in zip(before, after):  # the failed blend wrote nothing
        assert np.array_equal(a, b)
    # the hook was one-shot: the next update works and equals a context that
    # never ran the failed one
    ctx.update(w.orientation(2))
    ref.update(w.orientation(2))
    ctx.synchronize(timeout_ms=20000)
    for a, b in zip(atlases(ctx), atlases(ref)):
        assert np.array_equal(a, b)
    assert np.isfinite(after[0]).all()
    ctx.close()
    ref.close()


def test_inject_fault_rejects_unknown_bits(gpu_lib):
    w = small_room(abi.PRECISION_BF16)
    ctx = Context(w.grid)
    with pytest.raises(DDGIError) as e:
        ctx.inject_fault(0x80)
    assert e.value.status == 1
    ctx.close()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP32, abi.PRECISION_BF16])
def test_checkpoint_roundtrip(gpu_lib, tmp_path, precision):
    w = small_room(precision)
    a = context(w)
    for k in range(3):
        a.update(w.orientation(k))
    path = os.path.join(str(tmp_path), "atlas.ckpt")
    a.save_atlas(path)
    b = context(w)
    b.load_atlas(path)
    for x, y in zip(atlases(a), atlases(b)):
        assert np.array_equal(x, y)
    # resuming from the checkpoint continues exactly (FP16 atlases resume
    # from their FP32 accumulators too)
    a.update(w.orientation(3))
    b.update(w.orientation(3))
    for x, y in zip(atlases(a), atlases(b)):
        assert np.array_equal(x, y)
    a.close()
    b.close()


def test_checkpoint_refuses_files_that_do_not_fit(gpu_lib, tmp_path):
    w = small_room(abi.PRECISION_FP32)
    a = context(w)
    a.update(w.orientation(0))
    path = os.path.join(str(tmp_path), "atlas.ckpt")
    a.save_atlas(path)
    other = scenes.room_workload(51, n_boxes=60, resolution=(4, 4, 5), rays=64)
    b = Context(other.grid)
    c = Context(small_room(abi.PRECISION_BF16).grid)
    for ctx in (b, c):
        with pytest.raises(DDGIError) as e:
            ctx.load_atlas(path)
        assert e.value.status == abi.ERR_IO
    data = open(path, "rb").read()
    for bad in (data[:-4], data + b"x", b"NOTATLAS" + data[8:]):
        with open(path, "wb") as f:
            f.write(bad)
        with pytest.raises(DDGIError) as e:
            a.load_atlas(path)
        assert e.value.status == abi.ERR_IO
    with pytest.raises(DDGIError) as e:
        a.load_atlas(os.path.join(str(tmp_path), "missing.ckpt"))
    assert e.value.status == abi.ERR_IO
    for ctx in (a, b, c):
        ctx.close()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP32, abi.PRECISION_BF16])
def test_raw_atlas_readback(gpu_lib, precision):
    """ddgi_get_atlas_raw returns the storage format (FP16 texels for the
    BF16 form), which widened equals ddgi_get_atlas bit for bit."""
    w = small_room(precision)
    ctx = context(w)
    ctx.update(w.orientation(0))
    for kind in (abi.ATLAS_COLOR, abi.ATLAS_DEPTH):
        raw = ctx.get_atlas_raw(kind)
        assert raw.dtype == (np.float16 if precision == abi.PRECISION_BF16 else np.float32)
        assert np.array_equal(raw.astype(np.float32).view(np.uint32), ctx.get_atlas(kind).view(np.uint32))
    with pytest.raises(AssertionError):
        ctx.get_atlas_raw(abi.ATLAS_COLOR, out=np.empty((1, 1, 4), np.float32))
    ctx.close()


def test_nonfinite_vertex_is_refused(gpu_lib):
    w = small_room(abi.PRECISION_FP32)
    sc = copy.deepcopy(w.scene)
    sc.vertices["pos"][sc.indices[5]] = (np.nan, 1.0, 1.0)
    ctx = Context(w.grid)
    with pytest.raises(DDGIError) as e:
        ctx.build_scene(sc)
    assert e.value.status == 1 and "not finite" in str(e.value)
    ctx.close()


@pytest.mark.parametrize("mode", ["fast_trace", "fast_build"])
def test_degenerate_triangles_never_hit(gpu_lib, mode):
    w = small_room(abi.PRECISION_FP32)
    sc = copy.deepcopy(w.scene)
    idx = sc.indices.reshape(-1, 3)
    rng = np.random.default_rng(3)
    pick = rng.choice(len(idx), size=len(idx) // 4, replace=False)
    idx[pick[0::2], 1] = idx[pick[0::2], 0]  # a repeated vertex: zero area
    idx[pick[1::2], 2] = idx[pick[1::2], 1]
    sc.indices = idx.reshape(-1).copy()
    ctx = Context(w.grid)
    ctx.set_build_mode(mode)
    ctx.build_scene(sc)
    o = Oracle(sc)
    orig = rng.uniform(-1, 11, size=(20000, 3)).astype(np.float32)
    d = rng.normal(size=(20000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    g, _ = ctx.trace_rays(orig, d, 0.01, 500.0, 0xFF, False)
    r, _ = o.trace(orig, d, 0.01, 500.0, 0xFF, False)
    assert hits_equal(g, r).all()
    hit = g["instance"] != abi.MISS
    degenerate = np.zeros(len(idx), bool)
    degenerate[pick] = True
    # triangle of each hit in the whole index array: its mesh's first triangle + primitive
    mesh = sc.instances["mesh_index"][g["instance"][hit]]
    tri = sc.meshes["index_offset"][mesh] // 3 + g["primitive"][hit]
    assert hit.sum() > 1000 and not degenerate[tri].any()
    ctx.close()

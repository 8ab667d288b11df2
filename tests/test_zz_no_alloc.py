"""ddgi_blend_records_noalloc, the allocation-free BF16 blend.

It is meant for callers that cannot allocate device memory when they blend
(an engine with a pre-reserved memory budget, a frame loop that must not call
cudaMalloc/cudaFree).  The caller owns every input and output buffer (here:
torch tensors); the entry point's own working memory is a fixed __device__
array.  Its results must match the context-based ddgi_blend_records on the
same inputs, over two calls in a row (the second call reuses the array the
first one left behind), within the tolerance of the other blend tests:
|a - b| <= 1e-4 * max(|b|, 1e-2).

This file is collected last on purpose, so that a run stopping at its first
failure has run every other test already; it also passes alone.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context, load_library

pytestmark = pytest.mark.gpu

TOL = 1e-4
FLOOR = 1e-2


def records(rng, n, R, cell):
    rec = np.zeros((n, R, 4), np.float32)
    kind = rng.integers(0, 3, size=(n, R))
    rad = rng.uniform(0.0, 2.0, size=(n, R, 3))
    t = rng.uniform(0.02, 2.0 * cell, size=(n, R))
    rec[..., :3] = np.where((kind == 1)[..., None], 0.0, rad)
    rec[..., 3] = np.where(kind == 2, -1.0, np.where(kind == 1, 0.8 * t, t))
    return rec


def call_noalloc(lib, grid, orientation, d_list, n, d_rec, d_states, d_color, d_depth, d_acc_c, d_acc_d, stream):
    o = np.ascontiguousarray(orientation, np.float32).reshape(9)
    return lib.ddgi_blend_records_noalloc(C.byref(grid), C.c_void_p(o.ctypes.data),
                                          C.c_void_p(d_list) if d_list else None, n, C.c_void_p(d_rec),
                                          C.c_void_p(d_states), C.c_void_p(d_color), C.c_void_p(d_depth),
                                          C.c_void_p(d_acc_c), C.c_void_p(d_acc_d), C.c_void_p(stream))


@pytest.mark.parametrize("rays,color_res,depth_res,use_list", [
    (256, 8, 16, True),
    # the largest request the fixed scratch takes: 1024 rays x (256 + 256)
    # texel rows = exactly 2 MB of weights, every probe (no list)
    (1024, 18, 18, False),
])
def test_noalloc_blend_matches_context_blend(gpu_lib, rays, color_res, depth_res, use_list):
    import torch

    g = abi.make_grid((0, 0, 0), (10, 6, 8), (6, 4, 5), rays, color_res=color_res, depth_res=depth_res,
                      hysteresis=0.9, depth_sharpness=50.0, precision=abi.PRECISION_BF16)
    P, R = g.probe_count(), g.rays_per_probe
    cell = float(np.linalg.norm([(g.extent_max[k] - g.extent_min[k]) / (g.resolution[k] - 1) for k in range(3)]))
    rng = np.random.default_rng(99 + rays)
    plist = rng.permutation(P)[: P - 7].astype(np.uint32) if use_list else None
    n = P if plist is None else len(plist)
    recs = [records(rng, n, R, cell) for _ in range(2)]
    orients = [scenes.random_orientation(31, k) for k in range(2)]

    # the existing entry point (a context that allocated its buffers)
    ctx = Context(g)
    for k in range(2):
        ctx.blend_records(orients[k], recs[k], plist)
    ref_c = ctx.get_atlas(abi.ATLAS_COLOR)
    ref_d = ctx.get_atlas(abi.ATLAS_DEPTH)
    ref_s = ctx.get_probe_states()
    ctx.close()

    # the allocation-free entry point on caller-owned device buffers
    dev = torch.device("cuda", torch.cuda.current_device())
    ch, cw, _ = g.atlas_shape(abi.ATLAS_COLOR)
    dh, dw, _ = g.atlas_shape(abi.ATLAS_DEPTH)
    color = torch.zeros((ch, cw, 4), dtype=torch.float16, device=dev)
    depth = torch.zeros((dh, dw, 2), dtype=torch.float16, device=dev)
    acc_c = torch.zeros((ch, cw, 4), dtype=torch.float32, device=dev)
    acc_d = torch.zeros((dh, dw, 2), dtype=torch.float32, device=dev)
    states = torch.ones(P, dtype=torch.int32, device=dev)
    d_list = torch.from_numpy(plist.view(np.int32)).to(dev) if plist is not None else None
    lib = load_library()
    stream = torch.cuda.current_stream().cuda_stream
    for k in range(2):
        d_rec = torch.from_numpy(recs[k]).to(dev)
        torch.cuda.synchronize()
        st = call_noalloc(lib, g, orients[k], d_list.data_ptr() if d_list is not None else 0, n, d_rec.data_ptr(),
                          states.data_ptr(),
                          color.data_ptr(), depth.data_ptr(), acc_c.data_ptr(), acc_d.data_ptr(), stream)
        assert st == 0, abi.STATUS_NAMES.get(st, st)
    torch.cuda.synchronize()
    got_c = color.float().cpu().numpy()
    got_d = depth.float().cpu().numpy()
    assert rel_err(got_c, ref_c, FLOOR).max() <= TOL
    assert rel_err(got_d, ref_d, FLOOR).max() <= TOL
    assert (states.cpu().numpy().view(np.uint32) == ref_s).all()


def test_noalloc_rejects_requests_beyond_its_scratch(gpu_lib):
    lib = load_library()
    eye = np.eye(3, dtype=np.float32)
    # interior tiles above 16 x 16 texels do not fit the fixed scratch, also
    # at the largest ray count (one step above the largest accepted request)
    for rays, cres, dres in ((64, 8, 20), (1024, 18, 19), (1024, 19, 18)):
        g = abi.make_grid((0, 0, 0), (1, 1, 1), (2, 2, 2), rays, color_res=cres, depth_res=dres,
                          precision=abi.PRECISION_BF16)
        st = call_noalloc(lib, g, eye, 0, 8, 1, 1, 1, 1, 1, 1, 0)
        assert st == 7  # DDGI_ERR_UNSUPPORTED, before touching any pointer
    g = abi.make_grid((0, 0, 0), (1, 1, 1), (1, 2, 2), 64, precision=abi.PRECISION_BF16)
    assert call_noalloc(lib, g, eye, 0, 8, 1, 1, 1, 1, 1, 1, 0) == 1  # invalid grid

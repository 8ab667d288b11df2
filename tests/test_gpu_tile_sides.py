"""The atlas blend at the smallest, odd and largest tile sides a grid
accepts (texels per probe side, border included: 3 .. 64), for each blend
kernel: the FP32 per-probe kernel (fused pipeline), the FP32 shared-weight
kernel (wavefront pipeline) and the BF16 tensor-core kernel (interiors up to
16 x 16 texels; a depth and a colour interior whose padded rows pass 256
take two accumulators); then whole updates, the final gather and a batch
of volumes with such tiles.

Side 3 leaves one interior texel that feeds all eight border texels, side 4
puts the first and last interior rows next to each other
(probesCopyBorders.comp:21-245 hard-codes the tables of sides 8 and 16; the
generalised tables follow the same rules for any side); odd sides publish
tile rows that are not whole 16-byte groups.

Bars as in test_gpu_bf16.py: the FP32 forms within 1e-4 relative (floor
1e-2) of the FP32 oracle with equal probe states; the BF16 form within 1e-3
(max) and 5e-4 (RMS) of the FP64 oracle (its probe states follow FP32
accumulators, so they are not compared with the FP64 oracle's)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Batch, Context
from test_gpu_bf16 import BF16_MAX, BF16_RMS, FLOOR, cell_len, synthetic_records

pytestmark = pytest.mark.gpu


def grid(precision, rays, color_res, depth_res):
    return abi.make_grid((0, 0, 0), (10, 6, 8), (3, 3, 2), rays, color_res=color_res, depth_res=depth_res,
                         hysteresis=0.9, depth_sharpness=50.0, precision=precision)


@pytest.mark.parametrize("pipeline", [abi.PIPELINE_FUSED, abi.PIPELINE_WAVEFRONT])
@pytest.mark.parametrize("color_res,depth_res,rays", [(3, 3, 64), (4, 5, 33), (7, 9, 64), (64, 64, 32)])
def test_blend_fp32_tile_sides(gpu_lib, pipeline, color_res, depth_res, rays):
    g = grid(abi.PRECISION_FP32, rays, color_res, depth_res)
    rng = np.random.default_rng(color_res * 100 + depth_res)
    ctx = Context(g)
    ctx.set_pipeline(pipeline)
    c, d = zero_atlas(g)
    st = np.ones(g.probe_count(), np.uint32)
    for k in range(2):
        rec = synthetic_records(rng, g.probe_count(), rays, cell_len(g))
        o = scenes.random_orientation(41, k)
        ctx.blend_records(o, rec)
        Oracle.blend(g, o, rec, c, d, st)
    assert rel_err(ctx.get_atlas(abi.ATLAS_COLOR), c, FLOOR).max() <= 1e-4
    assert rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), d, FLOOR).max() <= 1e-4
    assert (ctx.get_probe_states() == st).all()
    ctx.close()


@pytest.mark.parametrize("color_res,depth_res,rays", [(3, 3, 64), (4, 5, 33), (7, 9, 64), (18, 3, 48), (3, 18, 100)])
def test_blend_bf16_tile_sides(gpu_lib, color_res, depth_res, rays):
    g = grid(abi.PRECISION_BF16, rays, color_res, depth_res)
    rng = np.random.default_rng(color_res * 100 + depth_res + 7)
    ctx = Context(g)
    c, d = zero_atlas(g, fp64=True)
    st = np.ones(g.probe_count(), np.uint32)
    for k in range(3):
        rec = synthetic_records(rng, g.probe_count(), rays, cell_len(g))
        o = scenes.random_orientation(43, k)
        ctx.blend_records(o, rec)
        Oracle.blend(g, o, rec, c, d, st)
    ec = rel_err(ctx.get_atlas(abi.ATLAS_COLOR)[..., :3], c[..., :3], FLOOR)
    ed = rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), d, FLOOR)
    assert ec.max() <= BF16_MAX and ed.max() <= BF16_MAX
    assert np.sqrt((ec ** 2).mean()) <= BF16_RMS and np.sqrt((ed ** 2).mean()) <= BF16_RMS
    assert np.isfinite(ctx.get_atlas(abi.ATLAS_COLOR)).all() and np.isfinite(ctx.get_atlas(abi.ATLAS_DEPTH)).all()
    ctx.close()


@pytest.mark.parametrize("pipeline", [abi.PIPELINE_FUSED, abi.PIPELINE_WAVEFRONT])
@pytest.mark.parametrize("color_res,depth_res,rays", [(3, 3, 64), (5, 7, 32)])
def test_update_small_and_odd_tiles(gpu_lib, pipeline, color_res, depth_res, rays):
    """Whole updates (trace, shading with the bounce lookup into the
    previous atlas, blend) with small and odd tiles: the lookup's bilinear
    taps stay inside their probe's tile at every side, so its in-atlas
    indexing matches the oracle's REPEAT addressing there too; hits
    bit-exact, ray records and atlases within 1e-4."""
    from test_gpu_parity import TOL, run_updates

    w = scenes.room_workload(23, n_boxes=40, resolution=(3, 3, 3), rays=rays, color_res=color_res,
                             depth_res=depth_res)
    gc, gd, gs, c, d, st = run_updates(w, 3, pipeline=pipeline)
    assert rel_err(gc, c, FLOOR).max() <= TOL
    assert rel_err(gd, d, FLOOR).max() <= TOL
    assert (gs == st).all()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP32, abi.PRECISION_BF16])
@pytest.mark.parametrize("color_res,depth_res", [(3, 3), (5, 7)])
def test_final_gather_small_and_odd_tiles(gpu_lib, precision, color_res, depth_res):
    """The final gather's atlas lookups (FinalGather.frag) on small and odd
    tiles, after two updates: within 1e-4 of the oracle, sky pixels exact."""
    import torch

    from test_gpu_gather import random_gbuffer

    w = scenes.room_workload(29, n_boxes=40, resolution=(4, 3, 4), rays=64, color_res=color_res,
                             depth_res=depth_res)
    g = w.grid.copy()
    g.precision = precision
    ctx = Context(g)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    for k in range(2):
        ctx.update(w.orientation(k))
    color, depth = ctx.get_atlas(abi.ATLAS_COLOR), ctx.get_atlas(abi.ATLAS_DEPTH)
    states = ctx.get_probe_states()
    H, W = 48, 64
    gb = random_gbuffer(np.random.default_rng(color_res), H, W, (-0.5, -0.5, -0.5), (10.5, 6.5, 10.5))
    origin = np.array([5.0, 3.0, -2.0], np.float32)
    dev = {k: None if v is None else torch.from_numpy(v.reshape(H, W, -1).squeeze(-1) if v.ndim == 1 else
                                                       v.reshape(H, W, 4)).cuda().contiguous()
           for k, v in gb.items()}
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    ctx.final_gather(dev, origin, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(-1, 4)
    want = Oracle.final_gather(g, w.light, states, color, depth, gb, origin)
    sky = gb["position_depth"][:, 3] <= 0
    assert sky.any() and (got[sky, :3] == np.asarray(w.light.sky[:3], np.float32)).all()
    assert rel_err(got[:, :3], want[:, :3], FLOOR).max() <= 1e-4
    ctx.close()


@pytest.mark.parametrize("graph", [True, False])
def test_batch_with_small_and_odd_tiles(gpu_lib, graph):
    """A batch whose volumes have tiles of sides 3, 5/7, 18/3 and 8/16 in
    both precisions (the batch's FP32, shared-weight FP32 and tensor-core
    blend kernels at those sides): every volume's atlases and probe states
    equal, bit for bit, those of its own context updated alone, over two
    updates."""
    from test_gpu_batch import assert_same, atlases, make_ctx, orientations

    specs = [(3, 3, 64, abi.PRECISION_FP32), (5, 7, 32, abi.PRECISION_FP32), (3, 3, 64, abi.PRECISION_BF16),
             (18, 3, 48, abi.PRECISION_BF16), (5, 7, 100, abi.PRECISION_BF16), (8, 16, 64, abi.PRECISION_FP32)]
    ws = [scenes.room_workload(50 + i, n_boxes=30 + 10 * i, resolution=(3 + i % 2, 3, 4), rays=r, precision=p,
                               color_res=cr, depth_res=dr) for i, (cr, dr, r, p) in enumerate(specs)]
    single = []
    for w in ws:
        ctx = make_ctx(w)
        for k in range(2):
            ctx.update(orientations([w], k)[0])
        ctx.synchronize()
        single.append(atlases(ctx))
        ctx.close()
    ctxs = [make_ctx(w) for w in ws]
    b = Batch(ctxs)
    b.use_graph(graph)
    for k in range(2):
        b.update(orientations(ws, k))
    b.synchronize()
    for v, (ctx, ref) in enumerate(zip(ctxs, single)):
        assert_same(atlases(ctx), ref, "volume %d (%s, tiles %d/%d)" % (v, ws[v].name, specs[v][0], specs[v][1]))
    b.close()
    for c in ctxs:
        c.close()

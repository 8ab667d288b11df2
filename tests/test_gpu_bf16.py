"""The atlas blend on the GPU, alone: the FP32 SIMT kernel against the FP32
oracle, and the BF16 tensor-core (tcgen05) kernel against the FP64 oracle.

Bars: FP32 form |gpu - oracle| <= 1e-4 * max(|oracle|, 1e-2) per texel.
BF16 form (BF16 operands, FP32 accumulation, FP16 atlas): relative error
against FP64 at most BF16_MAX per texel and BF16_RMS as root-mean-square,
both with the same 1e-2 floor."""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context

pytestmark = pytest.mark.gpu

FLOOR = 1e-2
BF16_MAX = 1e-3
BF16_RMS = 5e-4


def synthetic_records(rng, n, R, cell):
    """Ray records with the reference's three kinds of rays: lit hits
    (radiance, t), backfaces (0, 0.8 t) and misses (sky, -1)."""
    rec = np.zeros((n, R, 4), np.float32)
    kind = rng.integers(0, 3, size=(n, R))
    rad = rng.uniform(0.0, 2.0, size=(n, R, 3)) * rng.uniform(0.1, 1.0, size=(n, 1, 1))
    t = rng.uniform(0.02, 2.0 * cell, size=(n, R))
    rec[..., :3] = np.where((kind == 1)[..., None], 0.0, rad)
    rec[..., 3] = np.where(kind == 2, -1.0, np.where(kind == 1, 0.8 * t, t))
    return rec


def grid_for(precision, rays=256, res=(6, 4, 5), color_res=8, depth_res=16):
    return abi.make_grid((0, 0, 0), (10, 6, 8), res, rays, color_res=color_res, depth_res=depth_res,
                         hysteresis=0.9, depth_sharpness=50.0, precision=precision)


def cell_len(g):
    return float(np.linalg.norm([(g.extent_max[k] - g.extent_min[k]) / (g.resolution[k] - 1) for k in range(3)]))


@pytest.mark.parametrize("rays", [256, 100])
def test_blend_fp32_matches_oracle(gpu_lib, rays):
    g = grid_for(abi.PRECISION_FP32, rays)
    rng = np.random.default_rng(rays)
    ctx = Context(g)
    c, d = zero_atlas(g)
    st = np.ones(g.probe_count(), np.uint32)
    for k in range(2):
        rec = synthetic_records(rng, g.probe_count(), rays, cell_len(g))
        o = scenes.random_orientation(17, k)
        ctx.blend_records(o, rec)
        Oracle.blend(g, o, rec, c, d, st)
    assert rel_err(ctx.get_atlas(abi.ATLAS_COLOR), c, FLOOR).max() <= 1e-4
    assert rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), d, FLOOR).max() <= 1e-4
    assert (ctx.get_probe_states() == st).all()
    ctx.close()


@pytest.mark.parametrize("rays,color_res,depth_res", [(256, 8, 16), (128, 6, 14), (512, 8, 16), (64, 8, 16)])
def test_blend_bf16_error_vs_fp64(gpu_lib, rays, color_res, depth_res):
    g = grid_for(abi.PRECISION_BF16, rays, color_res=color_res, depth_res=depth_res)
    rng = np.random.default_rng(rays + color_res)
    ctx = Context(g)
    c, d = zero_atlas(g, fp64=True)
    st = np.ones(g.probe_count(), np.uint32)
    for k in range(3):
        rec = synthetic_records(rng, g.probe_count(), rays, cell_len(g))
        o = scenes.random_orientation(23, k)
        ctx.blend_records(o, rec)
        Oracle.blend(g, o, rec, c, d, st)
    gc = ctx.get_atlas(abi.ATLAS_COLOR)
    gd = ctx.get_atlas(abi.ATLAS_DEPTH)
    ec = rel_err(gc[..., :3], c[..., :3], FLOOR)
    ed = rel_err(gd, d, FLOOR)
    print("bf16 blend rays=%d res=%d/%d: colour max %.2e rms %.2e, depth max %.2e rms %.2e"
          % (rays, color_res, depth_res, ec.max(), np.sqrt((ec ** 2).mean()), ed.max(), np.sqrt((ed ** 2).mean())))
    assert ec.max() <= BF16_MAX and ed.max() <= BF16_MAX
    assert np.sqrt((ec ** 2).mean()) <= BF16_RMS and np.sqrt((ed ** 2).mean()) <= BF16_RMS
    ctx.close()


def test_blend_bf16_tiny_and_zero_radiance(gpu_lib):
    """Probes whose largest radiance is zero, denormal or tiny: the per-probe
    scale of the BF16 operands stays finite, so the atlas has no NaN (an
    infinite reciprocal once turned 0 x inf into NaN for such a probe)."""
    g = grid_for(abi.PRECISION_BF16, 256)
    rng = np.random.default_rng(4)
    ctx = Context(g)
    c, d = zero_atlas(g, fp64=True)
    st = np.ones(g.probe_count(), np.uint32)
    rec = synthetic_records(rng, g.probe_count(), 256, cell_len(g))
    rec[0, :, :3] = 0.0
    rec[0, 7, 1] = 1e-39   # denormal maximum
    rec[1, :, :3] = 0.0
    rec[1, 3, 0] = 3e-36   # below the smallest scale
    rec[2, :, :3] = 0.0    # all zero
    rec[3, :, :3] *= 1e-20  # tiny but scaled
    o = scenes.random_orientation(29, 0)
    ctx.blend_records(o, rec)
    Oracle.blend(g, o, rec, c, d, st)
    gc = ctx.get_atlas(abi.ATLAS_COLOR)
    gd = ctx.get_atlas(abi.ATLAS_DEPTH)
    assert np.isfinite(gc).all() and np.isfinite(gd).all()
    assert rel_err(gc[..., :3], c[..., :3], FLOOR).max() <= BF16_MAX
    ctx.close()


def test_update_bf16_room_vs_fp64(gpu_lib):
    """Whole update in the BF16 form: hit IDs stay bit-exact (geometry is
    FP32), the atlas after three updates stays within the BF16 bars."""
    w = scenes.room_workload(77, n_boxes=80, resolution=(6, 5, 6), rays=128, precision=abi.PRECISION_BF16)
    ctx = Context(w.grid)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    ctx.record_hits(True)
    o = Oracle(w.scene)
    c, d = zero_atlas(w.grid, fp64=True)
    st = np.ones(w.grid.probe_count(), np.uint32)
    for k in range(3):
        ctx.update(w.orientation(k))
        ctx.synchronize()
        _, hits = o.update(w.grid, w.light, w.orientation(k), c, d, st, fp64=True, want_hits=True)
        gh = ctx.get_hits(w.grid.probe_count())
        assert (gh["instance"] == hits["instance"]).all() and (gh["primitive"] == hits["primitive"]).all()
    ec = rel_err(ctx.get_atlas(abi.ATLAS_COLOR)[..., :3], c[..., :3], FLOOR)
    ed = rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), d, FLOOR)
    print("bf16 update: colour max %.2e rms %.2e, depth max %.2e rms %.2e"
          % (ec.max(), np.sqrt((ec ** 2).mean()), ed.max(), np.sqrt((ed ** 2).mean())))
    assert ec.max() <= BF16_MAX and ed.max() <= BF16_MAX
    ctx.close()


def test_update_bf16_terrain_full_size_finite(gpu_lib):
    """The 32x16x32-probe, 256-ray terrain update at full size in the BF16
    form: four updates keep every atlas texel finite, and the atlas stays
    close to the FP32 form's (both trace the same hits; the BF16 form's
    shading samples the FP16 atlas)."""
    w = scenes.workload(1)
    atl = {}
    for prec in (abi.PRECISION_BF16, abi.PRECISION_FP32):
        g = w.grid.copy()
        g.precision = prec
        ctx = Context(g)
        ctx.set_pipeline(abi.PIPELINE_WAVEFRONT)
        ctx.build_scene(w.scene)
        ctx.set_light(w.light)
        for k in range(4):
            ctx.update(w.orientation(k))
        atl[prec] = (ctx.get_atlas(abi.ATLAS_COLOR), ctx.get_atlas(abi.ATLAS_DEPTH))
        ctx.close()
    bc, bd = atl[abi.PRECISION_BF16]
    fc, fd = atl[abi.PRECISION_FP32]
    assert np.isfinite(bc).all() and np.isfinite(bd).all()
    ec, ed = rel_err(bc[..., :3], fc[..., :3], FLOOR), rel_err(bd, fd, FLOOR)
    print("terrain bf16 vs fp32 after 4 updates: colour max %.2e rms %.2e, depth max %.2e rms %.2e"
          % (ec.max(), np.sqrt((ec ** 2).mean()), ed.max(), np.sqrt((ed ** 2).mean())))
    assert np.sqrt((ec ** 2).mean()) <= 1e-3 and np.sqrt((ed ** 2).mean()) <= 1e-3

"""Parity at the sizes the benchmark times (GPU tests).

* The FP32 wavefront form on the whole 32x16x32-probe, 256-ray terrain grid
  (~1M unique triangles, 4097 instances) for three successive updates, so the
  bounce lookup (sampleProbes into the previous, non-zero atlas) is checked
  on every probe: hit IDs, distance and facing bit-identical; atlas texels
  within 1e-4 relative (floor 1e-2); ray records as the test says; probe
  states exact.
* The BF16 precision form (BF16 tensor-core blend with FP32 accumulation,
  FP32 hysteresis accumulator, FP16 atlas) for ten updates against the FP64
  oracle, on the room workload (8x8x8 probes, 128 rays) and on the terrain
  workload: per-texel relative error at most 1e-3 (floor 1e-2), RMS at most
  5e-4, hit IDs bit-identical on every update.
"""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context

pytestmark = pytest.mark.gpu

TOL = 1e-4
FLOOR = 1e-2
BF16_MAX = 1e-3
BF16_RMS = 5e-4


def make_ctx(w, precision):
    g = w.grid.copy()
    g.precision = precision
    ctx = Context(g)
    ctx.set_pipeline(abi.PIPELINE_WAVEFRONT)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    ctx.record_hits(True)
    return ctx


def hit_mismatches(gh, oh):
    return int(((gh["instance"] != oh["instance"]) | (gh["primitive"] != oh["primitive"])).sum())


@pytest.fixture(scope="module")
def terrain():
    return scenes.workload(1)


@pytest.fixture(scope="module")
def terrain_oracle(terrain):
    o = Oracle(terrain.scene)
    yield o
    o.close()


def test_terrain_full_grid_fp32_three_updates(gpu_lib, terrain, terrain_oracle):
    """Ray records: within 1e-4 of the FP32 oracle on the first update (zero
    atlas, no bounce).  Later updates read the previous atlas through
    sampleProbes, whose Chebyshev visibility term cancels catastrophically
    for some hits: there the FP32 restatement itself lies up to 1e-2 from the
    FP64 one, so single records of the two FP32 implementations can differ
    by more than 1e-4 (4 of 12.6 M record channels on the second update).
    The bar for those updates: at most 1e-5 of the record channels beyond
    1e-4, and the GPU no farther from the FP64 oracle than the FP32 oracle
    is (1.25x its largest deviation).  Atlas texels: 1e-4 on every update."""
    w = terrain
    P = w.grid.probe_count()
    ctx = make_ctx(w, abi.PRECISION_FP32)
    c, d = zero_atlas(w.grid)
    c64, d64 = zero_atlas(w.grid, fp64=True)
    st = np.ones(P, np.uint32)
    st64 = np.ones(P, np.uint32)
    for k in range(3):
        ctx.update(w.orientation(k))
        rays, hits = terrain_oracle.update(w.grid, w.light, w.orientation(k), c, d, st, want_rays=True,
                                           want_hits=True)
        gh = ctx.get_hits(P)
        assert hit_mismatches(gh, hits) == 0, "update %d" % k
        hit = hits["instance"] != abi.MISS
        assert (gh["t"][hit].view(np.uint32) == hits["t"][hit].view(np.uint32)).all(), "update %d: t" % k
        assert (gh["backface"][hit] == hits["backface"][hit]).all()
        gr = ctx.get_ray_records(P)
        er = rel_err(gr, rays, FLOOR)
        if k == 0:
            assert er.max() <= TOL, "ray records, update 0: %g" % er.max()
        else:
            rays64, _ = terrain_oracle.update(w.grid, w.light, w.orientation(k), c64, d64, st64, fp64=True,
                                              want_rays=True)
            frac = float((er > TOL).mean())
            g64, c64err = rel_err(gr, rays64, FLOOR).max(), rel_err(rays, rays64, FLOOR).max()
            print("update %d records: %.2e beyond 1e-4 (max %.2e); vs fp64: gpu %.2e, fp32 oracle %.2e"
                  % (k, frac, er.max(), g64, c64err))
            assert frac <= 1e-5, "ray records, update %d: %.2e beyond 1e-4" % (k, frac)
            assert g64 <= 1.25 * c64err + 1e-6, "update %d: gpu %.2e from fp64, fp32 oracle %.2e" % (k, g64, c64err)
        if k == 0:  # the FP64 chain starts from the same first update
            terrain_oracle.update(w.grid, w.light, w.orientation(0), c64, d64, st64, fp64=True)
        ec = rel_err(ctx.get_atlas(abi.ATLAS_COLOR), c, FLOOR).max()
        ed = rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), d, FLOOR).max()
        print("terrain fp32 update %d: colour %.2e depth %.2e" % (k, ec, ed))
        assert ec <= TOL and ed <= TOL, "atlas, update %d" % k
        assert (ctx.get_probe_states() == st).all()
    ctx.close()


def bf16_ten_updates(w, oracle):
    P = w.grid.probe_count()
    ctx = make_ctx(w, abi.PRECISION_BF16)
    c, d = zero_atlas(w.grid, fp64=True)
    st = np.ones(P, np.uint32)
    for k in range(10):
        ctx.update(w.orientation(k))
        _, hits = oracle.update(w.grid, w.light, w.orientation(k), c, d, st, fp64=True, want_hits=True)
        assert hit_mismatches(ctx.get_hits(P), hits) == 0, "update %d" % k
    ec = rel_err(ctx.get_atlas(abi.ATLAS_COLOR)[..., :3], c[..., :3], FLOOR)
    ed = rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), d, FLOOR)
    ctx.close()
    r = {"color_max": ec.max(), "color_rms": np.sqrt((ec ** 2).mean()), "depth_max": ed.max(),
         "depth_rms": np.sqrt((ed ** 2).mean())}
    print("%s bf16 after 10 updates vs fp64: %s" % (w.name, {k: "%.2e" % v for k, v in r.items()}))
    return r


def check_bf16(r):
    assert r["color_max"] <= BF16_MAX and r["depth_max"] <= BF16_MAX, r
    assert r["color_rms"] <= BF16_RMS and r["depth_rms"] <= BF16_RMS, r


def test_bf16_room_ten_updates_vs_fp64(gpu_lib):
    w = scenes.workload(0)
    o = Oracle(w.scene)
    check_bf16(bf16_ten_updates(w, o))
    o.close()


def test_bf16_terrain_ten_updates_vs_fp64(gpu_lib, terrain, terrain_oracle):
    check_bf16(bf16_ten_updates(terrain, terrain_oracle))


def test_terrain_wide_nodes_same_hits_and_atlas(gpu_lib, terrain):
    """The eight-wide quantised trees (node_width 8) on the whole terrain grid:
    hits, ray records and atlases bit-identical to the binary trees' over two
    updates (primary rays, shadow rays and the bounce lookup)."""
    w = terrain
    P = w.grid.probe_count()
    out = []
    for width in (2, 8):
        ctx = make_ctx(w, abi.PRECISION_FP32)
        ctx.set_trace_tuning(node_width=width)
        for k in range(2):
            ctx.update(w.orientation(k))
        out.append((ctx.get_hits(P), ctx.get_ray_records(P), ctx.get_atlas(abi.ATLAS_COLOR),
                    ctx.get_atlas(abi.ATLAS_DEPTH)))
        ctx.close()
    (h2, r2, c2, d2), (h8, r8, c8, d8) = out
    assert hit_mismatches(h2, h8) == 0
    assert (r2.view(np.uint32) == r8.view(np.uint32)).all()
    assert (c2.view(np.uint32) == c8.view(np.uint32)).all() and (d2.view(np.uint32) == d8.view(np.uint32)).all()

"""The reference-format atlas form (DDGI_PRECISION_REFERENCE_FORMAT): the FP32
blend with every stored texel rounded to the reference's image formats,
B10G11R11 unsigned floats for irradiance and RG16F for depth
(src/IrradianceProbes.cpp:41, 63), so the next update's bounce lookup reads
rounded values as the reference's does (GPU tests).

Bars, against the oracle run in the same form: hit IDs bit-identical; every
stored texel representable in its format; every texel within two steps of
its format of the oracle's (rounding maps values a few float ulps apart,
near a rounding boundary, to neighbouring format values: one step, and that
difference feeds the next update's bounce); at most 0.1 % of texels differ
by more than 1e-4 relative (floor 1e-2)."""
import numpy as np
import pytest

from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context

pytestmark = pytest.mark.gpu

MBITS_COLOR = (6, 6, 5)  # R, G: 11-bit; B: 10-bit unsigned floats
MBITS_DEPTH = (10, 10)   # halves


def format_step(v, mbits):
    """Spacing of a 5-bit-exponent float format with `mbits` mantissa bits
    at |v| (the subnormal spacing below 2^-14)."""
    a = np.maximum(np.abs(v.astype(np.float64)), 2.0 ** -14)
    return 2.0 ** (np.floor(np.log2(a)) - mbits)


def check_channels(gpu, cpu, mbits, what):
    for c, mb in enumerate(mbits):
        kind = 2 if mb == 10 else (0 if mb == 6 else 1)
        g, o = gpu[..., c], cpu[..., c]
        assert (Oracle.round_store(kind, g).view(np.uint32) == g.view(np.uint32)).all(), "%s %d not rounded" % (what, c)
        steps = np.abs(g.astype(np.float64) - o) / format_step(o, mb)
        assert steps.max() <= 2.0 + 1e-9, "%s channel %d: %.2f format steps" % (what, c, steps.max())
    rel = np.abs(gpu[..., :len(mbits)].astype(np.float64) - cpu[..., :len(mbits)]) / np.maximum(
        np.abs(cpu[..., :len(mbits)]), 1e-2)
    frac = float((rel > 1e-4).mean())
    print("%s: %.3e of channels beyond 1e-4, max %.2e" % (what, frac, rel.max()))
    assert frac <= 1e-3, "%s: %.3e of channels beyond 1e-4" % (what, frac)


@pytest.mark.parametrize("pipeline", [abi.PIPELINE_WAVEFRONT, abi.PIPELINE_FUSED])
def test_reference_format_room_three_updates(gpu_lib, pipeline):
    w = scenes.room_workload(1234, precision=abi.PRECISION_REFERENCE_FORMAT)
    P = w.grid.probe_count()
    ctx = Context(w.grid)
    ctx.set_pipeline(pipeline)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    ctx.record_hits(True)
    o = Oracle(w.scene)
    c, d = zero_atlas(w.grid)
    st = np.ones(P, np.uint32)
    for k in range(3):
        ctx.update(w.orientation(k))
        _, hits = o.update(w.grid, w.light, w.orientation(k), c, d, st, want_hits=True)
        gh = ctx.get_hits(P)
        assert (gh["instance"] == hits["instance"]).all() and (gh["primitive"] == hits["primitive"]).all()
        check_channels(ctx.get_atlas(abi.ATLAS_COLOR), c, MBITS_COLOR, "update %d colour" % k)
        check_channels(ctx.get_atlas(abi.ATLAS_DEPTH), d, MBITS_DEPTH, "update %d depth" % k)
    assert (ctx.get_atlas(abi.ATLAS_COLOR)[..., 3][ctx.get_atlas(abi.ATLAS_COLOR)[..., 3] != 0] == 1.0).all()
    ctx.close()
    o.close()


def test_reference_format_differs_from_fp32_by_rounding(gpu_lib):
    """One update from a zero atlas: the reference-format atlas is the FP32
    form's atlas rounded texel by texel (no earlier rounding feeds it)."""
    w = scenes.room_workload(77, n_boxes=80, resolution=(6, 5, 6), rays=128)
    atl = {}
    for prec in (abi.PRECISION_FP32, abi.PRECISION_REFERENCE_FORMAT):
        g = w.grid.copy()
        g.precision = prec
        ctx = Context(g)
        ctx.build_scene(w.scene)
        ctx.set_light(w.light)
        ctx.update(w.orientation(0))
        atl[prec] = (ctx.get_atlas(abi.ATLAS_COLOR), ctx.get_atlas(abi.ATLAS_DEPTH))
        ctx.close()
    fc, fd = atl[abi.PRECISION_FP32]
    rc, rd = atl[abi.PRECISION_REFERENCE_FORMAT]
    for ch, kind in ((0, 0), (1, 0), (2, 1)):
        assert (Oracle.round_store(kind, fc[..., ch]).view(np.uint32) == rc[..., ch].view(np.uint32)).all()
    for ch in (0, 1):
        assert (Oracle.round_store(2, fd[..., ch]).view(np.uint32) == rd[..., ch].view(np.uint32)).all()

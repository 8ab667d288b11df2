"""The atmospheric-sky miss mode (ddgi_set_sky_mode(DDGI_SKY_ATMOSPHERE):
src/shaders/sky.glsl:60-127 called from miss.rmiss:22) against the oracle's
restatement of the same shader (GPU tests): on an open terrain scene where
many probe rays miss, hit IDs bit-identical and ray records and atlas texels
within 1e-4 relative (floor 1e-2) over two updates (the second reads the
first's atlas through the bounce lookup); the final gather's sky pixels in
the same mode; the calls that do not take the mode refuse it."""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Batch, Context, DDGIError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def open_terrain():
    w = scenes.terrain_workload(91, resolution=(6, 3, 6), rays=64, updates=2, n_instances=48, boxes_per_cluster=150,
                                cells=48)
    w.light.color[3] = 10.0  # LightBuffer's default colour.a: the sun brightness of the sky
    return w


@pytest.fixture
def atmosphere():
    Oracle.set_sky_mode(1)
    yield
    Oracle.set_sky_mode(0)


@pytest.mark.parametrize("pipeline", [abi.PIPELINE_WAVEFRONT, abi.PIPELINE_FUSED])
def test_sky_update_matches_oracle(gpu_lib, open_terrain, atmosphere, pipeline):
    w = open_terrain
    P = w.grid.probe_count()
    ctx = Context(w.grid)
    ctx.set_pipeline(pipeline)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    ctx.set_sky_mode(abi.SKY_ATMOSPHERE)
    ctx.record_hits(True)
    o = Oracle(w.scene)
    c, d = zero_atlas(w.grid)
    st = np.ones(P, np.uint32)
    for k in range(2):
        ctx.update(w.orientation(k))
        rays, hits = o.update(w.grid, w.light, w.orientation(k), c, d, st, want_rays=True, want_hits=True)
        gh = ctx.get_hits(P)
        assert (gh["instance"] == hits["instance"]).all() and (gh["primitive"] == hits["primitive"]).all()
        gr = ctx.get_ray_records(P)
        miss = rays[..., 3] == -1.0
        assert miss.mean() > 0.2  # an open scene: many rays see the sky
        assert not np.allclose(rays[miss][:, :3], np.asarray(w.light.sky[:3], np.float32))  # not the constant
        assert rel_err(gr, rays, 1e-2).max() <= 1e-4, "update %d records" % k
    assert rel_err(ctx.get_atlas(abi.ATLAS_COLOR), c, 1e-2).max() <= 1e-4
    assert rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), d, 1e-2).max() <= 1e-4
    ctx.close()
    o.close()


def test_sky_final_gather_matches_oracle(gpu_lib, open_terrain, atmosphere):
    import torch

    w = open_terrain
    ctx = Context(w.grid)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    ctx.set_sky_mode(abi.SKY_ATMOSPHERE)
    ctx.update(w.orientation(0))
    color, depth, states = ctx.get_atlas(abi.ATLAS_COLOR), ctx.get_atlas(abi.ATLAS_DEPTH), ctx.get_probe_states()
    rng = np.random.default_rng(9)
    H, W = 32, 48
    n = H * W
    dirs = rng.normal(size=(n, 3))
    gb = {"position_depth": np.column_stack([dirs, np.zeros(n)]).astype(np.float32),  # all sky pixels
          "normal_metalness": np.zeros((n, 4), np.float32), "albedo_roughness": np.zeros((n, 4), np.float32),
          "emissive": np.zeros((n, 4), np.float32), "direct_light": np.zeros(n, np.float32)}
    origin = np.array([3.0, 12.0, -4.0], np.float32)
    dev = {k: torch.from_numpy(v.reshape(H, W) if v.ndim == 1 else v.reshape(H, W, 4)).cuda().contiguous()
           for k, v in gb.items()}
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    ctx.final_gather(dev, origin, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(-1, 4)
    want = Oracle.final_gather(w.grid, w.light, states, color, depth, gb, origin)
    assert rel_err(got[:, :3], want[:, :3], 1e-2).max() <= 1e-4
    assert got[:, :3].std() > 0  # direction-dependent
    ctx.close()


def test_sky_mode_refused_where_unsupported(gpu_lib, open_terrain):
    w = open_terrain
    ctx = Context(w.grid)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    with pytest.raises(DDGIError):
        ctx.set_sky_mode(7)
    ctx.set_sky_mode(abi.SKY_ATMOSPHERE)
    with pytest.raises(DDGIError) as e:
        ctx.forward_record(np.stack([w.orientation(0)]), 1)
    assert e.value.status == 7
    with pytest.raises(DDGIError) as e:
        b = Batch([ctx])
        b.update(np.stack([w.orientation(0)]))
    assert e.value.status == 7
    ctx.close()

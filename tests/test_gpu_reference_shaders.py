"""The CUDA path against the reference's own shaders (GPU tests).

tests/golden/reference_shaders.npz holds what the reference's src/shaders
files produced, compiled as C++ and run on the host (oracle/build_ref_glsl.py,
tests/golden/make_reference_vectors.py): a probe trace + update of a closed
room from a previous atlas of random texels and states, and of the editor
scene file from a cleared atlas; and the update passes alone on given ray
records.  The C ABI runs the same updates in the reference-format form
(DDGI_PRECISION_REFERENCE_FORMAT, atmospheric sky) from the same previous
atlas, probe states, orientation and probe list.  Bars:

* ray directions within one float step (2.4e-7) of the reference's
  rayDirection image;
* ray records: hit distance bit for bit, radiance within 1e-5 relative
  (floor 1e-3; the reference build and the CUDA path round pow and the
  transcendental functions differently);
* atlases: every texel within two steps of its format (values a few float
  ulps apart near a rounding boundary land on neighbouring format values),
  at most 1 % of texels not bit-identical; probe states equal;
* the passes alone (ddgi_blend_records on the fixture's records): the same
  atlas bars, states equal; at 192 rays depth only (the reference's
  irradiance pass loads 36 directions, probesUpdate.glsl:63-68);
* probe classification (ddgi_init_probes against probesInit.rgen): every
  state equal;
* probe selection (ddgi_update_scheduled against the reference's
  selectProbesToUpdate): the 16-call sequence's lists, each call's states
  set before it;
* final gather (ddgi_final_gather against FinalGather.frag, on the room's
  updated atlas): surface pixels within 1e-5 relative, sky pixels within
  1e-4 (the view direction is the camera ray computed in double)."""
import os

import numpy as np
import pytest

from test_reference_shaders import atlas_from, format_steps, gather_inputs, grid_from, light_from, rel, room_scene
from vulkanexp_gb300 import abi, ingest
from vulkanexp_gb300.ddgi import Context

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def vec():
    return np.load(os.path.join(GOLDEN, "reference_shaders.npz"))


def check_atlases(ctx, rc, rd, what):
    c = ctx.get_atlas(abi.ATLAS_COLOR)
    d = ctx.get_atlas(abi.ATLAS_DEPTH)
    for ch, mb in enumerate((6, 6, 5)):
        s = format_steps(c[..., ch], rc[..., ch], mb).max()
        assert s <= 2.0 + 1e-9, "%s colour %d: %.2f format steps" % (what, ch, s)
    for ch in range(2):
        s = format_steps(d[..., ch], rd[..., ch], 10).max()
        assert s <= 2.0 + 1e-9, "%s depth %d: %.2f format steps" % (what, ch, s)
    fc = (c[..., :3] != rc).any(axis=-1).mean()
    fd = (d != rd).any(axis=-1).mean()
    print("%s: colour texels not bit-identical %.4f, depth %.4f" % (what, fc, fd))
    assert fc <= 0.01 and fd <= 0.01
    return c, d


def prepared(g, L, sc, c, d, st):
    ctx = Context(g)
    ctx.set_sky_mode(abi.SKY_ATMOSPHERE)
    if sc is not None:
        ctx.build_scene(sc)
    if L is not None:
        ctx.set_light(L)
    ctx.set_atlas(abi.ATLAS_COLOR, c)
    ctx.set_atlas(abi.ATLAS_DEPTH, d)
    ctx.set_probe_states(st)
    return ctx


@pytest.mark.parametrize("name", ["room", "editor"])
def test_update_against_reference_shaders(gpu_lib, vec, name):
    k = "trace_%s_" % name
    sc = room_scene(vec) if name == "room" else ingest.load(os.path.join(GOLDEN, "editor_room.scene"))
    g, L = grid_from(vec[k + "grid"]), light_from(vec[k + "light"])
    assert g.precision == abi.PRECISION_REFERENCE_FORMAT
    c, d = atlas_from(vec, k, g)
    lst = vec[k + "list"]
    ctx = prepared(g, L, sc, c, d, vec[k + "states_in"])
    ctx.update(vec[k + "orientation"], probe_list=lst)
    ctx.synchronize(timeout_ms=60000)
    dirs = ctx.get_ray_directions()
    assert np.abs(dirs[:, :3] - vec[k + "dirs"][:, :3]).max() <= 2.4e-7
    rays = ctx.get_ray_records(len(lst))
    ref = vec[k + "rays"]
    assert (rays[..., 3].view(np.uint32) == ref[..., 3].view(np.uint32)).all(), \
        "%d hit distances differ" % (rays[..., 3] != ref[..., 3]).sum()
    r = rel(rays[..., :3], ref[..., :3], 1e-3).max()
    print("%s: radiance max rel %.2e" % (name, r))
    assert r <= 1e-5
    check_atlases(ctx, vec[k + "color_out"].astype(np.float32), vec[k + "depth_out"].astype(np.float32), name)
    assert (ctx.get_probe_states() == vec[k + "states_out"]).all()
    ctx.close()


@pytest.mark.parametrize("R", [32, 192])
def test_passes_against_reference_shaders(gpu_lib, vec, R):
    k = "upd%d_" % R
    g = grid_from(vec[k + "grid"])
    c, d = atlas_from(vec, k, g)
    ctx = prepared(g, None, None, c, d, vec[k + "states_in"])
    ctx.blend_records(vec[k + "orientation"], vec[k + "rays"], probe_list=vec[k + "list"])
    ctx.synchronize(timeout_ms=60000)
    rc = vec[k + "color_out"].astype(np.float32)
    rd = vec[k + "depth_out"].astype(np.float32)
    if R <= 36:
        check_atlases(ctx, rc, rd, "passes R=%d" % R)
        assert (ctx.get_probe_states() == vec[k + "states_out"]).all()
    else:
        dd = ctx.get_atlas(abi.ATLAS_DEPTH)
        for ch in range(2):
            assert format_steps(dd[..., ch], rd[..., ch], 10).max() <= 2.0 + 1e-9
        assert (dd != rd).any(axis=-1).mean() <= 0.01
    ctx.close()


@pytest.mark.parametrize("name", ["room", "editor"])
def test_probe_classification_against_reference_shaders(gpu_lib, vec, name):
    sc = room_scene(vec) if name == "room" else ingest.load(os.path.join(GOLDEN, "editor_room.scene"))
    g = grid_from(vec["init_%s_grid" % name])
    ctx = Context(g)
    ctx.build_scene(sc)
    ctx.init_probes(vec["init_%s_orientation" % name])
    st = ctx.get_probe_states()
    ref = vec["init_%s_states" % name]
    assert (st == ref).all(), "%d of %d probe states differ" % ((st != ref).sum(), len(st))
    ctx.close()


def test_final_gather_against_reference_shaders(gpu_lib, vec):
    import torch

    g, L, c, d, st, gb, cam, sky = gather_inputs(vec)
    H, W = vec["gather_out"].shape[:2]
    ctx = Context(g)
    ctx.set_sky_mode(abi.SKY_ATMOSPHERE)
    ctx.set_light(L)
    ctx.set_atlas(abi.ATLAS_COLOR, c)
    ctx.set_atlas(abi.ATLAS_DEPTH, d)
    ctx.set_probe_states(st)
    dev = {k: torch.from_numpy(v.reshape(H, W) if v.ndim == 1 else v.reshape(H, W, 4)).cuda().contiguous()
           for k, v in gb.items()}
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    ctx.final_gather(dev, cam, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(-1, 4)
    ref = vec["gather_out"].reshape(-1, 4)
    r = rel(got[:, :3], ref[:, :3], 1e-3)
    print("final gather: surface max rel %.2e, sky max rel %.2e" % (r[~sky].max(), r[sky].max()))
    assert r[~sky].max() <= 1e-5 and r[sky].max() <= 1e-4
    ctx.close()


def test_probe_selection_against_reference(gpu_lib, vec):
    from vulkanexp_gb300 import scenes
    sc = ingest.load(os.path.join(GOLDEN, "editor_room.scene"))
    g = scenes.fit_grid(sc, (6, 3, 6), 32)
    assert g.probe_count() == vec["sel_states"].shape[1]
    ctx = Context(g)
    ctx.build_scene(sc)
    ctx.set_light(scenes.default_light())
    for k in range(len(vec["sel_caps"])):
        ctx.set_probe_states(vec["sel_states"][k])
        ctx.update_scheduled(scenes.random_orientation(9, k), int(vec["sel_caps"][k]))
        s = ctx.schedule()
        assert np.array_equal(s["list"], vec["sel_lists"][k, :vec["sel_counts"][k]]), k
        assert s["offset"] == vec["sel_offsets"][k], k
    ctx.close()

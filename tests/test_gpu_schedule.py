"""Probe classification (ddgi_init_probes) and the on-device adaptive
schedule (ddgi_update_scheduled) on the GPU.

Bars: probe states after classification equal the oracle's exactly; every
scheduled update selects exactly the probes (and in the same visit order)
that the restated selectProbesToUpdate host loop selects from the GPU's own
probe states, with the same offset/loop bookkeeping; atlases after
scheduled FP32 updates agree with the oracle updating the same probe lists
within 1e-4 relative; the BF16 form of a scheduled update equals an
explicit-list update of the same probes bit for bit."""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, select_probes, zero_atlas
from test_schedule import box_grid, box_scene
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context, IrradianceProbes

pytestmark = pytest.mark.gpu


def make_ctx(scene, grid, light=None):
    ctx = Context(grid)
    ctx.build_scene(scene)
    ctx.set_light(light or scenes.default_light())
    return ctx


def small_terrain():
    w = scenes.terrain_workload(1235, resolution=(8, 4, 8), rays=256, n_instances=256, boxes_per_cluster=500,
                                cells=128)
    return w


@pytest.mark.parametrize("case", ["box", "room", "room_r64", "terrain"])
def test_init_states_match_oracle(gpu_lib, case):
    if case == "box":
        sc, g = box_scene(), box_grid()
    elif case == "terrain":
        w = small_terrain()
        sc, g = w.scene, w.grid
    else:
        w = scenes.workload(0)
        sc, g = w.scene, w.grid.copy()
        if case == "room_r64":
            g.rays_per_probe = 64  # 448 of the 512 init directions degenerate
    orient = scenes.random_orientation(99, 0)
    ctx = make_ctx(sc, g)
    ctx.init_probes(orient)
    got = ctx.get_probe_states()
    want = Oracle(sc).init_probes(g, orient)
    assert (got == want).all(), "%d of %d probe states differ" % ((got != want).sum(), got.size)
    assert {0, 1, 8} >= set(np.unique(got).tolist())
    ctx.close()


@pytest.mark.parametrize("cap", [0, 37])
def test_schedule_matches_host_loop_and_oracle(gpu_lib, room_workload, room_oracle, cap):
    w = room_workload
    ctx = make_ctx(w.scene, w.grid, w.light)
    ctx.init_probes(w.orientation(50))
    st = ctx.get_probe_states()
    assert (st == room_oracle.init_probes(w.grid, w.orientation(50))).all()
    c, d = zero_atlas(w.grid)
    ost = st.copy()
    off, loop = 0, 0
    for k in range(5):
        want, off, loop = select_probes(ctx.get_probe_states(), off, loop, cap)
        ctx.update_scheduled(w.orientation(k), cap)
        s = ctx.schedule()
        assert s["count"] == len(want) and (s["list"] == want).all(), "update %d: selection differs" % k
        assert (s["offset"], s["loop"]) == (off, loop)
        if len(want):
            room_oracle.update(w.grid, w.light, w.orientation(k), c, d, ost, probe_list=want)
        gc, gd = ctx.get_atlas(abi.ATLAS_COLOR), ctx.get_atlas(abi.ATLAS_DEPTH)
        assert rel_err(gc, c, 1e-2).max() <= 1e-4, "update %d colour" % k
        assert rel_err(gd, d, 1e-2).max() <= 1e-4, "update %d depth" % k
        assert (ctx.get_probe_states() == ost).all(), "update %d states" % k
    ctx.close()


def test_scheduled_bf16_equals_explicit_list(gpu_lib, room_workload):
    w = room_workload
    g = w.grid.copy()
    g.precision = abi.PRECISION_BF16
    a, b = make_ctx(w.scene, g, w.light), make_ctx(w.scene, g, w.light)
    for ctx in (a, b):
        ctx.init_probes(w.orientation(7))
    for k in range(3):
        a.update_scheduled(w.orientation(k), 100)
        lst = a.schedule()["list"]
        b.update(w.orientation(k), lst)
        for kind in (abi.ATLAS_COLOR, abi.ATLAS_DEPTH):
            x, y = a.get_atlas(kind), b.get_atlas(kind)
            assert (x.view(np.uint32) == y.view(np.uint32)).all(), "update %d atlas %d" % (k, kind)
        assert (a.get_probe_states() == b.get_probe_states()).all()
    a.close()
    b.close()


def test_off_probes_are_never_updated(gpu_lib):
    sc, g = box_scene(), box_grid()
    ctx = make_ctx(sc, g)
    ctx.init_probes(scenes.random_orientation(3, 0))
    st = ctx.get_probe_states()
    off = np.flatnonzero(st == 0)
    assert off.size > 0
    for k in range(3):
        ctx.update_scheduled(scenes.random_orientation(3, 1 + k))
        assert not np.isin(ctx.schedule()["list"], off).any()
    assert (ctx.get_probe_states()[off] == 0).all()
    ctx.close()


def test_set_schedule_and_mirror_ramp(gpu_lib, room_workload):
    w = room_workload
    ctx = make_ctx(w.scene, w.grid, w.light)
    ctx.set_schedule(17, 3)
    s = ctx.schedule(with_list=False)
    assert (s["offset"], s["loop"]) == (17, 3)
    ctx.close()

    p = IrradianceProbes()
    p.GridParameters = w.grid.copy()
    p.TargetHysteresis = 0.98
    p.init(w.grid.extent_min, w.grid.extent_max)
    p.setScene(w.scene)
    p.setLightBuffer(w.light)
    p.initProbes(w.orientation(0))
    assert p.GridParameters.hysteresis == 0.0 and p.hysteresis()[1] == 0.0
    hs = []
    for k in range(40):
        p.update(w.orientation(1 + k))
        hs.append(p.hysteresis()[1])
    # ramps up towards the target (one step per probe count of refreshed probes)
    assert hs == sorted(hs) and 0.2 < hs[-1] <= np.float32(0.98)
    p.destroy()

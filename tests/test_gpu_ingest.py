"""A scene file laid out as the editor saves one (tests/golden/
editor_room.scene, Scene::save's layout, src/Scene.cpp:710-817) traced and
shaded on the GPU: loaded by the package's ingest, two probe updates through
the C ABI against the oracle on the same arrays: hit IDs, distance and
facing bit-identical, atlas texels within 1e-4 relative (floor 1e-2)."""
import os

import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, ingest, scenes
from vulkanexp_gb300.ddgi import Context

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "editor_room.scene")


@pytest.mark.parametrize("build_mode", ["fast_trace", "fast_build"])
def test_editor_scene_traced_like_the_oracle(gpu_lib, build_mode):
    sc = ingest.load(FIXTURE)
    g = scenes.fit_grid(sc, (6, 3, 6), 96)
    L = scenes.default_light()
    P = g.probe_count()
    ctx = Context(g)
    ctx.set_build_mode(build_mode)  # SAH trees with spatial splits, linear BVHs
    ctx.build_scene(sc)
    ctx.set_light(L)
    ctx.record_hits(True)
    o = Oracle(sc)
    c, d = zero_atlas(g)
    st = np.ones(P, np.uint32)
    for k in range(2):
        orient = scenes.random_orientation(77, k)
        ctx.update(orient)
        _, hits = o.update(g, L, orient, c, d, st, want_hits=True)
        gh = ctx.get_hits(P)
        assert (gh["instance"] == hits["instance"]).all() and (gh["primitive"] == hits["primitive"]).all()
        hit = hits["instance"] != abi.MISS
        assert hit.mean() > 0.1  # the room is open above: 18 % of the rays hit (the oracle's count)
        assert (gh["t"][hit].view(np.uint32) == hits["t"][hit].view(np.uint32)).all()
    assert rel_err(ctx.get_atlas(abi.ATLAS_COLOR), c, 1e-2).max() <= 1e-4
    assert rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), d, 1e-2).max() <= 1e-4
    ctx.close()
    o.close()

"""Final gather (ddgi_final_gather) against the oracle's restatement of
src/shaders/FinalGather.frag, on a seeded random G-buffer over the room
after two probe updates.  Bar: 1e-4 relative (floor 1e-2), as the update's
parity; sky pixels exact."""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context

pytestmark = pytest.mark.gpu


def random_gbuffer(rng, h, w, lo, hi, with_reflection=True):
    n = h * w
    pos = rng.uniform(lo, hi, size=(n, 3))
    depth = np.where(rng.uniform(size=n) < 0.1, 0.0, rng.uniform(0.5, 20.0, size=n))
    nrm = rng.normal(size=(n, 3))
    g = {
        "position_depth": np.column_stack([pos, depth]),
        "normal_metalness": np.column_stack([nrm, rng.uniform(0, 1, n)]),
        "albedo_roughness": np.column_stack([rng.uniform(0, 1, (n, 3)), rng.uniform(0.05, 1, n)]),
        "emissive": np.column_stack([rng.uniform(0, 0.2, (n, 3)), np.zeros(n)]),
        "direct_light": rng.uniform(0, 1, n),
        "reflection": np.column_stack([rng.uniform(0, 2, (n, 3)), np.ones(n)]) if with_reflection else None,
    }
    return {k: None if v is None else v.astype(np.float32) for k, v in g.items()}


@pytest.mark.parametrize("precision", [abi.PRECISION_FP32, abi.PRECISION_BF16])
@pytest.mark.parametrize("with_reflection", [True, False])
def test_final_gather_matches_oracle(gpu_lib, room_workload, precision, with_reflection):
    import torch

    w = room_workload
    g = w.grid.copy()
    g.precision = precision
    ctx = Context(g)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    for k in range(2):
        ctx.update(w.orientation(k))
    color, depth = ctx.get_atlas(abi.ATLAS_COLOR), ctx.get_atlas(abi.ATLAS_DEPTH)
    states = ctx.get_probe_states()
    H, W = 96, 160
    rng = np.random.default_rng(5)
    gb = random_gbuffer(rng, H, W, (-0.5, -0.5, -0.5), (10.5, 6.5, 10.5), with_reflection)
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
    err = rel_err(got[:, :3], want[:, :3], 1e-2)
    assert err.max() <= 1e-4, "max rel err %.3g" % err.max()
    assert (got[:, 3] == 1.0).all()
    ctx.close()


def test_final_gather_rejects_bad_input(gpu_lib, room_workload):
    import torch

    from vulkanexp_gb300.ddgi import DDGIError

    ctx = Context(room_workload.grid)
    z4 = torch.zeros((4, 4, 4), device="cuda")
    z1 = torch.zeros((4, 4), device="cuda")
    gb = {"position_depth": z4, "normal_metalness": z4, "albedo_roughness": z4, "emissive": z4, "direct_light": z1}
    with pytest.raises(DDGIError):
        ctx.final_gather(gb, [np.inf, 0, 0], z4)
    ctx.close()

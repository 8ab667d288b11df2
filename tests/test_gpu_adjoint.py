"""Gradients of an atlas loss through K recurrent updates (GPU adjoint)
against central finite differences of the FP64 oracle.

Workload (the differentiation configuration): the room generator with 1000
boxes (12,012 triangles), 16x8x16 probes, 256 rays, K = 8 updates from a zero
atlas, checkpoints every 2 updates.  Loss: sum of squared differences between
the colour atlas after K updates and a target atlas made with the same seed
and re-drawn albedos.  Parameters: 64 material albedos (RGB), sun radiance,
sky radiance; 32 of them chosen at random are checked with h = 1e-4 on the
FP64 oracle replaying the recorded hit set.

Bar: |grad - fd| <= 1e-3 * max(|fd|, 1e-3 * max|fd|) for every checked
parameter (the GPU runs the FP32 form; FP64 finite differences)."""
import numpy as np
import pytest

from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import scenes

pytestmark = pytest.mark.gpu

H = 1e-4


def fp64_loss_fn(oracle, w, orients, recording, target):
    def loss(albedo, sun, sky):
        c, d = zero_atlas(w.grid, fp64=True)
        st = np.ones(w.grid.probe_count(), np.uint32)
        oracle.replay(w.grid, w.light, orients, st, c, d, recording, albedo, sun, sky)
        return float(((c[..., :3] - target[..., :3]) ** 2).sum())
    return loss


def run_check(w, K, n_check, seed):
    import torch

    from ddgi_autograd import AtlasFunction, Runner

    orients = np.stack([w.orientation(k) for k in range(K)])
    o = Oracle(w.scene)
    c, d = zero_atlas(w.grid, fp64=True)
    st = np.ones(w.grid.probe_count(), np.uint32)
    recording = o.record(w.grid, w.light, orients, st, c, d)
    albedo = w.scene.materials["base_color"].astype(np.float64)
    sun = np.array(w.light.color[:3], np.float64)
    sky = np.array(w.light.sky[:3], np.float64)
    rng = np.random.default_rng(seed)
    # re-drawn albedos: a second stream of the workload seed (drawing from the
    # seed itself would repeat the scene's own albedos)
    target_albedo = np.random.default_rng([w.seed, 2]).uniform(0.2, 0.8, size=albedo.shape)
    tc, td = zero_atlas(w.grid, fp64=True)
    o.replay(w.grid, w.light, orients, np.ones(w.grid.probe_count(), np.uint32), tc, td, recording, target_albedo)

    runner = Runner(w, orients, checkpoint_every=2)
    ta = torch.tensor(albedo, requires_grad=True)
    ts = torch.tensor(sun, requires_grad=True)
    tk = torch.tensor(sky, requires_grad=True)
    atlas = AtlasFunction.apply(ta, ts, tk, runner)
    target = torch.from_numpy(tc.astype(np.float32))
    loss = ((atlas[..., :3] - target[..., :3]) ** 2).sum()
    loss.backward()
    runner.close()
    grads = np.concatenate([ta.grad.numpy().reshape(-1), ts.grad.numpy(), tk.grad.numpy()])

    f = fp64_loss_fn(o, w, orients, recording, tc)
    n_params = grads.size
    pick = rng.choice(n_params, size=n_check, replace=False)
    fd = np.zeros(n_check)
    for j, p in enumerate(pick):
        vals = []
        for s in (1.0, -1.0):
            a, su, sk = albedo.copy(), sun.copy(), sky.copy()
            if p < albedo.size:
                a.reshape(-1)[p] += s * H
            elif p < albedo.size + 3:
                su[p - albedo.size] += s * H
            else:
                sk[p - albedo.size - 3] += s * H
            vals.append(f(a, su, sk))
        fd[j] = (vals[0] - vals[1]) / (2 * H)
    got = grads[pick]
    scale = np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
    err = np.abs(got - fd) / scale
    print("adjoint vs FD: %d params, max rel err %.2e, median %.2e" % (n_check, err.max(), np.median(err)))
    return err


def test_adjoint_small_matches_fd(gpu_lib):
    w = scenes.room_workload(41, n_boxes=150, resolution=(6, 4, 6), rays=64, updates=3)
    err = run_check(w, K=3, n_check=24, seed=3)
    assert err.max() <= 1e-3


def test_adjoint_differentiation_workload_matches_fd(gpu_lib):
    w = scenes.workload(3)
    err = run_check(w, K=8, n_check=32, seed=1237)
    assert err.max() <= 1e-3


def test_forward_record_refuses_what_the_adjoint_does_not_model(gpu_lib):
    """The reverse pass differentiates the FP32 blend with the grid's fixed
    hysteresis and a constant sky: recording is refused
    (DDGI_ERR_UNSUPPORTED) while a hysteresis ramp is on, for the
    atmospheric sky and for a BF16 context, and works again once the ramp is
    off."""
    from vulkanexp_gb300 import abi
    from vulkanexp_gb300.ddgi import Context, DDGIError

    w = scenes.room_workload(43, n_boxes=40, resolution=(3, 3, 3), rays=32)
    orients = np.stack([w.orientation(k) for k in range(2)])
    ctx = Context(w.grid)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    ctx.set_target_hysteresis(0.9)
    with pytest.raises(DDGIError) as e:
        ctx.forward_record(orients, 1)
    assert e.value.status == 7
    ctx.set_target_hysteresis(-1.0)
    ctx.forward_record(orients, 1)
    ctx.set_sky_mode(abi.SKY_ATMOSPHERE)
    with pytest.raises(DDGIError) as e:
        ctx.forward_record(orients, 1)
    assert e.value.status == 7
    ctx.close()
    g = w.grid.copy()
    g.precision = abi.PRECISION_BF16
    ctx = Context(g)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    with pytest.raises(DDGIError) as e:
        ctx.forward_record(orients, 1)
    assert e.value.status == 7
    ctx.close()

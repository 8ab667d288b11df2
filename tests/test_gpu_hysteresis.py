"""The hysteresis ramp of IrradianceProbes::update in the C ABI (GPU tests).

src/IrradianceProbes.cpp:462-476, restated below as the reference's host
loop (`reference_ramp`), is the oracle: after every update the library's
blended value, host-side value and probe counter must equal the restatement's
bit for bit (float32 arithmetic, one rounding per operation, the 0.05
comparison in double), for full updates, explicit probe lists and device-side
scheduled selections (whose counts are read back only by the test).  The FP32
atlas after a ramped sequence must equal the CPU oracle run with the
restatement's blended value per update (1e-4, floor 1e-2)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle.oracle import Oracle, zero_atlas
from vulkanexp_gb300 import abi, scenes
from vulkanexp_gb300.ddgi import Context

pytestmark = pytest.mark.gpu


class ReferenceRamp:
    """GridParameters.hysteresis, the uploaded uniform and the static
    updatedProbes counter of the reference, stepped like its update()."""

    def __init__(self, hysteresis, target):
        self.param = np.float32(hysteresis)
        self.uniform = np.float32(hysteresis)
        self.target = np.float32(target)
        self.counted = 0

    def update(self, probe_count, P):
        if self.counted >= P:
            if abs(float(self.param - self.target)) > 0.05:
                self.uniform = self.param  # updateUniforms() before the increment
                self.param = np.float32(self.param + np.float32(np.float32(0.1) * (self.target - self.param)))
            elif self.param != self.target:
                self.param = self.target
                self.uniform = self.param
            self.counted -= P
        self.counted += probe_count
        return self.uniform


def small_room(precision=abi.PRECISION_FP32, hysteresis=0.0):
    w = scenes.room_workload(41, n_boxes=40, resolution=(4, 3, 4), rays=64, precision=precision)
    w.grid.hysteresis = hysteresis
    return w


def make_ctx(w):
    ctx = Context(w.grid)
    ctx.build_scene(w.scene)
    ctx.set_light(w.light)
    return ctx


def check_state(ctx, ref):
    b, p, c = ctx.hysteresis()
    assert np.float32(b) == ref.uniform and np.float32(p) == ref.param and c == ref.counted, \
        ((b, p, c), (ref.uniform, ref.param, ref.counted))


def test_ramp_off_by_default(gpu_lib):
    w = small_room(hysteresis=0.5)
    ctx = make_ctx(w)
    ctx.update(w.orientation(0))
    assert ctx.hysteresis() == (0.5, 0.5, 0)
    ctx.close()


def test_ramp_full_updates_and_atlas(gpu_lib):
    """30 full updates from h = 0 towards 0.97: every blended value and the
    final FP32 atlas against the oracle blended with the same values."""
    w = small_room()
    P = w.grid.probe_count()
    ctx = make_ctx(w)
    ctx.set_target_hysteresis(0.97)
    ref = ReferenceRamp(0.0, 0.97)
    o = Oracle(w.scene)
    c, d = zero_atlas(w.grid)
    st = np.ones(P, np.uint32)
    g = w.grid.copy()
    used = []
    for k in range(30):
        ctx.update(w.orientation(k))
        h = ref.update(P, P)
        used.append(float(h))
        check_state(ctx, ref)
        g.hysteresis = float(h)
        o.update(g, w.light, w.orientation(k), c, d, st)
    assert used[0] == 0.0 and 0.9 < used[-1] <= np.float32(0.97)
    assert len(set(used)) > 10  # it did ramp
    assert rel_err(ctx.get_atlas(abi.ATLAS_COLOR), c, 1e-2).max() <= 1e-4
    assert rel_err(ctx.get_atlas(abi.ATLAS_DEPTH), d, 1e-2).max() <= 1e-4
    ctx.close()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP32, abi.PRECISION_BF16])
def test_ramp_probe_lists_and_schedule(gpu_lib, precision):
    """Partial updates: explicit lists of varying length, then device-side
    selections capped at ProbesPerUpdate; set_grid (updateUniforms) and
    init_probes change the ramp like the reference's calls do."""
    w = small_room(precision, hysteresis=0.2)
    P = w.grid.probe_count()
    ctx = make_ctx(w)
    ctx.set_target_hysteresis(0.95)
    ref = ReferenceRamp(0.2, 0.95)
    rng = np.random.default_rng(5)
    for k in range(25):
        n = int(rng.integers(1, P + 1))
        plist = np.sort(rng.permutation(P)[:n]).astype(np.uint32)
        ctx.update(w.orientation(k), plist)
        ref.update(n, P)
        check_state(ctx, ref)
    # updateUniforms() with a new hysteresis: both values follow it
    g = w.grid.copy()
    g.hysteresis = 0.5
    ctx.set_grid(g)
    ref.param = ref.uniform = np.float32(0.5)
    check_state(ctx, ref)
    # initProbes zeroes the host-side value only
    ctx.init_probes(w.orientation(99))
    ref.param = np.float32(0.0)
    check_state(ctx, ref)
    for k in range(30):
        ctx.update_scheduled(w.orientation(100 + k), 7)
        n = ctx.schedule(with_list=False)["count"]
        ref.update(n, P)
        check_state(ctx, ref)
    # a new target keeps the counter and values; a negative one switches off
    ctx.set_target_hysteresis(0.5)
    ref.target = np.float32(0.5)
    ctx.update(w.orientation(200))
    ref.update(P, P)
    check_state(ctx, ref)
    ctx.set_target_hysteresis(-1)
    assert ctx.hysteresis() == (np.float32(0.5), np.float32(0.5), 0)
    ctx.close()


def test_ramp_rejects_bad_targets(gpu_lib):
    from vulkanexp_gb300.ddgi import DDGIError

    ctx = Context(small_room().grid)
    for t in (float("nan"), float("inf"), 1.5):
        with pytest.raises(DDGIError):
            ctx.set_target_hysteresis(t)
    ctx.close()


def test_autotune_keeps_the_ramp(gpu_lib):
    """ddgi_autotune runs many trial updates; with the ramp on they step it,
    so the ramp's state (and its pending start) is restored with the
    atlases: afterwards the context ramps and blends exactly like a twin
    that was never tuned."""
    w = small_room(hysteresis=0.3)
    tuned, twin = make_ctx(w), make_ctx(w)
    for ctx in (tuned, twin):
        ctx.set_target_hysteresis(0.9)
    tuned.autotune(w.orientation(7), reps=1)
    for k in range(6):
        for ctx in (tuned, twin):
            ctx.update(w.orientation(k))
        assert tuned.hysteresis() == twin.hysteresis()
    for kind in (abi.ATLAS_COLOR, abi.ATLAS_DEPTH):
        a, b = tuned.get_atlas(kind), twin.get_atlas(kind)
        assert (a.view(np.uint32) == b.view(np.uint32)).all()
    tuned.close()
    twin.close()

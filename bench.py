"""DDGI probe-update benchmark.

A step is one probe update (trace + shade of every probe ray, atlas blend with
hysteresis, border copy) of the 32x16x32-probe, 256-ray grid over the seeded
terrain + box-cluster scene (4097 instances, ~1M unique triangles).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is primary probe rays per second (Grays/s) with the scene and atlas
resident in HBM, from CUDA events on the launching stream around each
update; L2 is flushed (a 256 MB write) before every timed update.  `e2e` is
the same metric through the public C-ABI calls a host program makes per
update: host->device upload of the step's inputs (rotation-derived ray
table) and device->host read of both atlases into pinned host memory.

--impl reference times the CPU restatement of the reference's probe update
(the reference itself is Vulkan/GLSL and cannot run here) on the host cores,
on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DDGI update Grays/s & ms/update (32x16x32, 256 rays) vs plain FP32; bwd/fwd ratio"
UNIT = "Grays/s"
L2_FLUSH_BYTES = 256 << 20


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, device):
    """The largest value of x over the ranks of the default process group
    (the slowest replica's time); x itself when there is no group or one
    rank."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measure_l2_copy_gbs(reps=50, mbytes=24):
    """L2-resident copy bandwidth of this GPU, measured here (no driver
    figure exists for it): a device-to-device copy between two `mbytes` MB
    buffers, both far below the 129 MB L2, repeated `reps` times after a
    warm-up; (bytes read + bytes written) / CUDA-event time.  The
    denominator for kernels whose fetches the L2 serves."""
    import torch

    n = mbytes << 20
    a = torch.empty(n, dtype=torch.uint8, device="cuda")
    b = torch.empty(n, dtype=torch.uint8, device="cuda")
    a.fill_(1)
    for _ in range(5):
        b.copy_(a)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        b.copy_(a)
    e1.record()
    torch.cuda.synchronize()
    return 2.0 * n * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, n in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(n)
        out.update(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                   reasons=sorted(reasons), samples=len(rows))
        return out


def cpu_baseline(w, sample_probes, threads=None, oracle=None, orientation=0):
    """Times the CPU oracle on `sample_probes` probes of the workload (0 or
    more than the grid: all of them), one update from a zero atlas, on
    `threads` host threads (default: all cores)."""
    from oracle.oracle import Oracle, zero_atlas

    threads = threads or os.cpu_count()
    own = oracle is None
    t0 = time.perf_counter()
    o = oracle or Oracle(w.scene, threads=threads)
    build_s = time.perf_counter() - t0
    P = w.grid.probe_count()
    n = P if sample_probes <= 0 or sample_probes >= P else sample_probes
    plist = None
    if n < P:
        rng = np.random.default_rng(5 + orientation)
        plist = np.sort(rng.permutation(P)[:n]).astype(np.uint32)
    c, d = zero_atlas(w.grid)
    st = np.ones(P, np.uint32)
    t0 = time.perf_counter()
    o.update(w.grid, w.light, w.orientation(orientation), c, d, st, plist)
    dt = time.perf_counter() - t0
    rays = n * w.grid.rays_per_probe
    if own:
        o.close()
    probes = "all %d probes" % P if n == P else "%d of %d probes" % (n, P)
    sample = "%s x %d rays, 1 update from a zero atlas (%.1f s%s)" % (
        probes, w.grid.rays_per_probe, dt, "; BVH build %.1f s untimed" % build_s if own else "")
    return {"value": rays / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
            "ms_per_update_extrapolated": dt * 1e3 * P / n}


def measure_fp64_error(w, updates, stream, threads=None):
    """Atlas error of the GPU forms against the FP64 oracle on the full
    workload: the BF16 headline form, the FP32 wavefront form and the
    reference-format form (FP32 blend, texels stored rounded to the
    reference's R11G11B10F / RG16F image formats) each run
    `updates` successive updates from a zero atlas with the same rotations as
    the FP64 restatement of the reference's update (its shading and blend in
    double; geometry in FP32, so its hit set is the GPU's).  Per texel
    relative error |gpu - fp64| / max(|fp64|, 1e-2) over every texel of both
    atlases (colour RGB, depth mean and mean square), max and RMS; closest-hit
    IDs of every ray of every update compared with the oracle's.  Rank 0 only,
    outside every timed region."""
    from oracle.oracle import Oracle, zero_atlas
    from vulkanexp_gb300 import abi

    floor = 1e-2
    P = w.grid.probe_count()
    t0 = time.perf_counter()
    o = Oracle(w.scene, threads=threads or os.cpu_count())
    c64, d64 = zero_atlas(w.grid, fp64=True)
    st64 = np.ones(P, np.uint32)
    ctxs = {}
    for name, prec in (("bf16", abi.PRECISION_BF16), ("fp32", abi.PRECISION_FP32),
                       ("reference_format", abi.PRECISION_REFERENCE_FORMAT)):
        ctx, _ = build_context(w, prec, abi.PIPELINE_WAVEFRONT, stream)
        ctx.record_hits(True)
        ctxs[name] = ctx
    mism = {k: 0 for k in ctxs}
    for k in range(updates):
        _, hits = o.update(w.grid, w.light, w.orientation(k), c64, d64, st64, fp64=True, want_hits=True)
        for name, ctx in ctxs.items():
            ctx.update(w.orientation(k), stream=stream)
            gh = ctx.get_hits(P, stream)
            mism[name] += int(((gh["instance"] != hits["instance"]) | (gh["primitive"] != hits["primitive"])).sum())
    out = {"updates": updates, "probes": P, "rays_compared": updates * P * w.grid.rays_per_probe,
           "floor": floor, "oracle": "FP64 CPU restatement (double shading and blend, FP32 geometry)"}
    def err(a, b):
        ec = np.abs(a[0][..., :3].astype(np.float64) - b[0][..., :3]) / np.maximum(np.abs(b[0][..., :3]), floor)
        ed = np.abs(a[1].astype(np.float64) - b[1]) / np.maximum(np.abs(b[1]), floor)
        return {"color_max": float(ec.max()), "color_rms": float(np.sqrt((ec ** 2).mean())),
                "depth_max": float(ed.max()), "depth_rms": float(np.sqrt((ed ** 2).mean()))}

    atl = {}
    for name, ctx in ctxs.items():
        atl[name] = (ctx.get_atlas(abi.ATLAS_COLOR, stream=stream), ctx.get_atlas(abi.ATLAS_DEPTH, stream=stream))
        gs = ctx.get_probe_states(stream)
        ctx.close()
        rec = err(atl[name], (c64, d64))
        rec.update(hit_id_mismatches=mism[name], probe_state_mismatches=int((gs != st64).sum()))
        if name == "bf16":
            out.update(rec)  # the headline form's numbers at the top
        else:
            out[{"fp32": "fp32_wavefront", "reference_format": "reference_format"}[name]] = rec
    # how far the FP32 and BF16 forms drift from the reference-format form
    # (the atlas the reference's R11G11B10F / RG16F images would hold)
    out["drift_from_reference_format"] = {"fp32_wavefront": err(atl["fp32"], atl["reference_format"]),
                                          "bf16": err(atl["bf16"], atl["reference_format"])}
    o.close()
    out["seconds"] = time.perf_counter() - t0
    return out


def run_reference(args, w):
    """The reference arm: the CPU restatement of the reference's probe-update
    shaders on all host cores (the reference itself is Vulkan/GLSL), each
    step one update of a bounded probe sample (--ref-probes) with a new
    ray-set rotation; the median over the timed steps."""
    from oracle.oracle import Oracle

    rank, world, _ = dist_env()
    if rank != 0:
        return
    o = Oracle(w.scene, threads=os.cpu_count())
    vals = []
    for k in range(args.warmup):
        cpu_baseline(w, args.ref_probes, oracle=o, orientation=k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        vals.append(cpu_baseline(w, args.ref_probes, oracle=o, orientation=args.warmup + k))
    wall = time.perf_counter() - t0
    o.close()
    v = statistics.median(x["value"] for x in vals)
    cb = dict(vals[0])
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall * 1e3 / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": config_dict(w, args, "fp32"), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference is Vulkan/GLSL (no graphics stack on this box); timed here is the C++ restatement "
                    "of its probe-update shaders on the host cores"}
    print(json.dumps(line), flush=True)


def config_dict(w, args, precision="bf16"):
    """Workload description; `precision` names the timed form ("bf16": FP32
    trace, BF16 tensor-core blend, FP16 atlas; "fp32": the CPU restatement's
    arithmetic)."""
    g = w.grid
    return {"workload": w.name, "probes": g.probe_count(), "grid": list(g.resolution), "rays_per_probe":
            g.rays_per_probe, "triangles": w.scene.triangle_count, "unique_triangles": w.scene.unique_triangle_count,
            "instances": int(len(w.scene.instances)), "color_res": g.color_res, "depth_res": g.depth_res,
            "precision": precision, "l2": "flushed (256 MB write) before each timed update", "seed": w.seed}


def build_context(w, precision, pipeline, stream):
    from vulkanexp_gb300 import abi
    from vulkanexp_gb300.ddgi import Context

    g = w.grid.copy()
    g.precision = precision
    ctx = Context(g)
    ctx.set_pipeline(pipeline)
    t0 = time.perf_counter()
    ctx.build_scene(w.scene, stream)
    build_s = time.perf_counter() - t0
    ctx.set_light(w.light)
    return ctx, build_s


def time_updates(ctx, w, steps, warmup, stream, flush, first=0):
    """Device time of `steps` updates (CUDA events on the launching stream,
    L2 flushed before each), after `warmup` untimed updates."""
    import torch

    for k in range(warmup):
        ctx.update(w.orientation(first + k), stream=stream)
    ctx.synchronize(stream)
    ctx.enable_timing(True)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    stages = {"trace_shade": [], "primary_traversal": [], "blend_border": []}
    for k in range(steps):
        flush.fill_(k & 255)
        ev[k][0].record(stream)
        ctx.update(w.orientation(first + warmup + k), stream=stream)
        ev[k][1].record(stream)
        t = ctx.timings()  # waits for this update's last event
        stages["trace_shade"].append(t["trace_ms"])
        stages["primary_traversal"].append(t["primary_ms"])
        stages["blend_border"].append(t["blend_ms"])
    torch.cuda.synchronize()
    ctx.enable_timing(False)
    ms = [a.elapsed_time(b) for a, b in ev]
    return float(np.mean(ms)), {k: float(np.mean(v)) for k, v in stages.items()}


def measure_differentiation(stream, reps=3):
    """Forward (K recorded updates) and backward (adjoint through them) on the
    differentiation workload: room + 1000 boxes, 16x8x16 probes, 256 rays,
    K = 8, checkpoints every 2 updates.  CUDA events around each call."""
    import torch

    from vulkanexp_gb300 import abi, scenes
    from vulkanexp_gb300.ddgi import Context

    w = scenes.workload(3)
    K = 8
    orients = np.stack([w.orientation(k) for k in range(K)])
    ctx = Context(w.grid)
    ctx.build_scene(w.scene, stream)
    ctx.set_light(w.light)
    zc = np.zeros(ctx.atlas_shape(abi.ATLAS_COLOR), np.float32)
    zd = np.zeros(ctx.atlas_shape(abi.ATLAS_DEPTH), np.float32)
    grad = np.ones_like(zc)
    fwd, bwd = [], []
    for rep in range(reps + 1):
        ctx.set_atlas(abi.ATLAS_COLOR, zc, stream)
        ctx.set_atlas(abi.ATLAS_DEPTH, zd, stream)
        torch.cuda.synchronize()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        ctx.forward_record(orients, 2, stream)
        e1.record(stream)
        ctx.backward(grad, len(w.scene.materials), stream)
        e2.record(stream)
        torch.cuda.synchronize()
        if rep > 0:  # the first repetition warms up
            fwd.append(e0.elapsed_time(e1))
            bwd.append(e1.elapsed_time(e2))
    ctx.close()
    f, b = float(np.mean(fwd)), float(np.mean(bwd))
    return {"workload": w.name, "updates": K, "checkpoint_every": 2, "forward_ms": f, "backward_ms": b,
            "bwd_fwd_ratio": b / f, "parameters": len(w.scene.materials) * 3 + 6}


def measure_batching(stream, steps, warmup, flush):
    """The batching workload: 48 seeded volumes (room or terrain generator,
    5k-300k triangles, 4x4x4..24x12x24 probes, 64-512 rays, 8/16 or 6/14
    tiles, FP32 or BF16 form) updated together per step: one persistent
    work-queue traversal over every volume's rays, replayed from a CUDA graph,
    launch parameters from the autotuner.  Reports aggregate primary rays/s,
    per-volume completion time (update start -> the volume's last blend work
    item) p50/p99 over all timed steps, and the same volumes updated one
    context at a time for comparison.  CUDA events on the launching stream;
    the per-ray buffers (~1.3 GB) exceed L2, which is also flushed."""
    import torch

    from vulkanexp_gb300 import scenes
    from vulkanexp_gb300.ddgi import Batch, Context

    ws = scenes.batch_workloads()
    ctxs = []
    for w in ws:
        c = Context(w.grid)
        c.build_scene(w.scene, stream)
        c.set_light(w.light)
        ctxs.append(c)
    b = Batch(ctxs, stream)

    def orient(k):
        return np.stack([scenes.random_orientation(w.seed, k) for w in ws])

    t0 = time.perf_counter()
    tuning = b.autotune(orient(0), reps=3, stream=stream)
    tune_s = time.perf_counter() - t0
    for k in range(warmup):
        b.update(orient(1 + k), stream)
    b.synchronize(stream)
    ms, comp = [], []
    for k in range(steps):
        flush.fill_(k & 255)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.update(orient(1 + warmup + k), stream)
        e1.record(stream)
        b.synchronize(stream)
        ms.append(e0.elapsed_time(e1))
        comp.append(b.completion_ms())
    seq = []
    for k in range(steps):
        flush.fill_(k & 255)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for c, w in zip(ctxs, ws):
            c.update(scenes.random_orientation(w.seed, 100 + k), stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        seq.append(e0.elapsed_time(e1))
    rays = b.ray_count
    comp = np.concatenate(comp)
    t = float(np.median(ms))
    out = {"workload": "48 volumes (seed 1238): room/terrain, 5k-300k triangles, 4x4x4..24x12x24 probes, "
                       "64-512 rays, 8/16 or 6/14 tiles, mixed FP32/BF16",
           "volumes": len(ws), "bf16_volumes": int(sum(w.grid.precision for w in ws)),
           "probes": int(sum(w.grid.probe_count() for w in ws)), "rays_per_update": rays,
           "unique_triangles": int(sum(w.scene.unique_triangle_count for w in ws)),
           "ms_per_update": t, "value": rays / (t * 1e-3) / 1e9, "unit": "Grays/s",
           "completion_ms_p50": float(np.percentile(comp, 50)), "completion_ms_p99": float(np.percentile(comp, 99)),
           "tuning": tuning, "autotune_s": tune_s, "graph": True,
           "one_by_one_ms": float(np.median(seq)), "speedup_vs_one_by_one": float(np.median(seq)) / t}
    b.close()
    for c in ctxs:
        c.close()
    return out


def profiled_traffic(summary, key="traffic_bytes_per_launch"):
    """Bytes per launch recorded in a committed ncu summary under profiles/
    (one capture of the same workload), or None: by default the DRAM bytes
    (dram__bytes_read.sum + dram__bytes_write.sum); key
    "l2_traffic_bytes_per_launch" gives the L2 bytes (lts__t_bytes.sum)."""
    import re

    try:
        with open(os.path.join(ROOT, "profiles", summary)) as f:
            m = re.search(r"^" + key + r":\s*(\d+)", f.read(), re.M)
    except OSError:
        return None
    return int(m.group(1)) if m else None


def rendered_gbuffer(ctx, w, width, height):
    """A G-buffer as the reference's GBuffer pass would leave it for a camera
    view of the scene: one camera ray per pixel (60-degree vertical field of
    view, from above one side of the probe grid towards the ground at its
    centre) traced
    by ddgi_trace_rays; position and depth from the hit, the interpolated
    vertex normal in world space, the hit material's albedo, roughness,
    metalness and emissive, direct light 1 where a shadow ray towards the
    sun (tmin 0.1, any hit) escapes, reflection 0; sky pixels (misses) carry
    depth 0 and the view direction in position.xyz.  Host arrays."""
    from vulkanexp_gb300 import abi

    g, sc = w.grid, w.scene
    lo, hi = np.array(g.extent_min, np.float64), np.array(g.extent_max, np.float64)
    c, ext = 0.5 * (lo + hi), hi - lo
    eye = np.array([c[0], lo[1] + 0.8 * ext[1], lo[2] + 0.05 * ext[2]])
    fwd = np.array([c[0], lo[1], c[2]]) - eye  # towards the ground at the grid's centre
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, [0.0, 1.0, 0.0])
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    th = np.tan(np.radians(30.0))
    px = (np.arange(width) + 0.5) / width * 2 - 1
    py = 1 - (np.arange(height) + 0.5) / height * 2
    X, Y = np.meshgrid(px * th * width / height, py * th)
    d = fwd[None, None] + X[..., None] * right[None, None] + Y[..., None] * up[None, None]
    d = (d / np.linalg.norm(d, axis=-1, keepdims=True)).reshape(-1, 3).astype(np.float32)
    n = len(d)
    o = np.repeat(eye[None].astype(np.float32), n, 0)
    tmax = float(np.linalg.norm(ext)) * 4
    hits, bary = ctx.trace_rays(o, d, 0.01, tmax, 0xFF, False)
    hit = hits["instance"] != abi.MISS
    t = np.where(hit, hits["t"], 0.0).astype(np.float32)
    pos = np.where(hit[:, None], o + d * t[:, None], d)
    inst = sc.instances[np.where(hit, hits["instance"], 0)]
    off = sc.offsets[inst["custom_index"]]
    tri = off["index_offset"][:, None] + 3 * hits["primitive"][:, None].astype(np.int64) + np.arange(3)[None]
    vi = off["vertex_offset"][:, None] + sc.indices[np.where(hit[:, None], tri, 0)]
    nv = sc.vertices["normal"][vi].astype(np.float64)
    b1, b2 = bary[:, 0:1].astype(np.float64), bary[:, 1:2].astype(np.float64)
    nrm = nv[:, 0] * (1 - b1 - b2) + nv[:, 1] * b1 + nv[:, 2] * b2
    A = inst["transform"].reshape(-1, 3, 4)[:, :, :3].astype(np.float64)
    nrm = np.einsum("kij,kj->ki", np.linalg.inv(A).transpose(0, 2, 1), nrm)  # normal matrix
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    mat = sc.materials[off["material_index"]]
    sun = np.repeat(np.array(w.light.direction[:3], np.float32)[None], n, 0)
    sh, _ = ctx.trace_rays(pos.astype(np.float32), sun, 0.1, 1e4, 0xFF, True)
    lit = (sh["instance"] == abi.MISS) & hit
    f4 = lambda a: np.ascontiguousarray(a.reshape(height, width, 4), np.float32)
    z = np.zeros((n, 1))
    return {"position_depth": f4(np.concatenate([pos, t[:, None]], 1)),
            "normal_metalness": f4(np.concatenate([nrm, mat["metallic"][:, None]], 1)),
            "albedo_roughness": f4(np.concatenate([mat["base_color"], mat["roughness"][:, None]], 1)),
            "emissive": f4(np.concatenate([mat["emissive"], z], 1)),
            "direct_light": np.ascontiguousarray(lit.reshape(height, width), np.float32),
            "reflection": f4(np.zeros((n, 4)))}, eye, float(hit.mean())


def measure_final_gather(ctx, w, stream, flush, reps=10, width=1920, height=1080, view="scattered"):
    """The atlas consumer: FinalGather.frag over a 1920x1080 G-buffer on the
    context's current atlas.  view "rendered": the G-buffer of a camera view
    of the scene (rendered_gbuffer), whose neighbouring pixels look up
    neighbouring probes, as a renderer's do; "scattered": a seeded
    worst case (positions uniform inside the probe grid, random normals and
    materials, 10% sky pixels), where no two pixels of a warp share probes.
    CUDA events over `reps` launches, L2 flushed before each; algorithmic
    bytes per pixel: the G-buffer read (4 x float4 + float + float4
    reflection) and the float4 written = 100 B (probe-atlas texels are
    L2-resident)."""
    import torch

    g = w.grid
    n = width * height
    extra = {}
    if view == "rendered":
        host, eye, hit_frac = rendered_gbuffer(ctx, w, width, height)
        gb = {k: torch.from_numpy(v).cuda() for k, v in host.items()}
        origin = [float(x) for x in eye]
        extra = {"surface_pixels": hit_frac}
    else:
        gen = torch.Generator(device="cuda").manual_seed(1239)
        lo = torch.tensor(list(g.extent_min), device="cuda")
        hi = torch.tensor(list(g.extent_max), device="cuda")
        pos = lo + (hi - lo) * torch.rand((n, 3), device="cuda", generator=gen)
        depth = torch.where(torch.rand(n, device="cuda", generator=gen) < 0.1, 0.0, 1.0)
        u = lambda *sh: torch.rand(sh, device="cuda", generator=gen)
        gb = {"position_depth": torch.cat([pos, depth[:, None]], 1).reshape(height, width, 4).contiguous(),
              "normal_metalness": torch.cat([torch.randn((n, 3), device="cuda", generator=gen), u(n, 1)], 1)
              .reshape(height, width, 4).contiguous(),
              "albedo_roughness": u(n, 4).reshape(height, width, 4).contiguous(),
              "emissive": (0.1 * u(n, 4)).reshape(height, width, 4).contiguous(),
              "direct_light": u(n).reshape(height, width).contiguous(),
              "reflection": u(n, 4).reshape(height, width, 4).contiguous()}
        origin = [0.5 * (a + b) for a, b in zip(g.extent_min, g.extent_max)]
    out = torch.empty((height, width, 4), dtype=torch.float32, device="cuda")
    for _ in range(3):
        ctx.final_gather(gb, origin, out, stream)
    ms = []
    for k in range(reps):
        flush.fill_(k & 255)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.final_gather(gb, origin, out, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    t = float(np.median(ms))
    hbm, _, _ = load_peaks()
    gbs = n * 100 / (t * 1e-3) / 1e9
    return dict({"kernel": "k_final_gather", "view": view, "pixels": n, "ms": t,
                 "gpixels_per_s": n / (t * 1e-3) / 1e9, "achieved_gbs": gbs, "frac_hbm": gbs / hbm,
                 "bytes_per_pixel": 100}, **extra)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--cpu-probes", type=int, default=0,
                    help="probes of the CPU-baseline sample (0: the whole grid, one full update)")
    ap.add_argument("--ref-probes", type=int, default=4096,
                    help="probes per step of the reference arm's sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--err-updates", type=int, default=10,
                    help="updates of the atlas-error check against the FP64 oracle (0: skip)")
    ap.add_argument("--only", default=None, choices=["batching"],
                    help="run one sub-measurement alone and print it")
    ap.add_argument("--headline-only", action="store_true",
                    help="the three update forms, e2e and rooflines only (no differentiation, batching, final "
                         "gather or CPU baseline): the profiling command for the launch list")
    ap.add_argument("--profile", action="store_true",
                    help="profiling target: scene build, then two BF16 wavefront updates and two FP32 ones, no timing")
    args = ap.parse_args()

    rank, world, local = dist_env()
    from vulkanexp_gb300 import scenes

    w = scenes.workload(args.config)
    if args.impl == "reference":
        run_reference(args, w)
        return

    import torch

    from vulkanexp_gb300 import abi, build

    build.build()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    P, R = w.grid.probe_count(), w.grid.rays_per_probe

    if args.profile:
        flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        for prec in (abi.PRECISION_BF16, abi.PRECISION_FP32):
            ctx, _ = build_context(w, prec, abi.PIPELINE_WAVEFRONT, stream)
            for k in range(2):
                ctx.update(w.orientation(k), stream=stream)
            ctx.synchronize(stream)
            if prec == abi.PRECISION_BF16:  # one final gather over the BF16 atlas
                measure_final_gather(ctx, w, stream, flush, reps=1, view="rendered")
            ctx.close()
        print(json.dumps({"profile_target": w.name, "updates": 4, "final_gathers": 4}), flush=True)
        return

    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    if args.only == "batching":
        print(json.dumps({"batching": measure_batching(stream, args.steps, args.warmup, flush)}), flush=True)
        return
    forms = {}
    sampler = ClockSampler(local)
    sampler.start()
    # the reference-like plain FP32 form, the FP32 wavefront form, and the
    # headline: wavefront trace + BF16 tensor-core blend with an FP16 atlas
    for name, prec, pipe in (("plain_fp32", abi.PRECISION_FP32, abi.PIPELINE_FUSED),
                             ("wavefront_fp32", abi.PRECISION_FP32, abi.PIPELINE_WAVEFRONT),
                             ("wavefront_bf16", abi.PRECISION_BF16, abi.PIPELINE_WAVEFRONT)):
        ctx, build_s = build_context(w, prec, pipe, stream)
        if world > 1:
            torch.distributed.barrier()
        ms, stages = time_updates(ctx, w, args.steps, args.warmup, stream, flush)
        info = ctx.scene_info()
        forms[name] = {"ms_per_update": ms, "value": P * R / (ms * 1e-3) / 1e9, "stage_ms": stages,
                       "scene_build_s": build_s, "mesh_tree_build_gpu_ms": info["tree_build_ms"],
                       "tree_nodes": info["nodes"], "triangle_refs": info["tri_refs"]}
        if name != "wavefront_bf16":
            ctx.close()
    clocks = sampler.stop()
    # every per-form time is the slowest replica's
    for f in forms.values():
        f["ms_per_update"] = max_over_ranks(f["ms_per_update"], "cuda")
        f["value"] = world * P * R / (f["ms_per_update"] * 1e-3) / 1e9
        f["stage_ms"] = {k: max_over_ranks(v, "cuda") for k, v in f["stage_ms"].items()}
    head = forms["wavefront_bf16"]
    ms = head["ms_per_update"]
    value = world * P * R / (ms * 1e-3) / 1e9

    # e2e through the host-buffer API: the step's ray table up, both atlases
    # down into pinned host memory in their storage format (FP16 texels, the
    # format a renderer samples; the reference's atlases are 16-bit images)
    ch, cw, cc = ctx.atlas_shape(abi.ATLAS_COLOR)
    dh, dw, dc = ctx.atlas_shape(abi.ATLAS_DEPTH)
    host_c = torch.empty((ch, cw, cc), dtype=torch.float16, pin_memory=True).numpy()
    host_d = torch.empty((dh, dw, dc), dtype=torch.float16, pin_memory=True).numpy()
    e2e_ms = []
    if world > 1:
        torch.distributed.barrier()
    for k in range(max(args.steps, 1)):
        flush.fill_(k & 255)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.update(w.orientation(k), stream=stream)
        ctx.get_atlas_raw(abi.ATLAS_COLOR, host_c, stream)
        ctx.get_atlas_raw(abi.ATLAS_DEPTH, host_d, stream)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_mean = max_over_ranks(float(np.mean(e2e_ms)), "cuda")
    e2e_val = world * P * R / (e2e_mean * 1e-3) / 1e9

    # rooflines: the dominant kernel (primary traversal, L1/L2-resident node
    # fetches counted per launch) and the tensor-core blend
    fetches = ctx.count_fetches(w.orientation(0), stream=stream)
    hbm, bf16_peak, peak_kind = load_peaks()
    prim_ms = head["stage_ms"]["primary_traversal"]
    alg_bytes = fetches["nodes"] * 64 + fetches["tris"] * 48 + fetches["instances"] * 64
    achieved = alg_bytes / (prim_ms * 1e-3) / 1e9
    l2 = measure_l2_copy_gbs()
    l2_bytes = profiled_traffic("k_primary_terrain_32x16x32_r256.md", "l2_traffic_bytes_per_launch")
    roofline = {"bound": "hbm", "kernel": "k_primary", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_source": peak_kind,
                "l2_copy_gbs": l2, "frac_l2": achieved / l2,
                "l2_source": "measured in this run: L2-resident 24 MB device copy (read + write bytes / time)",
                "traffic": profiled_traffic("k_primary_terrain_32x16x32_r256.md"),
                "traffic_source": "ncu capture, profiles/k_primary_terrain_32x16x32_r256.md",
                "l2_traffic": l2_bytes,
                "l2_achieved_gbs": l2_bytes / (prim_ms * 1e-3) / 1e9 if l2_bytes else None,
                "l2_traffic_source": "lts__t_bytes.sum of one ncu capture, profiles/k_primary_terrain_32x16x32_r256.md",
                "algorithmic_bytes_per_launch": alg_bytes, "kernel_ms": prim_ms,
                "note": "fetch-counted node/triangle/instance bytes of the primary rays; they are served mostly by "
                        "L1/L2, so frac > 1 is cache reuse, not DRAM traffic",
                "fetches_per_launch": fetches}
    nc, nd = w.grid.color_res - 2, w.grid.depth_res - 2
    blend_flop = 2.0 * P * R * (nc * nc * 3 + nd * nd * 2)
    blend_ms = head["stage_ms"]["blend_border"]
    blend_bytes = P * R * 16 + 2 * (w.grid.atlas_shape(0)[0] * w.grid.atlas_shape(0)[1] * 8 +
                                     w.grid.atlas_shape(1)[0] * w.grid.atlas_shape(1)[1] * 4)
    roofline_blend = {"kernel": "k_blend_tc (+ k_tc_weights)", "bound": "hbm", "kernel_ms": blend_ms,
                      "algorithmic_bytes": blend_bytes, "achieved_gbs": blend_bytes / (blend_ms * 1e-3) / 1e9,
                      "frac_hbm": blend_bytes / (blend_ms * 1e-3) / 1e9 / hbm,
                      "useful_tflops": blend_flop / (blend_ms * 1e-3) / 1e12, "peak_bf16_tflops": bf16_peak,
                      "traffic": profiled_traffic("k_blend_tc_terrain_32x16x32_r256.md"),
                      "traffic_source": "ncu capture, profiles/k_blend_tc_terrain_32x16x32_r256.md"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 trace / bf16 blend", "data": "synthetic (seeded)",
            "config": config_dict(w, args), "impl": "ours",
            "form": "wavefront trace (persistent traversal) + BF16 tcgen05 blend, FP16 atlas",
            "forms": forms,
            # against the reference-like fused FP32 form, and against the FP32
            # wavefront form (same trees and traversal: the BF16 blend's own gain)
            "speedup_vs_plain_fp32": forms["plain_fp32"]["ms_per_update"] / head["ms_per_update"],
            "speedup_vs_wavefront_fp32": forms["wavefront_fp32"]["ms_per_update"] / head["ms_per_update"],
            # per update: k_primary, k_shade_classify, k_shade_front, k_shadow, k_tc_weights, k_blend_tc
            "gpu_launches": 6 * args.steps, "clocks": clocks, "roofline": roofline,
            "roofline_blend": roofline_blend,
            "e2e": {"value": e2e_val, "unit": UNIT, "ms_per_step": e2e_mean,
                    "h2d_bytes_per_step": R * 20, "d2h_bytes_per_step": int(host_c.nbytes + host_d.nbytes)},
            # sanity of the last e2e step's result as read back
            "atlas_finite": bool(np.isfinite(host_c).all() and np.isfinite(host_d).all())}
    if not args.headline_only:
        line["final_gather"] = measure_final_gather(ctx, w, stream, flush, view="rendered")
        line["final_gather_scattered"] = measure_final_gather(ctx, w, stream, flush, view="scattered")
    ctx.close()
    if not args.headline_only:
        line["differentiation"] = measure_differentiation(stream)
        line["batching"] = measure_batching(stream, args.steps, args.warmup, flush)
    if rank == 0 and world == 1 and not args.no_cpu_baseline and not args.headline_only:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_probes)
        if args.err_updates > 0:
            line["atlas_err_vs_fp64"] = measure_fp64_error(w, args.err_updates, stream)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""Python binding of the C ABI in include/ddgi.h.

`IrradianceProbes` keeps the names of VulkanExp's class
(src/IrradianceProbes.hpp:16-129): `GridParameters`, `TargetHysteresis`,
`init`, `initProbes`, `update`, `updateUniforms`, `setLightBuffer`,
`getProbeCount`.  The scene binding that the reference does through
descriptors (`writeDescriptorSet`, src/IrradianceProbes.cpp:312-321) is
`setScene`, which builds the GPU acceleration structures.

There is no CPU fallback: if the CUDA library cannot be loaded, every call
raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import HIT_DTYPE, BatchTuning, GBuffer, GridDesc, Light, SceneDesc, SceneInfo, Timings, TraceTuning

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libddgi_gb300.so")


class DDGIError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (abi.STATUS_NAMES.get(status, status), message))
        self.status = status


_lib = None

# (name, restype, argtypes) of every exported entry point
_SIGNATURES = [
    ("ddgi_status_string", C.c_char_p, [C.c_int]),
    ("ddgi_last_error", C.c_char_p, [C.c_void_p]),
    ("ddgi_create", C.c_int, [C.POINTER(GridDesc), C.POINTER(C.c_void_p)]),
    ("ddgi_destroy", C.c_int, [C.c_void_p]),
    ("ddgi_set_grid", C.c_int, [C.c_void_p, C.POINTER(GridDesc)]),
    ("ddgi_get_grid", C.c_int, [C.c_void_p, C.POINTER(GridDesc)]),
    ("ddgi_probe_count", C.c_uint32, [C.c_void_p]),
    ("ddgi_scene_build", C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.c_void_p]),
    ("ddgi_set_light", C.c_int, [C.c_void_p, C.POINTER(Light)]),
    ("ddgi_update", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    ("ddgi_get_atlas", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p]),
    ("ddgi_set_atlas", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p]),
    ("ddgi_atlas_dims", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                  C.POINTER(C.c_uint32)]),
    ("ddgi_get_ray_records", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    ("ddgi_record_hits", C.c_int, [C.c_void_p, C.c_int]),
    ("ddgi_get_hits", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    ("ddgi_get_ray_directions", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    ("ddgi_get_probe_states", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    ("ddgi_set_probe_states", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    ("ddgi_atlas_device_ptr", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    ("ddgi_trace_rays", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_float, C.c_float, C.c_uint32,
                                  C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddgi_count_fetches", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("ddgi_synchronize", C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    ("ddgi_get_timings", C.c_int, [C.c_void_p, C.POINTER(Timings)]),
    ("ddgi_enable_timing", C.c_int, [C.c_void_p, C.c_int]),
    ("ddgi_set_pipeline", C.c_int, [C.c_void_p, C.c_int]),
    ("ddgi_blend_records", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_size_t,
                                     C.c_void_p]),
    ("ddgi_set_materials", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    ("ddgi_forward_record", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]),
    ("ddgi_backward", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddgi_blend_records_noalloc", C.c_int, [C.POINTER(GridDesc), C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p]),
    ("ddgi_update_instances", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p]),
    ("ddgi_final_gather", C.c_int, [C.c_void_p, C.POINTER(GBuffer), C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddgi_set_trace_tuning", C.c_int, [C.c_void_p, C.POINTER(TraceTuning)]),
    ("ddgi_set_target_hysteresis", C.c_int, [C.c_void_p, C.c_float]),
    ("ddgi_set_sky_mode", C.c_int, [C.c_void_p, C.c_int]),
    ("ddgi_get_hysteresis", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddgi_set_leaf_size", C.c_int, [C.c_void_p, C.c_uint32]),
    ("ddgi_set_build_mode", C.c_int, [C.c_void_p, C.c_int]),
    ("ddgi_get_scene_info", C.c_int, [C.c_void_p, C.POINTER(SceneInfo)]),
    ("ddgi_read_trees", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p]),
    ("ddgi_get_atlas_raw", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p]),
    ("ddgi_set_spatial_splits", C.c_int, [C.c_void_p, C.c_float]),
    ("ddgi_inject_fault", C.c_int, [C.c_void_p, C.c_uint32]),
    ("ddgi_atlas_save", C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p]),
    ("ddgi_atlas_load", C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p]),
    ("ddgi_get_trace_tuning", C.c_int, [C.c_void_p, C.POINTER(TraceTuning)]),
    ("ddgi_autotune", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(TraceTuning)]),
    ("ddgi_init_probes", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddgi_update_scheduled", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    ("ddgi_get_schedule", C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                    C.c_void_p, C.c_size_t, C.c_void_p]),
    ("ddgi_set_schedule", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]),
    ("ddgi_batch_create", C.c_int, [C.POINTER(C.c_void_p), C.c_uint32, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("ddgi_batch_destroy", C.c_int, [C.c_void_p]),
    ("ddgi_batch_last_error", C.c_char_p, [C.c_void_p]),
    ("ddgi_batch_ray_count", C.c_uint64, [C.c_void_p]),
    ("ddgi_batch_get_tuning", C.c_int, [C.c_void_p, C.POINTER(BatchTuning)]),
    ("ddgi_batch_set_tuning", C.c_int, [C.c_void_p, C.POINTER(BatchTuning)]),
    ("ddgi_batch_use_graph", C.c_int, [C.c_void_p, C.c_int]),
    ("ddgi_batch_update", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddgi_batch_synchronize", C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    ("ddgi_batch_completion_ms", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    ("ddgi_batch_autotune", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(BatchTuning)]),
]


def load_library(path=None):
    """Loads libddgi_gb300.so (built by vulkanexp_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise DDGIError(2, "CUDA library %s is missing: run vulkanexp_gb300.build.build()" % path)
    lib = C.CDLL(path)
    for name, res, args in _SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return [s[0] for s in _SIGNATURES]


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _stream_ptr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(int(getattr(stream, "cuda_stream", stream)))


def scene_desc(scene):
    d = SceneDesc()
    d.vertices = scene.vertices.ctypes.data
    d.vertex_count = len(scene.vertices)
    d.indices = scene.indices.ctypes.data
    d.index_count = scene.indices.size
    d.meshes = scene.meshes.ctypes.data
    d.mesh_count = len(scene.meshes)
    d.instances = scene.instances.ctypes.data
    d.instance_count = len(scene.instances)
    d.offsets = scene.offsets.ctypes.data
    d.offset_count = len(scene.offsets)
    d.materials = scene.materials.ctypes.data
    d.material_count = len(scene.materials)
    return d


class Context:
    """Owns one ddgi_ctx."""

    def __init__(self, grid):
        self.lib = load_library()
        h = C.c_void_p()
        self._check(self.lib.ddgi_create(C.byref(grid), C.byref(h)), ctx=None)
        self.h = h
        self.grid = grid.copy()
        self._scene_keepalive = None

    def _check(self, status, ctx="self"):
        if status != 0:
            handle = self.h if ctx == "self" else None
            msg = self.lib.ddgi_last_error(handle).decode() if handle else ""
            raise DDGIError(status, msg)

    def close(self):
        if getattr(self, "h", None):
            self.lib.ddgi_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- setup -----------------------------------------------------------
    def set_grid(self, grid):
        self._check(self.lib.ddgi_set_grid(self.h, C.byref(grid)))
        self.grid = grid.copy()

    def build_scene(self, scene, stream=None):
        d = scene_desc(scene)
        self._check(self.lib.ddgi_scene_build(self.h, C.byref(d), _stream_ptr(stream)))

    def update_instances(self, transforms, ids=None, rebuild=False, stream=None):
        """New object-to-world transforms (n x 12, row-major 3x4) for the
        instances `ids` (default 0..n-1): top-level refit, or rebuild."""
        t = np.ascontiguousarray(transforms, np.float32).reshape(-1, 12)
        i = None if ids is None else np.ascontiguousarray(ids, np.uint32)
        self._check(self.lib.ddgi_update_instances(self.h, _ptr(i), _ptr(t), len(t), int(bool(rebuild)),
                                                   _stream_ptr(stream)))

    def set_sky_mode(self, mode):
        """abi.SKY_CONSTANT (default) or abi.SKY_ATMOSPHERE."""
        self._check(self.lib.ddgi_set_sky_mode(self.h, int(mode)))

    def set_target_hysteresis(self, target):
        """Hysteresis ramp towards `target` (None or negative: off)."""
        self._check(self.lib.ddgi_set_target_hysteresis(self.h, -1.0 if target is None else float(target)))

    def hysteresis(self, stream=None):
        """(blended, host-side value, probes counted) of the ramp."""
        b, p, c = C.c_float(), C.c_float(), C.c_uint32()
        self._check(self.lib.ddgi_get_hysteresis(self.h, C.byref(b), C.byref(p), C.byref(c), _stream_ptr(stream)))
        return b.value, p.value, c.value

    def set_light(self, light):
        self._check(self.lib.ddgi_set_light(self.h, C.byref(light)))

    def record_hits(self, on=True):
        self._check(self.lib.ddgi_record_hits(self.h, int(on)))

    def enable_timing(self, on=True):
        self._check(self.lib.ddgi_enable_timing(self.h, int(on)))

    def set_pipeline(self, pipeline):
        self._check(self.lib.ddgi_set_pipeline(self.h, int(pipeline)))

    # ---- update ----------------------------------------------------------
    def update(self, orientation, probe_list=None, stream=None):
        o = np.ascontiguousarray(orientation, np.float32).reshape(9)
        pl = None if probe_list is None else np.ascontiguousarray(probe_list, np.uint32)
        self._check(self.lib.ddgi_update(self.h, _ptr(o), _ptr(pl), 0 if pl is None else len(pl),
                                         _stream_ptr(stream)))

    def final_gather(self, gbuffer, origin, out, stream=None):
        """FinalGather.frag over a device G-buffer.  gbuffer: dict of
        contiguous float32 CUDA tensors position_depth, normal_metalness,
        albedo_roughness, emissive (H x W x 4), direct_light (H x W) and
        optionally reflection (H x W x 4); out: H x W x 4 CUDA tensor."""
        h, w = out.shape[0], out.shape[1]
        gb = GBuffer()
        for k in ("position_depth", "normal_metalness", "albedo_roughness", "emissive", "direct_light"):
            t = gbuffer[k]
            assert t.is_cuda and t.is_contiguous() and t.shape[0] == h and t.shape[1] == w
            setattr(gb, k, t.data_ptr())
        r = gbuffer.get("reflection")
        gb.reflection = None if r is None else r.data_ptr()
        gb.width, gb.height = w, h
        o = np.ascontiguousarray(origin, np.float32).reshape(3)
        self._check(self.lib.ddgi_final_gather(self.h, C.byref(gb), _ptr(o), C.c_void_p(out.data_ptr()),
                                               _stream_ptr(stream)))

    def set_leaf_size(self, max_triangles):
        """Triangles per mesh-tree leaf for the next build_scene."""
        self._check(self.lib.ddgi_set_leaf_size(self.h, int(max_triangles)))

    def set_build_mode(self, mode):
        """Tree builder for the next build_scene: "fast_trace" (SAH trees
        with spatial splits built on the GPU), "fast_build" (GPU linear BVHs)
        or "fast_trace_host" (the fast-trace trees built on the host)."""
        modes = {"fast_trace": 0, "fast_build": 1, "fast_trace_host": 2}
        if mode not in modes:
            raise ValueError("build mode %r: want one of %s" % (mode, sorted(modes)))
        self._check(self.lib.ddgi_set_build_mode(self.h, modes[mode]))

    def set_spatial_splits(self, overlap):
        """Spatial splits of the next build_scene's fast-trace mesh trees
        (overlap fraction of the root's surface area; 0 = off)."""
        self._check(self.lib.ddgi_set_spatial_splits(self.h, float(overlap)))

    def trace_tuning(self):
        t = TraceTuning()
        self._check(self.lib.ddgi_get_trace_tuning(self.h, C.byref(t)))
        return {k: int(getattr(t, k)) for k, _ in t._fields_}

    def set_trace_tuning(self, **kw):
        t = TraceTuning()
        self._check(self.lib.ddgi_get_trace_tuning(self.h, C.byref(t)))
        for k, v in kw.items():
            setattr(t, k, int(v))
        self._check(self.lib.ddgi_set_trace_tuning(self.h, C.byref(t)))

    def autotune(self, orientation, reps=3, stream=None):
        """Picks the fastest traversal launch tuning (see ddgi_autotune)."""
        o = np.ascontiguousarray(orientation, np.float32).reshape(9)
        t = TraceTuning()
        self._check(self.lib.ddgi_autotune(self.h, _ptr(o), int(reps), _stream_ptr(stream), C.byref(t)))
        return {k: int(getattr(t, k)) for k, _ in t._fields_}

    def init_probes(self, orientation, stream=None):
        """Probe classification (probesInit): states 0 (OFF), 1 or 8."""
        o = np.ascontiguousarray(orientation, np.float32).reshape(9)
        self._check(self.lib.ddgi_init_probes(self.h, _ptr(o), _stream_ptr(stream)))

    def update_scheduled(self, orientation, max_probes=0, stream=None):
        """Update of the probes the on-device schedule selects."""
        o = np.ascontiguousarray(orientation, np.float32).reshape(9)
        self._check(self.lib.ddgi_update_scheduled(self.h, _ptr(o), int(max_probes), _stream_ptr(stream)))

    def schedule(self, with_list=True, stream=None):
        """The last selection and the schedule state (synchronises)."""
        cnt, off, loop = C.c_uint32(), C.c_uint32(), C.c_uint32()
        P = self.grid.probe_count()
        lst = np.zeros(P, np.uint32) if with_list else None
        self._check(self.lib.ddgi_get_schedule(self.h, C.byref(cnt), C.byref(off), C.byref(loop), _ptr(lst),
                                               P if with_list else 0, _stream_ptr(stream)))
        out = {"count": int(cnt.value), "offset": int(off.value), "loop": int(loop.value)}
        if with_list:
            out["list"] = lst[:cnt.value].copy()
        return out

    def set_schedule(self, offset, loop, stream=None):
        self._check(self.lib.ddgi_set_schedule(self.h, int(offset), int(loop), _stream_ptr(stream)))

    def scene_info(self):
        """Tree sizes, depths, builder and GPU build time of the built scene."""
        info = SceneInfo()
        self._check(self.lib.ddgi_get_scene_info(self.h, C.byref(info)))
        return {"nodes": int(info.node_count), "tri_refs": int(info.tri_refs), "depth_blas": int(info.depth_blas),
                "depth_tlas": int(info.depth_tlas), "build_mode": int(info.build_mode),
                "tree_build_ms": float(info.tree_build_ms)}

    def read_trees(self, stream=None):
        """The built trees: nodes (N x 16 words of 32 bits) and triangles in
        leaf order (M x 12 words), as uint32 arrays."""
        info = self.scene_info()
        nodes = np.zeros((info["nodes"], 16), np.uint32)
        tris = np.zeros((info["tri_refs"], 12), np.uint32)
        self._check(self.lib.ddgi_read_trees(self.h, _ptr(nodes), nodes.shape[0], _ptr(tris), tris.shape[0],
                                             _stream_ptr(stream)))
        return nodes, tris

    def count_fetches(self, orientation, probe_list=None, stream=None):
        """Fetch counters of one trace + shade pass (see ddgi_count_fetches)."""
        o = np.ascontiguousarray(orientation, np.float32).reshape(9)
        pl = None if probe_list is None else np.ascontiguousarray(probe_list, np.uint32)
        out = np.zeros(11, np.uint64)
        self._check(self.lib.ddgi_count_fetches(self.h, _ptr(o), _ptr(pl), 0 if pl is None else len(pl), _ptr(out),
                                                _stream_ptr(stream)))
        keys = ("nodes", "tris", "instances", "rays", "shade_bytes", "shadow_nodes", "shadow_tris",
                "shadow_instances", "shadow_rays", "top_nodes", "shadow_top_nodes")
        return {k: int(v) for k, v in zip(keys, out)}

    def blend_records(self, orientation, records, probe_list=None, stream=None):
        """Blend + border copy of given ray records (n x R x 4 float32)."""
        o = np.ascontiguousarray(orientation, np.float32).reshape(9)
        pl = None if probe_list is None else np.ascontiguousarray(probe_list, np.uint32)
        rec = np.ascontiguousarray(records, np.float32)
        self._check(self.lib.ddgi_blend_records(self.h, _ptr(o), _ptr(pl), 0 if pl is None else len(pl), _ptr(rec),
                                                rec.size // 4, _stream_ptr(stream)))

    def set_materials(self, materials):
        m = np.ascontiguousarray(materials)
        self._check(self.lib.ddgi_set_materials(self.h, _ptr(m), len(m)))

    def forward_record(self, orientations, checkpoint_every=2, stream=None):
        """K recorded updates (orientations K x 9) for a later backward()."""
        o = np.ascontiguousarray(orientations, np.float32).reshape(-1, 9)
        self._check(self.lib.ddgi_forward_record(self.h, len(o), _ptr(o), int(checkpoint_every),
                                                 _stream_ptr(stream)))

    def backward(self, dL_dcolor, n_materials, stream=None):
        """Gradients (albedo [M, 3], sun [3], sky [3]) of a loss whose
        gradient with respect to the final colour atlas is dL_dcolor."""
        g = np.ascontiguousarray(dL_dcolor, np.float32)
        assert g.shape == self.atlas_shape(abi.ATLAS_COLOR)
        ga = np.zeros((n_materials, 3), np.float32)
        gs = np.zeros(3, np.float32)
        gk = np.zeros(3, np.float32)
        self._check(self.lib.ddgi_backward(self.h, _ptr(g), g.nbytes, _ptr(ga), _ptr(gs), _ptr(gk),
                                           _stream_ptr(stream)))
        return ga, gs, gk

    def synchronize(self, stream=None, timeout_ms=-1):
        self._check(self.lib.ddgi_synchronize(self.h, _stream_ptr(stream), int(timeout_ms)))

    # ---- readback ----------------------------------------------------------
    def atlas_shape(self, kind):
        w, h, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self._check(self.lib.ddgi_atlas_dims(self.h, kind, C.byref(w), C.byref(h), C.byref(c)))
        return h.value, w.value, c.value

    def get_atlas(self, kind, out=None, stream=None):
        shape = self.atlas_shape(kind)
        if out is None:
            out = np.empty(shape, np.float32)
        assert out.shape == shape and out.dtype == np.float32 and out.flags.c_contiguous
        self._check(self.lib.ddgi_get_atlas(self.h, kind, _ptr(out), out.nbytes, _stream_ptr(stream)))
        return out

    def get_atlas_raw(self, kind, out=None, stream=None):
        """The atlas in its storage format: float32 (FP32 context) or float16
        (BF16-blend context) texels, H x W x channels."""
        shape = self.atlas_shape(kind)
        dtype = np.float16 if self.grid.precision == abi.PRECISION_BF16 else np.float32
        if out is None:
            out = np.empty(shape, dtype)
        assert out.shape == shape and out.dtype == dtype and out.flags.c_contiguous
        self._check(self.lib.ddgi_get_atlas_raw(self.h, kind, _ptr(out), out.nbytes, _stream_ptr(stream)))
        return out

    def save_atlas(self, path, stream=None):
        """Checkpoint of the atlases (and accumulators, probe states) to a file."""
        self._check(self.lib.ddgi_atlas_save(self.h, os.fsencode(path), _stream_ptr(stream)))

    def load_atlas(self, path, stream=None):
        """Restores a checkpoint written by save_atlas for the same grid."""
        self._check(self.lib.ddgi_atlas_load(self.h, os.fsencode(path), _stream_ptr(stream)))

    def inject_fault(self, faults):
        """One-shot failure-detection test hooks (abi.FAULT_*)."""
        self._check(self.lib.ddgi_inject_fault(self.h, int(faults)))

    def set_atlas(self, kind, data, stream=None):
        data = np.ascontiguousarray(data, np.float32)
        assert data.shape == self.atlas_shape(kind)
        self._check(self.lib.ddgi_set_atlas(self.h, kind, _ptr(data), data.nbytes, _stream_ptr(stream)))

    def get_ray_records(self, count_probes, stream=None):
        R = self.grid.rays_per_probe
        out = np.empty((count_probes, R, 4), np.float32)
        self._check(self.lib.ddgi_get_ray_records(self.h, _ptr(out), count_probes * R, _stream_ptr(stream)))
        return out

    def get_hits(self, count_probes, stream=None):
        R = self.grid.rays_per_probe
        out = np.empty((count_probes, R), HIT_DTYPE)
        self._check(self.lib.ddgi_get_hits(self.h, _ptr(out), count_probes * R, _stream_ptr(stream)))
        return out

    def get_ray_directions(self):
        R = self.grid.rays_per_probe
        out = np.empty((R, 4), np.float32)
        self._check(self.lib.ddgi_get_ray_directions(self.h, _ptr(out), R))
        return out

    def get_probe_states(self, stream=None):
        n = self.grid.probe_count()
        out = np.empty(n, np.uint32)
        self._check(self.lib.ddgi_get_probe_states(self.h, _ptr(out), n, _stream_ptr(stream)))
        return out

    def set_probe_states(self, states, stream=None):
        s = np.ascontiguousarray(states, np.uint32)
        self._check(self.lib.ddgi_set_probe_states(self.h, _ptr(s), len(s), _stream_ptr(stream)))

    def atlas_device_ptr(self, kind):
        p = C.c_void_p()
        self._check(self.lib.ddgi_atlas_device_ptr(self.h, kind, C.byref(p)))
        return p.value

    def timings(self):
        t = Timings()
        self._check(self.lib.ddgi_get_timings(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in Timings._fields_}

    def trace_rays(self, origins, dirs, tmin, tmax, mask=0xFF, any_hit=False, stream=None):
        origins = np.ascontiguousarray(origins, np.float32)
        dirs = np.ascontiguousarray(dirs, np.float32)
        n = len(origins)
        hits = np.zeros(n, HIT_DTYPE)
        bary = np.zeros((n, 2), np.float32)
        self._check(self.lib.ddgi_trace_rays(self.h, _ptr(origins), _ptr(dirs), n, tmin, tmax, mask, int(any_hit),
                                             _ptr(hits), _ptr(bary), _stream_ptr(stream)))
        return hits, bary


class Batch:
    """Owns one ddgi_batch over a list of Contexts (which must outlive it)."""

    def __init__(self, contexts, stream=None):
        self.lib = load_library()
        self.contexts = list(contexts)
        arr = (C.c_void_p * len(self.contexts))(*[c.h.value for c in self.contexts])
        h = C.c_void_p()
        st = self.lib.ddgi_batch_create(arr, len(self.contexts), _stream_ptr(stream), C.byref(h))
        if st != 0:
            raise DDGIError(st, "ddgi_batch_create")
        self.h = h

    def _check(self, status):
        if status != 0:
            raise DDGIError(status, self.lib.ddgi_batch_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.ddgi_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def ray_count(self):
        return int(self.lib.ddgi_batch_ray_count(self.h))

    def tuning(self):
        t = BatchTuning()
        self._check(self.lib.ddgi_batch_get_tuning(self.h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw):
        t = BatchTuning()
        self._check(self.lib.ddgi_batch_get_tuning(self.h, C.byref(t)))
        for k, v in kw.items():
            setattr(t, k, int(v))
        self._check(self.lib.ddgi_batch_set_tuning(self.h, C.byref(t)))

    def use_graph(self, on=True):
        self._check(self.lib.ddgi_batch_use_graph(self.h, int(on)))

    def _orients(self, orientations):
        o = np.ascontiguousarray(orientations, np.float32).reshape(len(self.contexts), 9)
        return o

    def update(self, orientations, stream=None):
        o = self._orients(orientations)
        self._check(self.lib.ddgi_batch_update(self.h, _ptr(o), _stream_ptr(stream)))

    def synchronize(self, stream=None, timeout_ms=-1):
        self._check(self.lib.ddgi_batch_synchronize(self.h, _stream_ptr(stream), int(timeout_ms)))

    def completion_ms(self):
        out = np.zeros(len(self.contexts), np.float32)
        self._check(self.lib.ddgi_batch_completion_ms(self.h, _ptr(out), len(out)))
        return out

    def autotune(self, orientations, reps=3, stream=None):
        o = self._orients(orientations)
        t = BatchTuning()
        self._check(self.lib.ddgi_batch_autotune(self.h, _ptr(o), int(reps), _stream_ptr(stream), C.byref(t)))
        return t.as_dict()


class IrradianceProbes:
    """Drop-in mirror of VulkanExp's IrradianceProbes over the C ABI.

    The hysteresis ramp of the reference's update (TargetHysteresis,
    src/IrradianceProbes.cpp:462-476) runs in the library
    (ddgi_set_target_hysteresis): GridParameters.hysteresis here is the value
    updateUniforms() uploads; the ramp's current values are `hysteresis()`."""

    MaxRaysPerProbe = 1024

    def __init__(self):
        # GridInfo defaults (src/IrradianceProbes.hpp:49-60)
        self.GridParameters = abi.make_grid((0, 0, 0), (1, 1, 1), (32, 16, 32), 192, 8, 16, 0.0, 12.0, 0.3)
        self._target = 0.98
        self.ProbesPerUpdate = 0
        self.ctx = None
        self._shadow = 0.0

    @property
    def TargetHysteresis(self):
        return self._target

    @TargetHysteresis.setter
    def TargetHysteresis(self, value):
        self._target = float(value)
        if self.ctx:
            self.ctx.set_target_hysteresis(self._target)

    def init(self, extent_min, extent_max):
        self.GridParameters.extent_min[:] = [float(v) for v in extent_min]
        self.GridParameters.extent_max[:] = [float(v) for v in extent_max]
        if self.ctx:
            self.ctx.close()
        self.ctx = Context(self.GridParameters)
        self._shadow = self.GridParameters.hysteresis
        self.ctx.set_target_hysteresis(self._target)

    def setScene(self, scene, stream=None):
        self.ctx.build_scene(scene, stream)

    def setLightBuffer(self, light):
        self.ctx.set_light(light)

    def updateUniforms(self):
        """ddgi_set_grid.  Keeps the ramp's current value unless
        GridParameters.hysteresis was changed since it was last in step with
        the library (syncHysteresis reads it back)."""
        if np.float32(self.GridParameters.hysteresis) == np.float32(self._shadow):
            self.GridParameters.hysteresis = self.ctx.hysteresis()[1]
        self.ctx.set_grid(self.GridParameters)
        self._shadow = self.GridParameters.hysteresis

    def syncHysteresis(self, stream=None):
        """Reads the ramp's current value into GridParameters.hysteresis."""
        self.GridParameters.hysteresis = self._shadow = self.ctx.hysteresis(stream)[1]

    def getProbeCount(self):
        r = self.GridParameters.resolution
        return int(r[0]) * int(r[1]) * int(r[2])

    def initProbes(self, orientation, stream=None):
        """IrradianceProbes::initProbes (src/IrradianceProbes.cpp:357-394):
        classify the probes; the ramp's host-side value restarts from 0."""
        self.ctx.init_probes(orientation, stream)
        self.GridParameters.hysteresis = self._shadow = 0.0

    def hysteresis(self, stream=None):
        """(value the last update blended with, host-side value, probes
        counted since the last ramp step)."""
        return self.ctx.hysteresis(stream)

    def update(self, orientation, probe_list=None, stream=None):
        """IrradianceProbes::update (src/IrradianceProbes.cpp:426-594):
        `orientation` is the 3x3 ray-set rotation.  Without a probe list the
        probes are the ones selectProbesToUpdate picks (chosen on the device,
        at most ProbesPerUpdate, 0 = no cap); the hysteresis ramp steps on
        the device, with no readback."""
        if probe_list is not None:
            self.ctx.update(orientation, probe_list, stream)
        else:
            self.ctx.update_scheduled(orientation, self.ProbesPerUpdate, stream)

    def getIrradiance(self):
        return self.ctx.get_atlas(abi.ATLAS_COLOR)

    def getDepth(self):
        return self.ctx.get_atlas(abi.ATLAS_DEPTH)

    def destroy(self):
        if self.ctx:
            self.ctx.close()
            self.ctx = None

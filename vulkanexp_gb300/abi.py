"""ctypes / numpy mirrors of the structs declared in include/ddgi.h.

The numpy dtypes give the exact byte layout of the C structs so that scene
arrays can be passed to the library (and to the CPU checker) without copies.
"""
import ctypes as C

import numpy as np

VERTEX_DTYPE = np.dtype(
    [("pos", "<f4", 3), ("color", "<f4", 3), ("normal", "<f4", 3), ("tangent", "<f4", 4), ("uv", "<f4", 2), ("padding", "<u4")]
)
MATERIAL_DTYPE = np.dtype(
    [
        ("metallic", "<f4"),
        ("roughness", "<f4"),
        ("base_color", "<f4", 3),
        ("emissive", "<f4", 3),
        ("albedo_texture", "<u4"),
        ("normal_texture", "<u4"),
        ("metallic_roughness_texture", "<u4"),
        ("emissive_texture", "<u4"),
    ]
)
OFFSET_DTYPE = np.dtype([("material_index", "<u4"), ("vertex_offset", "<u4"), ("index_offset", "<u4")])
MESH_DTYPE = np.dtype([("vertex_offset", "<u4"), ("vertex_count", "<u4"), ("index_offset", "<u4"), ("index_count", "<u4")])
INSTANCE_DTYPE = np.dtype(
    [("transform", "<f4", 12), ("custom_index", "<u4"), ("mask", "<u4"), ("mesh_index", "<u4"), ("padding", "<u4")]
)
HIT_DTYPE = np.dtype([("instance", "<u4"), ("primitive", "<u4"), ("t", "<f4"), ("backface", "<u4")])

assert VERTEX_DTYPE.itemsize == 64
assert MATERIAL_DTYPE.itemsize == 48
assert INSTANCE_DTYPE.itemsize == 64

NO_TEXTURE = 0xFFFFFFFF
MISS = 0xFFFFFFFF

PRECISION_FP32 = 0
PRECISION_BF16 = 1
PRECISION_REFERENCE_FORMAT = 2  # FP32 blend, texels rounded to R11G11B10F / RG16F on store
SKY_CONSTANT = 0
SKY_ATMOSPHERE = 1
ATLAS_COLOR = 0
ATLAS_DEPTH = 1

STATUS_NAMES = {
    0: "DDGI_OK",
    1: "DDGI_ERR_INVALID_ARGUMENT",
    2: "DDGI_ERR_CUDA",
    3: "DDGI_ERR_OUT_OF_MEMORY",
    4: "DDGI_ERR_NO_SCENE",
    5: "DDGI_ERR_TIMEOUT",
    6: "DDGI_ERR_DEVICE",
    7: "DDGI_ERR_UNSUPPORTED",
    8: "DDGI_ERR_IO",
}
ERR_DEVICE = 6
ERR_IO = 8
FAULT_STALL_TENSOR_WAIT = 1


class GridDesc(C.Structure):
    _fields_ = [
        ("extent_min", C.c_float * 3),
        ("depth_sharpness", C.c_float),
        ("extent_max", C.c_float * 3),
        ("hysteresis", C.c_float),
        ("resolution", C.c_int32 * 3),
        ("rays_per_probe", C.c_uint32),
        ("color_res", C.c_uint32),
        ("depth_res", C.c_uint32),
        ("shadow_bias", C.c_float),
        ("precision", C.c_uint32),
    ]

    def probe_count(self):
        r = self.resolution
        return int(r[0]) * int(r[1]) * int(r[2])

    def copy(self):
        g = GridDesc()
        C.pointer(g)[0] = self
        return g

    def atlas_shape(self, kind):
        res = self.color_res if kind == ATLAS_COLOR else self.depth_res
        w = res * self.resolution[0] * self.resolution[1]
        h = res * self.resolution[2]
        return int(h), int(w), (4 if kind == ATLAS_COLOR else 2)


assert C.sizeof(GridDesc) == 64


class Light(C.Structure):
    _fields_ = [("direction", C.c_float * 4), ("color", C.c_float * 4), ("sky", C.c_float * 4)]


class SceneDesc(C.Structure):
    _fields_ = [
        ("vertices", C.c_void_p),
        ("vertex_count", C.c_uint32),
        ("indices", C.c_void_p),
        ("index_count", C.c_uint32),
        ("meshes", C.c_void_p),
        ("mesh_count", C.c_uint32),
        ("instances", C.c_void_p),
        ("instance_count", C.c_uint32),
        ("offsets", C.c_void_p),
        ("offset_count", C.c_uint32),
        ("materials", C.c_void_p),
        ("material_count", C.c_uint32),
    ]


class Timings(C.Structure):
    _fields_ = [("total_ms", C.c_float), ("trace_ms", C.c_float), ("blend_ms", C.c_float), ("border_ms", C.c_float),
                ("copy_ms", C.c_float), ("primary_ms", C.c_float)]


class SceneInfo(C.Structure):
    """ddgi_scene_info: sizes of the built trees."""
    _fields_ = [("node_count", C.c_uint64), ("tri_refs", C.c_uint64), ("depth_blas", C.c_uint32),
                ("depth_tlas", C.c_uint32), ("build_mode", C.c_uint32), ("tree_build_ms", C.c_float)]


class BatchTuning(C.Structure):
    """ddgi_batch_tuning: launch parameters of a batch."""
    _fields_ = [("trace_ctas_per_sm", C.c_uint32), ("refill_lanes", C.c_uint32), ("smem_stack", C.c_uint32),
                ("blend_threads", C.c_uint32), ("rays_per_warp", C.c_uint32), ("node_width", C.c_uint32),
                ("straggler_lanes", C.c_uint32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class GBuffer(C.Structure):
    """ddgi_gbuffer: device pointers of a G-buffer (width x height pixels)."""
    _fields_ = [("position_depth", C.c_void_p), ("normal_metalness", C.c_void_p), ("albedo_roughness", C.c_void_p),
                ("emissive", C.c_void_p), ("direct_light", C.c_void_p), ("reflection", C.c_void_p),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class TraceTuning(C.Structure):
    """ddgi_trace_tuning: launch parameters of a context's traversals."""
    _fields_ = [("rays_per_warp", C.c_uint32), ("refill_lanes", C.c_uint32), ("smem_stack", C.c_uint32),
                ("ctas_per_sm", C.c_uint32), ("node_width", C.c_uint32), ("straggler_lanes", C.c_uint32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


PIPELINE_FUSED = 0
PIPELINE_WAVEFRONT = 1


def make_grid(extent_min, extent_max, resolution, rays, color_res=8, depth_res=16, hysteresis=0.97,
              depth_sharpness=50.0, shadow_bias=0.05, precision=PRECISION_FP32):
    g = GridDesc()
    g.extent_min[:] = [float(v) for v in extent_min]
    g.extent_max[:] = [float(v) for v in extent_max]
    g.resolution[:] = [int(v) for v in resolution]
    g.rays_per_probe = int(rays)
    g.color_res = int(color_res)
    g.depth_res = int(depth_res)
    g.hysteresis = float(hysteresis)
    g.depth_sharpness = float(depth_sharpness)
    g.shadow_bias = float(shadow_bias)
    g.precision = int(precision)
    return g


def make_light(direction, color, sky):
    L = Light()
    L.direction[:] = [float(direction[0]), float(direction[1]), float(direction[2]), 1.0]
    L.color[:] = [float(color[0]), float(color[1]), float(color[2]), 1.0]
    L.sky[:] = [float(sky[0]), float(sky[1]), float(sky[2]), 1.0]
    return L

"""ctypes binding of oracle/_ref/libref_glsl.so, the reference's own shader
code compiled as C++ (see oracle/build_ref_glsl.py): its helper functions,
its probe trace (ray generation, closest hit, miss and shadow-miss stages)
and its probe-update compute passes.  Test infrastructure: used by the
reference-shader tests and by tests/golden/make_reference_vectors.py to make
the committed fixtures; the library exists only where the reference's
sources were present to build it.
"""
import ctypes as C
import os

import numpy as np

from vulkanexp_gb300.abi import GridDesc

from .build_ref_glsl import LIB

_lib = None


def available():
    return os.path.exists(LIB)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB)
        L.ref_spherical_fibonacci.argtypes = [C.c_float, C.c_float, C.c_void_p]
        L.ref_oct_encode.argtypes = [C.c_void_p, C.c_void_p]
        L.ref_oct_decode.argtypes = [C.c_float, C.c_float, C.c_void_p]
        L.ref_sphere_to_oct_uv.argtypes = [C.c_void_p, C.c_void_p]
        L.ref_probe_world_position.argtypes = [C.POINTER(GridDesc), C.c_uint32, C.c_void_p]
        L.ref_sample_probes.argtypes = [C.POINTER(GridDesc)] + [C.c_void_p] * 7
        L.ref_pbr.argtypes = [C.c_void_p] * 5 + [C.c_float, C.c_float, C.c_void_p]
        L.ref_sky.argtypes = [C.c_void_p] * 4 + [C.c_float, C.c_int, C.c_void_p]
        L.ref_probes_update.argtypes = [C.POINTER(GridDesc), C.c_void_p, C.c_uint32] + [C.c_void_p] * 5
        L.ref_init_probes.argtypes = [C.POINTER(GridDesc), C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_int]
        L.ref_final_gather.argtypes = ([C.POINTER(GridDesc)] + [C.c_void_p] * 5 + [C.c_int, C.c_int] +
                                       [C.c_void_p] * 9 + [C.c_int])
        L.ref_select_sequence.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32] + [C.c_void_p] * 4
        L.ref_gen_basis.argtypes = [C.c_void_p] * 3
        L.ref_ramp_sequence.argtypes = [C.c_float, C.c_float, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                        C.c_void_p]
        L.ref_trace_probes.argtypes = ([C.POINTER(GridDesc)] + [C.c_void_p] * 7 + [C.c_uint32] + [C.c_void_p] * 4 +
                                       [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p] + [C.c_void_p] * 3 + [C.c_int])
        _lib = L
    return _lib


def f32(a):
    return np.ascontiguousarray(a, np.float32)


def spherical_fibonacci(i, n):
    out = np.zeros(3, np.float32)
    lib().ref_spherical_fibonacci(float(i), float(n), _ptr(out))
    return out


def oct_encode(v):
    out = np.zeros(2, np.float32)
    lib().ref_oct_encode(_ptr(f32(v)), _ptr(out))
    return out


def oct_decode(x, y):
    out = np.zeros(3, np.float32)
    lib().ref_oct_decode(float(x), float(y), _ptr(out))
    return out


def sphere_to_oct_uv(d):
    out = np.zeros(2, np.float32)
    lib().ref_sphere_to_oct_uv(_ptr(f32(d)), _ptr(out))
    return out


def probe_world_position(grid, index):
    out = np.zeros(3, np.float32)
    lib().ref_probe_world_position(C.byref(grid), int(index), _ptr(out))
    return out


def sample_probes(grid, states, color, depth, pos, nrm, view):
    """sampleProbes (irradiance.glsl) on float atlases: colour H x W x 4,
    depth H x W x 2."""
    out = np.zeros(3, np.float32)
    lib().ref_sample_probes(C.byref(grid), _ptr(np.ascontiguousarray(states, np.uint32)), _ptr(f32(color)),
                            _ptr(f32(depth)), _ptr(f32(pos)), _ptr(f32(nrm)), _ptr(f32(view)), _ptr(out))
    return out


def pbr(n, v, light_color, light_dir, albedo4, metal, rough):
    out = np.zeros(4, np.float32)
    lib().ref_pbr(*[_ptr(f32(x)) for x in (n, v, light_color, light_dir, albedo4)], float(metal), float(rough),
                  _ptr(out))
    return out


def sky(origin, direction, sun_pos, sun_color, brightness, show_sun=True):
    out = np.zeros(3, np.float32)
    lib().ref_sky(*[_ptr(f32(x)) for x in (origin, direction, sun_pos, sun_color)], float(brightness),
                  1 if show_sun else 0, _ptr(out))
    return out


def probes_update(grid, probe_list, rays, dirs, states, color, depth):
    """The reference's irradiance pass, depth pass and border copy of the
    listed probes, in place on `color` (H x W x 4 float32), `depth`
    (H x W x 2) and `states`; rays: n x R x 4 records, dirs: R x 4 (the
    ray-direction image)."""
    lst = np.ascontiguousarray(probe_list, np.uint32)
    assert color.dtype == np.float32 and depth.dtype == np.float32 and states.dtype == np.uint32
    lib().ref_probes_update(C.byref(grid), _ptr(lst), len(lst), _ptr(f32(rays)), _ptr(f32(dirs)), _ptr(states),
                            _ptr(color), _ptr(depth))


def trace_probes(oracle, scene, grid, light, orientation, probe_list, states, color, depth, dirs=None, threads=16):
    """The reference's probe trace of the listed probes (traceProbes.rgen with
    its closest-hit and miss stages), each traceRayEXT's hit found by the
    oracle's traversal.  Returns (rays n x R x 4, trace arguments n x R x 8,
    ray-direction image R x 4); `dirs` gives the image's prior content."""
    from oracle.oracle import Oracle

    lst = np.ascontiguousarray(probe_list, np.uint32)
    n, R = len(lst), grid.rays_per_probe
    rays = np.zeros((n, R, 4), np.float32)
    rec = np.zeros((n, R, 8), np.float32)
    dimg = np.zeros((R, 4), np.float32) if dirs is None else f32(dirs).copy()
    ld = f32(light.direction[:])
    lc = f32(light.color[:])
    trace_fn = C.cast(Oracle.lib().oracle_trace, C.c_void_p)
    lib().ref_trace_probes(C.byref(grid), _ptr(ld), _ptr(lc), _ptr(np.ascontiguousarray(scene.vertices)),
                           _ptr(np.ascontiguousarray(scene.indices, np.uint32)),
                           _ptr(np.ascontiguousarray(scene.offsets)), _ptr(np.ascontiguousarray(scene.materials)),
                           _ptr(np.ascontiguousarray(scene.instances)), len(scene.instances),
                           _ptr(states), _ptr(f32(color)), _ptr(f32(depth)),
                           _ptr(f32(np.asarray(orientation).reshape(9))), _ptr(lst), n, trace_fn,
                           C.c_void_p(oracle._h), _ptr(rays), _ptr(rec), _ptr(dimg), int(threads))
    return rays, rec, dimg


def init_probes(oracle, scene, grid, orientation, threads=16):
    """The reference's probe classification (probesInit.rgen with its miss
    and back-face closest-hit stages), hits found by the oracle's traversal:
    one state per probe (0 off, 1 near geometry, 8)."""
    from oracle.oracle import Oracle

    states = np.zeros(grid.probe_count(), np.uint32)
    trace_fn = C.cast(Oracle.lib().oracle_trace, C.c_void_p)
    lib().ref_init_probes(C.byref(grid), _ptr(np.ascontiguousarray(scene.instances)), len(scene.instances),
                          _ptr(f32(np.asarray(orientation).reshape(9))), trace_fn, C.c_void_p(oracle._h),
                          _ptr(states), int(threads))
    return states


def final_gather(grid, light, states, color, depth, gbuffer, view, proj, threads=16):
    """The reference's FinalGather.frag over an H x W G-buffer (dict of
    float32 arrays position_depth, normal_metalness, albedo_roughness,
    emissive, direct_light (.r used), reflection: H x W x 4); view, proj:
    4x4 row-major matrices (world to view, view to clip).  Returns
    H x W x 4."""
    h, w = gbuffer["position_depth"].shape[:2]
    ins = [f32(gbuffer[k]) for k in ("position_depth", "normal_metalness", "albedo_roughness", "emissive",
                                      "direct_light", "reflection")]
    out = np.zeros((h, w, 4), np.float32)
    lib().ref_final_gather(C.byref(grid), _ptr(f32(light.direction[:])), _ptr(f32(light.color[:])),
                           _ptr(np.ascontiguousarray(states, np.uint32)), _ptr(f32(color)), _ptr(f32(depth)), w, h,
                           *[_ptr(a) for a in ins], _ptr(f32(np.asarray(view).T)), _ptr(f32(np.asarray(proj).T)),
                           _ptr(out), int(threads))
    return out


def select_sequence(states, caps):
    """K successive calls of the reference's selectProbesToUpdate (its own
    source) on one object: states K x n, caps K (0 = no cap).  Returns the K
    lists and the offsets each call leaves.  Its loop index is a
    function-local static: a process's calls form one sequence."""
    states = np.ascontiguousarray(states, np.uint32)
    K, n = states.shape
    caps = np.ascontiguousarray(caps, np.uint32)
    lists = np.zeros((K, n), np.uint32)
    counts = np.zeros(K, np.uint32)
    offsets = np.zeros(K, np.uint32)
    lib().ref_select_sequence(_ptr(states), n, K, _ptr(caps), _ptr(lists), _ptr(counts), _ptr(offsets))
    return [lists[k, :counts[k]].copy() for k in range(K)], offsets


def gen_basis(n):
    """The reference's genBasis (its source over its vendored GLM): b1, b2."""
    b1, b2 = np.zeros(3, np.float32), np.zeros(3, np.float32)
    lib().ref_gen_basis(_ptr(f32(n)), _ptr(b1), _ptr(b2))
    return b1, b2


def ramp_sequence(h0, target, P, counts):
    """The reference's hysteresis ramp (its own block of update()) over
    updates of counts[k] probes: (uploaded value per update,
    GridParameters.hysteresis after it).  Its counter is a function-local
    static: a process's calls form one sequence."""
    counts = np.ascontiguousarray(counts, np.uint32)
    u = np.zeros(len(counts), np.float32)
    p = np.zeros(len(counts), np.float32)
    lib().ref_ramp_sequence(float(h0), float(target), int(P), _ptr(counts), len(counts), _ptr(u), _ptr(p))
    return u, p

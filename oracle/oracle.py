"""ctypes front end of the CPU checker (oracle/ddgi_oracle.cpp).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from vulkanexp_gb300.abi import HIT_DTYPE, GridDesc, Light, SceneDesc

REC_DTYPE = np.dtype([("inst", "<u4"), ("prim", "<u4"), ("t", "<f4"), ("b1", "<f4"), ("b2", "<f4"),
                      ("flags", "<u4")])

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")


def oracle_lib_path():
    return os.path.join(BUILD_DIR, "libddgi_oracle.so")


def build_oracle(force=False):
    """Compiles the checker with g++ (-ffp-contract=off: every operation
    rounded separately, as the hit-ID contract requires)."""
    out = oracle_lib_path()
    src = os.path.join(HERE, "ddgi_oracle.cpp")
    deps = [src, os.path.join(ROOT, "include", "ddgi.h"), os.path.join(ROOT, "include", "ddgi_exact.h")]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = out + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
           "-o", tmp, src]
    subprocess.check_call(cmd)
    os.replace(tmp, out)
    return out


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


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


class Oracle:
    """The CPU restatement of the probe update over one scene."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            # DDGI_ORACLE_LIB: a differently built checker (the sanitizer test)
            lib = C.CDLL(os.environ.get("DDGI_ORACLE_LIB") or build_oracle())
            lib.oracle_scene_create.restype = C.c_void_p
            lib.oracle_scene_create.argtypes = [C.POINTER(SceneDesc), C.c_int]
            lib.oracle_scene_destroy.argtypes = [C.c_void_p]
            lib.oracle_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_float, C.c_float,
                                         C.c_uint32, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
            lib.oracle_update.argtypes = [C.c_void_p, C.POINTER(GridDesc), C.POINTER(Light), C.c_void_p, C.c_void_p,
                                          C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                          C.c_void_p, C.c_int]
            lib.oracle_blend.argtypes = [C.POINTER(GridDesc), C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
            lib.oracle_blend64.argtypes = lib.oracle_blend.argtypes
            lib.oracle_rec_hit_bytes.restype = C.c_uint32
            lib.oracle_record.argtypes = [C.c_void_p, C.POINTER(GridDesc), C.POINTER(Light), C.c_void_p, C.c_uint32,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
            lib.oracle_replay.argtypes = [C.c_void_p, C.POINTER(GridDesc), C.POINTER(Light), C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_int]
            assert lib.oracle_rec_hit_bytes() == REC_DTYPE.itemsize
            lib.oracle_border_table.restype = C.c_uint32
            lib.oracle_border_table.argtypes = [C.c_int, C.c_void_p]
            lib.oracle_oct_decode.argtypes = [C.c_float, C.c_float, C.c_void_p]
            lib.oracle_sphere_to_oct_uv.argtypes = [C.c_void_p, C.c_void_p]
            lib.oracle_shade_rays.argtypes = [C.c_void_p, C.POINTER(GridDesc), C.POINTER(Light)] + [C.c_void_p] * 4 + [
                C.c_uint32, C.c_void_p, C.c_int]
            lib.oracle_probe_world_position.argtypes = [C.POINTER(GridDesc), C.c_uint32, C.c_void_p]
            lib.oracle_sky.argtypes = [C.c_void_p] * 4 + [C.c_float, C.c_void_p]
            lib.oracle_direction_table.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
            lib.oracle_round_store.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_uint32]
            lib.oracle_set_sky_mode.argtypes = [C.c_int]
            lib.oracle_texel_scale.restype = C.c_float
            lib.oracle_texel_scale.argtypes = [C.c_uint32]
            lib.oracle_pbr.argtypes = [C.c_void_p] * 5 + [C.c_float, C.c_float, C.c_void_p]
            lib.oracle_sample_probes.argtypes = [C.POINTER(GridDesc)] + [C.c_void_p] * 7
            lib.oracle_init_probes.argtypes = [C.c_void_p, C.POINTER(GridDesc), C.c_void_p, C.c_void_p, C.c_int]
            lib.oracle_final_gather.argtypes = [C.POINTER(GridDesc), C.POINTER(Light), C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_uint32] + [C.c_void_p] * 8 + [C.c_int]
            cls._lib = lib
        return cls._lib

    def __init__(self, scene, threads=None):
        self.threads = int(threads or os.cpu_count() or 1)
        self.scene = scene
        self._desc = scene_desc(scene)
        self._h = self.lib().oracle_scene_create(C.byref(self._desc), self.threads)

    def close(self):
        if self._h:
            self.lib().oracle_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- queries -------------------------------------------------------------
    def init_probes(self, grid, orientation):
        """Probe states from the probesInit classification (0 OFF, 1, 8)."""
        o = np.ascontiguousarray(orientation, np.float32).reshape(9)
        states = np.zeros(grid.probe_count(), np.uint32)
        self.lib().oracle_init_probes(self._h, C.byref(grid), _ptr(o), _ptr(states), self.threads)
        return states

    def trace(self, origins, dirs, tmin, tmax, mask=0xFF, any_hit=False):
        origins = np.ascontiguousarray(origins, np.float32)
        dirs = np.ascontiguousarray(dirs, np.float32)
        n = len(origins)
        hits = np.zeros(n, HIT_DTYPE)
        bary = np.zeros((n, 2), np.float32)
        self.lib().oracle_trace(self._h, _ptr(origins), _ptr(dirs), n, tmin, tmax, mask, int(any_hit), _ptr(hits),
                                _ptr(bary), self.threads)
        return hits, bary

    def update(self, grid, light, orientation, color, depth, states, probe_list=None, fp64=False, want_rays=False,
               want_hits=False):
        """One update in place on `color` (H x W x 4) and `depth` (H x W x 2)
        (float32, or float64 when fp64) and `states` (uint32 per probe).
        Returns (ray_records, hits) when requested."""
        dt = np.float64 if fp64 else np.float32
        assert color.dtype == dt and depth.dtype == dt and states.dtype == np.uint32
        assert color.flags.c_contiguous and depth.flags.c_contiguous and states.flags.c_contiguous
        orient = np.ascontiguousarray(orientation, np.float32).reshape(9)
        plist = None if probe_list is None else np.ascontiguousarray(probe_list, np.uint32)
        n = grid.probe_count() if plist is None else len(plist)
        R = grid.rays_per_probe
        rays = np.zeros((n, R, 4), np.float32) if want_rays else None
        hits = np.zeros((n, R), HIT_DTYPE) if want_hits else None
        self.lib().oracle_update(self._h, C.byref(grid), C.byref(light), _ptr(orient), _ptr(plist),
                                 0 if plist is None else len(plist), _ptr(states), _ptr(color), _ptr(depth), int(fp64),
                                 _ptr(rays), _ptr(hits), self.threads)
        return rays, hits

    # -- differentiation support (FP64, all probes, hit set recorded once) -----
    def shade_rays(self, grid, light, states, color, depth, rays):
        """Trace + shade (float) of given rays (n x 8: origin, direction,
        tmin, tmax) against the previous atlas: n x 4 records (radiance,
        hit distance) as the probe update writes them."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        out = np.zeros((len(rays), 4), np.float32)
        self.lib().oracle_shade_rays(self._h, C.byref(grid), C.byref(light), _ptr(states), _ptr(color), _ptr(depth),
                                     _ptr(rays), len(rays), _ptr(out), self.threads)
        return out

    def record(self, grid, light, orientations, states, color, depth):
        """K FP64 updates (orientations K x 9) in place on color/depth
        (float64) and states; returns the recording: hits (K, P, R) and the
        depth atlas after every update."""
        o = np.ascontiguousarray(orientations, np.float32).reshape(-1, 9)
        K, P, R = len(o), grid.probe_count(), grid.rays_per_probe
        assert color.dtype == np.float64 and depth.dtype == np.float64
        rec = np.zeros((K, P, R), REC_DTYPE)
        snap = np.zeros((K,) + depth.shape, np.float64)
        self.lib().oracle_record(self._h, C.byref(grid), C.byref(light), _ptr(o), K, _ptr(states), _ptr(color),
                                 _ptr(depth), _ptr(rec), _ptr(snap), self.threads)
        return rec, snap

    def replay(self, grid, light, orientations, states, color, depth, recording, albedo=None, sun=None, sky=None):
        """K FP64 updates shading the recorded hits with the given parameters
        (albedo: material_count x 3; sun, sky: 3 each; None = the scene's)."""
        rec, snap = recording
        o = np.ascontiguousarray(orientations, np.float32).reshape(-1, 9)
        K = len(o)
        assert rec.shape[0] == K and snap.shape[0] == K
        alb = None if albedo is None else np.ascontiguousarray(albedo, np.float64)
        sun = np.ascontiguousarray(light.color[:3] if sun is None else sun, np.float64)
        sky = np.ascontiguousarray(light.sky[:3] if sky is None else sky, np.float64)
        self.lib().oracle_replay(self._h, C.byref(grid), C.byref(light), _ptr(alb), _ptr(sun), _ptr(sky), _ptr(o), K,
                                 _ptr(states), _ptr(color), _ptr(depth), _ptr(np.ascontiguousarray(rec)), _ptr(snap),
                                 self.threads)

    # -- scene-independent entry points ---------------------------------------
    @classmethod
    def blend(cls, grid, orientation, rays, color, depth, states, probe_list=None, threads=None):
        """Blend + border copy of given float ray records into `color`/`depth`
        (float32 atlases, or float64 for the FP64 form)."""
        orient = np.ascontiguousarray(orientation, np.float32).reshape(9)
        plist = None if probe_list is None else np.ascontiguousarray(probe_list, np.uint32)
        rays = np.ascontiguousarray(rays, np.float32)
        fn = cls.lib().oracle_blend64 if color.dtype == np.float64 else cls.lib().oracle_blend
        fn(C.byref(grid), _ptr(orient), _ptr(plist), 0 if plist is None else len(plist), _ptr(rays), _ptr(states),
           _ptr(color), _ptr(depth), int(threads or os.cpu_count()))

    @classmethod
    def final_gather(cls, grid, light, states, color, depth, gbuffer, origin, threads=None):
        """FinalGather.frag per pixel.  gbuffer: dict of float32 arrays
        position_depth, normal_metalness, albedo_roughness, emissive (N x 4),
        direct_light (N), reflection (N x 4 or None).  Returns N x 4."""
        f = lambda a: None if a is None else np.ascontiguousarray(a, np.float32)
        pd = f(gbuffer["position_depth"])
        n = len(pd)
        out = np.zeros((n, 4), np.float32)
        o = np.ascontiguousarray(origin, np.float32)
        keep = [f(gbuffer[k]) for k in ("normal_metalness", "albedo_roughness", "emissive", "direct_light")]
        refl = f(gbuffer.get("reflection"))
        cls.lib().oracle_final_gather(C.byref(grid), C.byref(light), _ptr(np.ascontiguousarray(states, np.uint32)),
                                      _ptr(np.ascontiguousarray(color, np.float32)),
                                      _ptr(np.ascontiguousarray(depth, np.float32)), n, _ptr(pd),
                                      *[_ptr(k) for k in keep], _ptr(refl), _ptr(o), _ptr(out),
                                      int(threads or os.cpu_count() or 1))
        return out

    @classmethod
    def border_table(cls, n):
        count = cls.lib().oracle_border_table(n, None)
        out = np.zeros((count, 4), np.int32)
        cls.lib().oracle_border_table(n, _ptr(out))
        return out

    @classmethod
    def oct_decode(cls, x, y):
        out = np.zeros(3, np.float32)
        cls.lib().oracle_oct_decode(x, y, _ptr(out))
        return out

    @classmethod
    def sphere_to_oct_uv(cls, d):
        d = np.ascontiguousarray(d, np.float32)
        out = np.zeros(2, np.float32)
        cls.lib().oracle_sphere_to_oct_uv(_ptr(d), _ptr(out))
        return out

    @classmethod
    def probe_world_position(cls, grid, index):
        out = np.zeros(3, np.float32)
        cls.lib().oracle_probe_world_position(C.byref(grid), index, _ptr(out))
        return out

    @classmethod
    def sky(cls, origin, direction, sun_pos, sun_color, brightness):
        """The atmospheric sky radiance (float) seen along `direction`."""
        a = [np.ascontiguousarray(x, np.float32) for x in (origin, direction, sun_pos, sun_color)]
        out = np.zeros(3, np.float32)
        cls.lib().oracle_sky(*[_ptr(x) for x in a], brightness, _ptr(out))
        return out

    @classmethod
    def direction_table(cls, orientation, n):
        o = np.ascontiguousarray(orientation, np.float32).reshape(9)
        out = np.zeros((n, 4), np.float32)
        cls.lib().oracle_direction_table(_ptr(o), n, _ptr(out))
        return out

    @classmethod
    def set_sky_mode(cls, mode):
        """Miss radiance of later calls (process-wide): 0 the light's
        constant sky radiance, 1 the atmospheric sky of sky.glsl."""
        cls.lib().oracle_set_sky_mode(int(mode))

    @classmethod
    def round_store(cls, kind, values):
        """Reference-format storage rounding (0: 11-bit, 1: 10-bit unsigned
        float, 2: half) of float32 values."""
        v = np.ascontiguousarray(values, np.float32)
        out = np.empty_like(v)
        cls.lib().oracle_round_store(int(kind), _ptr(v), _ptr(out), v.size)
        return out

    @classmethod
    def texel_scale(cls, n):
        return cls.lib().oracle_texel_scale(n)

    @classmethod
    def pbr(cls, n, v, light_color, light_dir, albedo, metal, rough):
        a = [np.ascontiguousarray(x, np.float32) for x in (n, v, light_color, light_dir, albedo)]
        out = np.zeros(3, np.float32)
        cls.lib().oracle_pbr(*[_ptr(x) for x in a], metal, rough, _ptr(out))
        return out

    @classmethod
    def sample_probes(cls, grid, states, color, depth, pos, nrm, view):
        a = [np.ascontiguousarray(x, np.float32) for x in (pos, nrm, view)]
        out = np.zeros(3, np.float32)
        cls.lib().oracle_sample_probes(C.byref(grid), _ptr(states), _ptr(color), _ptr(depth), *[_ptr(x) for x in a],
                                       _ptr(out))
        return out


def zero_atlas(grid, fp64=False):
    dt = np.float64 if fp64 else np.float32
    ch, cw, _ = grid.atlas_shape(0)
    dh, dw, _ = grid.atlas_shape(1)
    return np.zeros((ch, cw, 4), dt), np.zeros((dh, dw, 2), dt)


def select_probes(states, offset, loop, max_probes=0):
    """IrradianceProbes::selectProbesToUpdate (src/IrradianceProbes.cpp:396-424)
    restated as the reference's host loop: visit probes cyclically from
    `offset`; probe idx is picked when its state s != 0 and
    (idx + loop) % s == 0; `loop` (the reference's static s_LoopIndex) grows
    by one at every wrap past the last probe; with max_probes > 0 the visit
    stops once that many are picked.  Returns (picked, next offset, next
    loop)."""
    n = len(states)
    picked = []
    idx, checked = offset, 0
    while checked < n and (max_probes == 0 or len(picked) < max_probes):
        s = int(states[idx])
        if s != 0 and (idx + loop) % s == 0:
            picked.append(idx)
        idx += 1
        if idx >= n:
            idx = 0
            loop += 1
        checked += 1
    return np.array(picked, np.uint32), idx, loop

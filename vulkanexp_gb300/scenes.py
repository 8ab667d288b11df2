"""Seeded synthetic scenes and probe grids for the DDGI update workloads.

The reference ships no usable scene for this path (its sample scenes are not
in the source tree), so every workload is generated here from a seed with
numpy's PCG64 generator.  The arrays use the exact layout of the C structs in
include/ddgi.h, so the same arrays feed the CUDA library and the CPU checker.

Conventions the generators follow:
  * triangles are counter-clockwise around their outward geometric normal,
    N = (v1 - v0) x (v2 - v0); a ray whose direction has dot(D, N) < 0 hits a
    front face.  Boxes face outward and the room faces inward, so that the
    backface rule of src/shaders/closesthit.glsl:137-141 separates "inside a
    wall" from visible geometry.
  * per-vertex normals are the flat face normals (boxes, room) or smooth
    finite-difference normals (terrain).
  * materials are metallic 0, roughness 1, emissive 0 with a random albedo
    (Material::Properties defaults to metallic 1, which would zero diffuse).
  * the light direction points TOWARDS the sun (src/Light.hpp:7), so a sun
    travelling along normalize(0.3, -1, 0.2) is passed as its negation.
"""
from dataclasses import dataclass, field

import numpy as np

from .abi import (INSTANCE_DTYPE, MATERIAL_DTYPE, MESH_DTYPE, NO_TEXTURE, OFFSET_DTYPE, PRECISION_FP32,
                  VERTEX_DTYPE, make_grid, make_light)

SUN_TRAVEL = np.array([0.3, -1.0, 0.2])
SUN_TOWARDS = -SUN_TRAVEL / np.linalg.norm(SUN_TRAVEL)
SUN_RADIANCE = (3.0, 3.0, 3.0)
SKY_RADIANCE = (0.4, 0.5, 0.7)


@dataclass
class Scene:
    vertices: np.ndarray
    indices: np.ndarray
    meshes: np.ndarray
    instances: np.ndarray
    offsets: np.ndarray
    materials: np.ndarray
    bounds: tuple = field(default=None)

    @property
    def triangle_count(self):
        """Triangles in the scene, counting each instance of a mesh."""
        per_mesh = self.meshes["index_count"] // 3
        return int(per_mesh[self.instances["mesh_index"]].sum())

    @property
    def unique_triangle_count(self):
        return int(self.indices.size // 3)


@dataclass
class Workload:
    name: str
    scene: Scene
    grid: object  # abi.GridDesc
    light: object  # abi.Light
    updates: int
    seed: int

    def orientation(self, k):
        """Row-major 3x3 ray-set rotation of update k."""
        return random_orientation(self.seed, k)


# ---------------------------------------------------------------------------
# geometry helpers
# ---------------------------------------------------------------------------
def box_geometry(lo, hi, inward=False):
    """24 vertices (4 per face, flat normals) and 12 triangles of an
    axis-aligned box."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    c = 0.5 * (lo + hi)
    h = 0.5 * (hi - lo)
    pos, nrm, tris = [], [], []
    for a in range(3):
        for s in (1.0, -1.0):
            u, v = (a + 1) % 3, (a + 2) % 3
            if s < 0:
                u, v = v, u
            n = np.zeros(3)
            n[a] = s
            base = len(pos)
            for su, sv in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
                p = c.copy()
                p[a] += s * h[a]
                p[u] += su * h[u]
                p[v] += sv * h[v]
                pos.append(p)
                nrm.append(-n if inward else n)
            if inward:
                tris += [(base, base + 2, base + 1), (base, base + 3, base + 2)]
            else:
                tris += [(base, base + 1, base + 2), (base, base + 2, base + 3)]
    return np.array(pos), np.array(nrm), np.array(tris, np.uint32)


def yaw_matrix(yaw):
    cy, sy = np.cos(yaw), np.sin(yaw)
    return np.array([[cy, 0.0, sy], [0.0, 1.0, 0.0], [-sy, 0.0, cy]])


def affine_3x4(linear, translation):
    m = np.zeros((3, 4))
    m[:, :3] = linear
    m[:, 3] = translation
    return m.reshape(12).astype(np.float32)


def make_vertices(pos, nrm):
    v = np.zeros(len(pos), VERTEX_DTYPE)
    v["pos"] = pos
    v["normal"] = nrm
    v["color"] = 1.0
    v["tangent"] = (1.0, 0.0, 0.0, 1.0)
    return v


def make_materials(rng, n, lo, hi):
    m = np.zeros(n, MATERIAL_DTYPE)
    m["metallic"] = 0.0
    m["roughness"] = 1.0
    m["base_color"] = rng.uniform(lo, hi, size=(n, 3))
    m["emissive"] = 0.0
    for k in ("albedo_texture", "normal_texture", "metallic_roughness_texture", "emissive_texture"):
        m[k] = NO_TEXTURE
    return m


def gen_basis(n):
    """genBasis of src/IrradianceProbes.cpp:347-355."""
    b1 = np.array([0.0, 1.0, 0.0]) if n[0] > 0.9 else np.array([1.0, 0.0, 0.0])
    b1 = b1 - n * np.dot(b1, n)
    b1 = b1 / np.linalg.norm(b1)
    b2 = np.cross(n, b1)
    return b1, b2


def random_orientation(seed, k):
    """Seeded stand-in for the unseeded glm::sphericalRand + genBasis of
    src/IrradianceProbes.cpp:455-460: rows X, Y, Z of
    transpose(mat3(X, Y, Z))."""
    rng = np.random.default_rng([int(seed), 7919, int(k)])
    z = rng.uniform(-1.0, 1.0)
    phi = rng.uniform(0.0, 2.0 * np.pi)
    r = np.sqrt(max(0.0, 1.0 - z * z))
    Z = np.array([r * np.cos(phi), r * np.sin(phi), z])
    X, Y = gen_basis(Z)
    return np.stack([X, Y, Z]).astype(np.float32).reshape(9)


def scene_bounds(scene):
    """World bounds of all instances ("Fit to Scene", src/UI.cpp:996-1000)."""
    lo = np.full(3, np.inf)
    hi = np.full(3, -np.inf)
    pos = scene.vertices["pos"].astype(np.float64)
    for mi, m in enumerate(scene.meshes):
        sel = scene.instances["mesh_index"] == mi
        if not sel.any():
            continue
        idx = scene.indices[m["index_offset"]:m["index_offset"] + m["index_count"]].astype(np.int64) + m["vertex_offset"]
        p = pos[idx]
        mlo, mhi = p.min(0), p.max(0)
        corners = np.array([[(mlo, mhi)[(c >> k) & 1][k] for k in range(3)] for c in range(8)])
        for t in scene.instances["transform"][sel]:
            M = t.reshape(3, 4).astype(np.float64)
            w = corners @ M[:, :3].T + M[:, 3]
            lo = np.minimum(lo, w.min(0))
            hi = np.maximum(hi, w.max(0))
    return lo, hi


# ---------------------------------------------------------------------------
# room + boxes (the small workload, and the differentiation workload)
# ---------------------------------------------------------------------------
def room_with_boxes(seed, n_boxes=200, n_materials=64, room=(10.0, 6.0, 10.0)):
    rng = np.random.default_rng(seed)
    materials = make_materials(rng, n_materials, 0.2, 0.8)
    rp, rn, rt = box_geometry((0, 0, 0), room, inward=True)
    cp, cn, ct = box_geometry((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    vertices = make_vertices(np.concatenate([rp, cp]), np.concatenate([rn, cn]))
    indices = np.concatenate([rt.reshape(-1), ct.reshape(-1)]).astype(np.uint32)
    meshes = np.zeros(2, MESH_DTYPE)
    meshes[0] = (0, len(rp), 0, rt.size)
    meshes[1] = (len(rp), len(cp), rt.size, ct.size)
    centres = rng.uniform((0.0, 0.0, 0.0), room, size=(n_boxes, 3))
    sides = rng.uniform(0.2, 1.5, size=(n_boxes, 3))
    yaws = rng.uniform(0.0, 2.0 * np.pi, size=n_boxes)
    mats = rng.integers(0, n_materials, size=n_boxes + 1)
    instances = np.zeros(n_boxes + 1, INSTANCE_DTYPE)
    offsets = np.zeros(n_boxes + 1, OFFSET_DTYPE)
    instances[0]["transform"] = affine_3x4(np.eye(3), np.zeros(3))
    instances[0]["custom_index"] = 0
    instances[0]["mask"] = 1
    instances[0]["mesh_index"] = 0
    offsets[0] = (mats[0], 0, 0)
    for i in range(n_boxes):
        lin = yaw_matrix(yaws[i]) @ np.diag(sides[i])
        instances[i + 1]["transform"] = affine_3x4(lin, centres[i])
        instances[i + 1]["custom_index"] = i + 1
        instances[i + 1]["mask"] = 1
        instances[i + 1]["mesh_index"] = 1
        offsets[i + 1] = (mats[i + 1], len(rp), rt.size)
    sc = Scene(vertices, indices, meshes, instances, offsets, materials)
    sc.bounds = scene_bounds(sc)
    return sc


# ---------------------------------------------------------------------------
# terrain + box clusters (the at-scale workload)
# ---------------------------------------------------------------------------
def value_noise(rng, n, octaves=4, base=4):
    """n x n samples of `octaves`-octave value noise in [0, 1]."""
    out = np.zeros((n, n))
    amp_sum = 0.0
    u = np.linspace(0.0, 1.0, n)
    for o in range(octaves):
        cells = base * (2 ** o)
        lattice = rng.uniform(0.0, 1.0, size=(cells + 1, cells + 1))
        x = u * cells
        i0 = np.minimum(np.floor(x).astype(np.int64), cells - 1)
        f = x - i0
        f = f * f * (3.0 - 2.0 * f)
        a = lattice[i0][:, i0]
        b = lattice[i0 + 1][:, i0]
        c = lattice[i0][:, i0 + 1]
        d = lattice[i0 + 1][:, i0 + 1]
        fi = f[:, None]
        fj = f[None, :]
        val = (a * (1 - fi) + b * fi) * (1 - fj) + (c * (1 - fi) + d * fi) * fj
        amp = 0.5 ** o
        out += amp * val
        amp_sum += amp
    out /= amp_sum
    return (out - out.min()) / max(out.max() - out.min(), 1e-12)


def terrain_mesh(rng, cells=512, size=256.0, amplitude=8.0):
    n = cells + 1
    h = value_noise(rng, n) * amplitude
    step = size / cells
    xs = np.arange(n) * step
    X, Z = np.meshgrid(xs, xs, indexing="ij")  # [i, j] -> x = i*step, z = j*step
    pos = np.stack([X, h, Z], -1).reshape(-1, 3)
    dhdx = np.gradient(h, step, axis=0)
    dhdz = np.gradient(h, step, axis=1)
    nrm = np.stack([-dhdx, np.ones_like(h), -dhdz], -1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    nrm = nrm.reshape(-1, 3)
    i, j = np.meshgrid(np.arange(cells), np.arange(cells), indexing="ij")
    a = (i * n + j).reshape(-1)
    b = ((i + 1) * n + j).reshape(-1)
    c = (i * n + j + 1).reshape(-1)
    d = ((i + 1) * n + j + 1).reshape(-1)
    tris = np.stack([np.stack([a, c, b], -1), np.stack([b, c, d], -1)], 1).reshape(-1, 3)
    return pos, nrm, tris.astype(np.uint32), h, step


def cluster_mesh(rng, n_boxes=5000, extent=2.0, height=4.0):
    cp, cn, ct = box_geometry((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    centres = np.column_stack([
        rng.uniform(-extent, extent, n_boxes), rng.uniform(0.0, height, n_boxes), rng.uniform(-extent, extent, n_boxes)])
    sides = rng.uniform(0.1, 0.6, size=(n_boxes, 3))
    yaws = rng.uniform(0.0, 2.0 * np.pi, size=n_boxes)
    cy, sy = np.cos(yaws), np.sin(yaws)
    R = np.zeros((n_boxes, 3, 3))
    R[:, 0, 0] = cy
    R[:, 0, 2] = sy
    R[:, 1, 1] = 1.0
    R[:, 2, 0] = -sy
    R[:, 2, 2] = cy
    lin = R * sides[:, None, :]
    pos = np.einsum("bij,vj->bvi", lin, cp) + centres[:, None, :]
    nrm = np.einsum("bij,vj->bvi", R, cn)
    tris = ct[None, :, :] + (np.arange(n_boxes) * len(cp))[:, None, None]
    return pos.reshape(-1, 3), nrm.reshape(-1, 3), tris.reshape(-1, 3).astype(np.uint32)


def terrain_with_clusters(seed, n_instances=4096, n_cluster_meshes=8, boxes_per_cluster=5000, n_materials=256,
                          cells=512, size=256.0, amplitude=8.0):
    rng = np.random.default_rng(seed)
    materials = make_materials(rng, n_materials, 0.1, 0.9)
    tp, tn, tt, heights, step = terrain_mesh(rng, cells, size, amplitude)
    parts_p, parts_n, parts_t = [tp], [tn], [tt.reshape(-1)]
    meshes = np.zeros(1 + n_cluster_meshes, MESH_DTYPE)
    meshes[0] = (0, len(tp), 0, tt.size)
    vofs, iofs = len(tp), tt.size
    for k in range(n_cluster_meshes):
        p, nr, t = cluster_mesh(rng, boxes_per_cluster)
        parts_p.append(p)
        parts_n.append(nr)
        parts_t.append(t.reshape(-1))
        meshes[1 + k] = (vofs, len(p), iofs, t.size)
        vofs += len(p)
        iofs += t.size
    vertices = make_vertices(np.concatenate(parts_p), np.concatenate(parts_n))
    indices = np.concatenate(parts_t).astype(np.uint32)

    which = rng.integers(0, n_cluster_meshes, size=n_instances)
    xz = rng.uniform(4.0, size - 4.0, size=(n_instances, 2))
    yaws = rng.uniform(0.0, 2.0 * np.pi, size=n_instances)
    scales = rng.uniform(0.5, 3.0, size=n_instances)
    mats = rng.integers(0, n_materials, size=n_instances + 1)
    # terrain height under each instance (bilinear on the vertex grid)
    gi = xz / step
    i0 = np.minimum(np.floor(gi).astype(np.int64), cells - 1)
    f = gi - i0
    h00 = heights[i0[:, 0], i0[:, 1]]
    h10 = heights[i0[:, 0] + 1, i0[:, 1]]
    h01 = heights[i0[:, 0], i0[:, 1] + 1]
    h11 = heights[i0[:, 0] + 1, i0[:, 1] + 1]
    y = (h00 * (1 - f[:, 0]) + h10 * f[:, 0]) * (1 - f[:, 1]) + (h01 * (1 - f[:, 0]) + h11 * f[:, 0]) * f[:, 1]

    instances = np.zeros(n_instances + 1, INSTANCE_DTYPE)
    offsets = np.zeros(n_instances + 1, OFFSET_DTYPE)
    instances[0]["transform"] = affine_3x4(np.eye(3), np.zeros(3))
    instances[0]["mask"] = 1
    instances[0]["custom_index"] = 0
    instances[0]["mesh_index"] = 0
    offsets[0] = (mats[0], 0, 0)
    for i in range(n_instances):
        m = meshes[1 + which[i]]
        lin = yaw_matrix(yaws[i]) * scales[i]
        instances[i + 1]["transform"] = affine_3x4(lin, (xz[i, 0], y[i], xz[i, 1]))
        instances[i + 1]["custom_index"] = i + 1
        instances[i + 1]["mask"] = 1
        instances[i + 1]["mesh_index"] = 1 + which[i]
        offsets[i + 1] = (mats[i + 1], m["vertex_offset"], m["index_offset"])
    sc = Scene(vertices, indices, meshes, instances, offsets, materials)
    sc.bounds = scene_bounds(sc)
    return sc


# ---------------------------------------------------------------------------
# named workloads
# ---------------------------------------------------------------------------
def default_light():
    return make_light(SUN_TOWARDS, SUN_RADIANCE, SKY_RADIANCE)


def fit_grid(scene, resolution, rays, precision=PRECISION_FP32, color_res=8, depth_res=16, hysteresis=0.97,
             depth_sharpness=50.0, shadow_bias=0.05):
    lo, hi = scene.bounds
    return make_grid(lo.astype(np.float32), hi.astype(np.float32), resolution, rays, color_res, depth_res, hysteresis,
                     depth_sharpness, shadow_bias, precision)


def room_workload(seed=1234, n_boxes=200, resolution=(8, 8, 8), rays=128, updates=1, precision=PRECISION_FP32,
                  color_res=8, depth_res=16):
    """Room 10x6x10 m + `n_boxes` boxes (12 triangles each), 8x8x8 probes,
    128 rays, one update from a zero atlas."""
    sc = room_with_boxes(seed, n_boxes)
    sc.bounds = (np.zeros(3), np.array([10.0, 6.0, 10.0]))  # the grid spans the room
    g = fit_grid(sc, resolution, rays, precision, color_res, depth_res)
    return Workload("room%d_%dx%dx%d_r%d" % (n_boxes, *resolution, rays), sc, g, default_light(), updates, seed)


def terrain_workload(seed=1235, resolution=(32, 16, 32), rays=256, updates=10, precision=PRECISION_FP32,
                     n_instances=4096, boxes_per_cluster=5000, cells=512):
    """512x512-cell terrain + 4096 instances of 8 box-cluster meshes
    (~1M unique triangles), 32x16x32 probes, 256 rays, 10 updates."""
    sc = terrain_with_clusters(seed, n_instances=n_instances, boxes_per_cluster=boxes_per_cluster, cells=cells)
    g = fit_grid(sc, resolution, rays, precision)
    return Workload("terrain_%dx%dx%d_r%d" % (*resolution, rays), sc, g, default_light(), updates, seed)


def batch_workloads(seed=1238, count=48, tri_range=(5000, 300000)):
    """The batching workload: `count` independent probe volumes of uneven
    sizes.  Volume v (own PCG64 stream [seed, v]) uses the room or the
    terrain generator with a unique-triangle count log-uniform in
    `tri_range`, a probe grid between 4x4x4 and 24x12x24, 64/128/256/512
    rays per probe, 8/16 or 6/14 atlas tiles and the FP32 or BF16 form."""
    out = []
    for v in range(count):
        rng = np.random.default_rng([int(seed), int(v)])
        target = float(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]))))
        kind = "room" if rng.uniform() < 0.5 else "terrain"
        res = (int(rng.integers(4, 25)), int(rng.integers(4, 13)), int(rng.integers(4, 25)))
        rays = int(rng.choice([64, 128, 256, 512]))
        color_res, depth_res = (8, 16) if rng.uniform() < 0.5 else (6, 14)
        precision = int(rng.integers(0, 2))
        vseed = int(rng.integers(0, 2 ** 31 - 1))
        if kind == "room":
            n_boxes = max(1, int(round((target - 12) / 12)))
            sc = room_with_boxes(vseed, n_boxes)
            sc.bounds = (np.zeros(3), np.array([10.0, 6.0, 10.0]))
        else:
            cells = max(24, int(round(np.sqrt(target / 4.0))))
            boxes = max(1, int(round(target / 2.0 / 24.0)))
            sc = terrain_with_clusters(vseed, n_instances=max(16, int(target) // 2000), n_cluster_meshes=2,
                                       boxes_per_cluster=boxes, cells=cells, size=cells * 0.5,
                                       amplitude=4.0)
        g = fit_grid(sc, res, rays, precision, color_res, depth_res)
        # room: instanced triangles (one box mesh), terrain: unique triangles
        tris = sc.triangle_count if kind == "room" else sc.unique_triangle_count
        name = "%s%d_%dx%dx%d_r%d_%d_%s" % (kind, tris, *res, rays, color_res,
                                            "bf16" if precision else "fp32")
        out.append(Workload(name, sc, g, default_light(), 1, vseed))
    return out


def workload(config, seed=None):
    """Workload of a numbered configuration: 0 room (plain FP32, 1 update),
    1 terrain at scale (FP32, 10 updates), 2 terrain with the BF16 blend,
    3 room with 1000 boxes on a 16x8x16 grid (differentiation)."""
    if config == 0:
        return room_workload(1234 if seed is None else seed)
    if config == 1:
        return terrain_workload(1235 if seed is None else seed)
    if config == 2:
        return terrain_workload(1235 if seed is None else seed, precision=1)
    if config == 3:
        return room_workload(1237 if seed is None else seed, n_boxes=1000, resolution=(16, 8, 16), rays=256, updates=8)
    raise ValueError("unknown configuration %r" % (config,))

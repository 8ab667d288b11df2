// common.cuh — device-side types and math shared by the DDGI kernels.
//
// Everything that decides WHICH triangle a ray hits (probe origin, ray
// transform, watertight triangle test, hit position) is written with
// explicitly rounded intrinsics (__fmul_rn / __fadd_rn / __fdiv_rn), so that
// no multiply-add is contracted and the result is bit-identical to a
// separately-rounded CPU evaluation.  The shading math below it may contract.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ddgi.h"
#include "../../include/ddgi_exact.h"

namespace ddgi {

// ---------------------------------------------------------------------------
// Device error word: kernels never trap; they record the first failure here
// and the host turns it into DDGI_ERR_DEVICE.
// ---------------------------------------------------------------------------
enum DeviceError : uint32_t {
    DEV_OK = 0,
    DEV_STACK_OVERFLOW = 1,
    DEV_BAD_INDEX = 2,
    DEV_WAIT_TIMEOUT = 3,
};

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t code) {
    if (err) atomicCAS(err, 0u, code);
}

// Device wall clock in nanoseconds (for per-volume completion stamps).
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------
// Acceleration-structure records (16-byte vectorised)
// ---------------------------------------------------------------------------
// Binary node, 64 bytes: the boxes of both children and their references.
//   a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   d = (ref0, ref1, unused, unused)
// ref >= 0: inner node index; ref < 0: leaf, ~ref = (first << 3) | (count - 1)
// with 1..8 primitives from `first` (triangles in a bottom level, one
// instance in the top level).
// Default of the traversals' straggler threshold: a warp leaves its
// node-search loop once at most this many lanes still look for a first leaf.
constexpr uint32_t kDefaultWait = 10;

struct __align__(16) BvhNode {
    float4 a, b, c;
    int4 d;
};
static_assert(sizeof(BvhNode) == 64, "node is 64 bytes");

// Triangle in leaf order, 48 bytes: v0 (w = primitive id), v1, v2.
struct __align__(16) BvhTri {
    float4 v0, v1, v2;
};

// Top-level instance record in leaf order, 64 bytes.
struct __align__(16) GpuInstance {
    float4 w2o[3];      // world-to-object rows
    int32_t blas_root;  // global node index of the mesh's root (-1: empty mesh)
    uint32_t custom;    // offset-table entry
    uint32_t mask;
    uint32_t id;        // index in the caller's instance array
};

// Eight-wide node, 96 bytes, collapsed from the binary trees, with the
// child boxes quantised to 8 bits per bound on a per-axis power-of-two grid
// anchored at the node box's lower corner (the compressed wide nodes of
// Ylitie, Karras & Laine, HPG 2017, with explicit child references):
//   org.xyz          grid origin o; org.w holds the biased exponents
//                    e_x | e_y << 8 | e_z << 16 of the grid steps 2^(e - 127)
//   q[a] (a = x,y,z) bytes 0..7 (.x = slots 0-3, .y = 4-7): lower bounds of
//                    the slots' boxes, bytes 8..15 (.z, .w): upper bounds, so
//                    slot k's box is [o + lo_k 2^(e-127), o + hi_k 2^(e-127)]
//                    per axis, rounded outwards (it contains the binary
//                    tree's enlarged box); an empty slot has lo 255, hi 0
//   ref[2]           the eight slots' references (>= 0: wide node, < 0: leaf
//                    as in BvhNode, kNone: empty)
// A slot's bit k of its number is set when its box lies on the low side of
// the node along axis k, so a ray visits slots in decreasing order of
// (slot ^ octant) for a near-first order without sorting.
struct __align__(16) WideNode {
    float4 org;
    uint4 q[3];
    int4 ref[2];
};
static_assert(sizeof(WideNode) == 96, "wide node is 96 bytes");
// Traversal stack entries of wide trees pack a node index into 23 bits.
constexpr uint32_t kMaxWideNodes = 0x7FFFFFu;

struct DeviceScene {
    const BvhNode* nodes;
    const BvhTri* tris;
    const GpuInstance* instances;        // leaf order (traversal)
    const GpuInstance* instances_by_id;  // caller order (shading)
    const float4* normals;  // per vertex (global vertex array), w unused
    const uint32_t* indices;
    const ddgi_offset_entry* offsets;
    const ddgi_material* materials;
    int32_t tlas_root;      // -1: empty scene
    uint32_t vertex_count, index_count, offset_count, material_count;
    uint32_t node_count, tri_count, instance_count;  // bounds of the references above
    // the same trees as eight-wide nodes; instances (leaf order) whose
    // blas_root is a wide-node index
    const WideNode* wnodes;
    const GpuInstance* winstances;
    int32_t wtlas_root;
    uint32_t wnode_count;
    // traversal step limits: a well-formed tree visits each node at most
    // once per ray (4 x (nodes + triangles + instances) + 64, binary / wide)
    uint32_t max_steps, wmax_steps;
};

inline void set_step_limits(DeviceScene& s) {
    s.max_steps = 4u * (s.node_count + s.tri_count + s.instance_count) + 64u;
    s.wmax_steps = 4u * (s.wnode_count + s.tri_count + s.instance_count) + 64u;
}

struct DeviceGrid {
    float mn[3], mx[3];
    float cell[3];        // (max - min) / (res - 1), exact
    float cell_len;       // length(cell)
    float tmax;           // length(max - min), exact
    int res[3];
    uint32_t rays, color_res, depth_res;
    float sharp, hyst, bias;
    uint32_t color_w, color_h, depth_w, depth_h;  // atlas sizes in texels
    uint32_t quant;  // reference-format atlas: stored texels rounded to R11G11B10F / RG16F
};

// Stored texel of the FP32 atlas forms: as computed, or (reference-format
// form) rounded to the reference's image formats, B10G11R11 unsigned floats
// for irradiance and RG16F for depth (src/IrradianceProbes.cpp:41, 63).
__device__ __forceinline__ float4 store_color(const DeviceGrid& g, float r, float gr, float b) {
    if (g.quant) return make_float4(ddgi_round_r11(r), ddgi_round_r11(gr), ddgi_round_b10(b), 1.0f);
    return make_float4(r, gr, b, 1.0f);
}
__device__ __forceinline__ float2 store_depth(const DeviceGrid& g, float m, float m2) {
    if (g.quant) return make_float2(ddgi_round_half(m), ddgi_round_half(m2));
    return make_float2(m, m2);
}

struct DeviceLight {
    float dir[3], color[3], sky[3];
    float sun_brightness;  // LightBuffer.color.a: the atmospheric sky's sun factor
    uint32_t sky_mode;     // ddgi_sky_mode of the miss radiance
};

// ---------------------------------------------------------------------------
// Exact helpers
// ---------------------------------------------------------------------------
// Border entry e of an octahedral tile of side n: (dst x, dst y, src x,
// src y), the table of src/shaders/probesCopyBorders.comp:21-245 generalised
// to any side: entries 0-3 the corners, then the four edges of n - 2 texels,
// each a copy of the mirrored interior texel next to the opposite edge.
__device__ __forceinline__ int4 border_entry(int e, int n) {
    int m = n - 2;
    if (e == 0) return make_int4(0, 0, n - 2, n - 2);
    if (e == 1) return make_int4(0, n - 1, n - 2, 1);
    if (e == 2) return make_int4(n - 1, 0, 1, n - 2);
    if (e == 3) return make_int4(n - 1, n - 1, 1, 1);
    e -= 4;
    int side = e / m, j = e % m + 1;
    if (side == 0) return make_int4(0, j, 1, n - 1 - j);
    if (side == 1) return make_int4(n - 1, j, n - 2, n - 1 - j);
    if (side == 2) return make_int4(j, 0, n - 1 - j, 1);
    return make_int4(j, n - 1, n - 1 - j, n - 2);
}

__device__ __forceinline__ float sel3(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ float3 probe_origin_exact(const DeviceGrid& g, uint32_t linear) {
    uint32_t rx = (uint32_t)g.res[0], rxy = (uint32_t)(g.res[0] * g.res[1]);
    int ix = (int)(linear % rx), iy = (int)((linear % rxy) / rx), iz = (int)(linear / rxy);
    return make_float3(__fadd_rn(__fmul_rn((float)ix, g.cell[0]), g.mn[0]),
                       __fadd_rn(__fmul_rn((float)iy, g.cell[1]), g.mn[1]),
                       __fadd_rn(__fmul_rn((float)iz, g.cell[2]), g.mn[2]));
}

struct Ray {
    float3 o, d, inv;
    float Sx, Sy, Sz;
    int kx, ky, kz;
};

// slab reciprocals of a direction (a zero component stands in as 1e-30)
__device__ __forceinline__ float3 ray_inv(float3 d) {
    return make_float3(1.0f / (d.x != 0.0f ? d.x : 1e-30f), 1.0f / (d.y != 0.0f ? d.y : 1e-30f),
                       1.0f / (d.z != 0.0f ? d.z : 1e-30f));
}

__device__ __forceinline__ void ray_setup(Ray& r, float3 o, float3 d) {
    r.o = o;
    r.d = d;
    r.inv = ray_inv(d);
    int kz = 0;
    if (fabsf(d.y) > fabsf(d.x)) kz = 1;
    if (fabsf(d.z) > fabsf(sel3(d, kz))) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    float dz = sel3(d, kz);
    if (dz < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = __fdiv_rn(sel3(d, kx), dz);
    r.Sy = __fdiv_rn(sel3(d, ky), dz);
    r.Sz = __fdiv_rn(1.0f, dz);
}

__device__ __forceinline__ void xform_exact(const float4 w[3], float3 o, float3 d, float3* oo, float3* od) {
    float r[3], s[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float4 m = w[k];
        float a = __fmul_rn(m.x, o.x), b = __fmul_rn(m.y, o.y), c = __fmul_rn(m.z, o.z);
        r[k] = __fadd_rn(__fadd_rn(__fadd_rn(a, b), c), m.w);
        float e = __fmul_rn(m.x, d.x), f = __fmul_rn(m.y, d.y), g = __fmul_rn(m.z, d.z);
        s[k] = __fadd_rn(__fadd_rn(e, f), g);
    }
    *oo = make_float3(r[0], r[1], r[2]);
    *od = make_float3(s[0], s[1], s[2]);
}

// Three-input min / max (PTX min.f32 / max.f32 with three sources, sm_100
// and later): exact, like the two-input forms, in one instruction.
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Watertight ray/triangle test (Woop, Benthin, Wald 2013), every operation
// rounded separately.  Accepts t in [tmin, tmax].
__device__ __forceinline__ bool tri_hit_exact(const Ray& r, float3 v0, float3 v1, float3 v2, float tmin, float tmax,
                                              float* t_out, float* b1, float* b2, bool* back) {
    float3 A = make_float3(__fsub_rn(v0.x, r.o.x), __fsub_rn(v0.y, r.o.y), __fsub_rn(v0.z, r.o.z));
    float3 B = make_float3(__fsub_rn(v1.x, r.o.x), __fsub_rn(v1.y, r.o.y), __fsub_rn(v1.z, r.o.z));
    float3 C = make_float3(__fsub_rn(v2.x, r.o.x), __fsub_rn(v2.y, r.o.y), __fsub_rn(v2.z, r.o.z));
    float Akz = sel3(A, r.kz), Bkz = sel3(B, r.kz), Ckz = sel3(C, r.kz);
    float Ax = __fsub_rn(sel3(A, r.kx), __fmul_rn(r.Sx, Akz));
    float Ay = __fsub_rn(sel3(A, r.ky), __fmul_rn(r.Sy, Akz));
    float Bx = __fsub_rn(sel3(B, r.kx), __fmul_rn(r.Sx, Bkz));
    float By = __fsub_rn(sel3(B, r.ky), __fmul_rn(r.Sy, Bkz));
    float Cx = __fsub_rn(sel3(C, r.kx), __fmul_rn(r.Sx, Ckz));
    float Cy = __fsub_rn(sel3(C, r.ky), __fmul_rn(r.Sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    // edge functions of mixed signs: outside (U, V, W are finite here)
    if (fmin3(U, V, W) < 0.0f && fmax3(U, V, W) > 0.0f) return false;
    float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    float Az = __fmul_rn(r.Sz, Akz), Bz = __fmul_rn(r.Sz, Bkz), Cz = __fmul_rn(r.Sz, Ckz);
    float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    float t = __fdiv_rn(T, det);
    if (!(t >= tmin && t <= tmax)) return false;
    *t_out = t;
    *b1 = __fdiv_rn(V, det);
    *b2 = __fdiv_rn(W, det);
    *back = det < 0.0f;
    return true;
}

// Slab test of both children of a node; returns the distances that order
// them (entry distances, or exit distances when the entries are equal).
__device__ __forceinline__ void node_hit(const Ray& r, const BvhNode& n, float tmin, float tmax, bool* h0, bool* h1,
                                         float* t0, float* t1) {
    float ox = r.o.x, oy = r.o.y, oz = r.o.z;
    float ix = r.inv.x, iy = r.inv.y, iz = r.inv.z;
    float a0 = (n.a.x - ox) * ix, a1 = (n.a.y - ox) * ix;
    float a2 = (n.a.z - oy) * iy, a3 = (n.a.w - oy) * iy;
    float a4 = (n.c.x - oz) * iz, a5 = (n.c.y - oz) * iz;
    float n0 = fmax3(fminf(a0, a1), fminf(a2, a3), fmaxf(fminf(a4, a5), tmin));
    float f0 = fmin3(fmaxf(a0, a1), fmaxf(a2, a3), fminf(fmaxf(a4, a5), tmax));
    float b0 = (n.b.x - ox) * ix, b1 = (n.b.y - ox) * ix;
    float b2 = (n.b.z - oy) * iy, b3 = (n.b.w - oy) * iy;
    float b4 = (n.c.z - oz) * iz, b5 = (n.c.w - oz) * iz;
    float n1 = fmax3(fminf(b0, b1), fminf(b2, b3), fmaxf(fminf(b4, b5), tmin));
    float f1 = fmin3(fmaxf(b0, b1), fmaxf(b2, b3), fminf(fmaxf(b4, b5), tmax));
    *h0 = n0 <= f0;
    *h1 = n1 <= f1;
    // near-first order by entry distance; when both boxes are entered at the
    // same distance (both hold the ray's start, common at the top levels), by
    // exit distance: the box left first is visited first (4 % fewer
    // primary-traversal cycles on the 1M-triangle terrain)
    *t0 = n0 == n1 ? f0 : n0;
    *t1 = n0 == n1 ? f1 : n1;
}

__device__ __forceinline__ BvhNode load_node(const BvhNode* nodes, int i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    BvhNode n;
    n.a = __ldg(p + 0);
    n.b = __ldg(p + 1);
    n.c = __ldg(p + 2);
    float4 dd = __ldg(p + 3);
    n.d = make_int4(__float_as_int(dd.x), __float_as_int(dd.y), __float_as_int(dd.z), __float_as_int(dd.w));
    return n;
}

// ---------------------------------------------------------------------------
// float3 helpers (shading; contraction allowed)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float3 f3(float a, float b, float c) { return make_float3(a, b, c); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(float3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ float3 norm3(float3 a) { return a * (1.0f / len3(a)); }
__device__ __forceinline__ float3 abs3(float3 a) { return f3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ float3 mix3(float3 a, float3 b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float gsign(float v) { return v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ float sign_nz(float v) { return v >= 0.0f ? 1.0f : -1.0f; }

// common.glsl:4
#define DDGI_PI 3.1415926538f

// irradiance.glsl:107-112
__device__ __forceinline__ float3 oct_decode(float ox, float oy) {
    float3 v = f3(ox, oy, 1.0f - fabsf(ox) - fabsf(oy));
    if (v.z < 0.0f) {
        float nx = (1.0f - fabsf(v.y)) * sign_nz(v.x);
        float ny = (1.0f - fabsf(v.x)) * sign_nz(v.y);
        v.x = nx;
        v.y = ny;
    }
    return norm3(v);
}

// irradiance.glsl:119-138
__device__ __forceinline__ float2 sphere_to_oct_uv(float3 d) {
    float3 oct = f3(gsign(d.x), gsign(d.y), gsign(d.z));
    float sum = dot3(d, oct);
    float3 o = f3(d.x / sum, d.y / sum, d.z / sum);
    if (o.z < 0.0f) {
        float3 a = abs3(o);
        float nx = oct.x * (1.0f - a.y);
        float ny = oct.y * (1.0f - a.x);
        o.x = nx;
        o.y = ny;
    }
    return make_float2(o.x * 0.5f + 0.5f, o.y * 0.5f + 0.5f);
}

// Texel-centre scale of probesUpdate.glsl:33-42 for interior side n.
__host__ __device__ __forceinline__ float texel_scale(uint32_t n) {
    if (n == 6) return 0.33333f;
    if (n == 14) return 0.142857f;
    return (float)(2.0 / (double)n);
}

// REPEAT addressing of texel index i on an axis of n texels.  Sample
// coordinates in [-0.5, 1.5] give indices in [-n, 2n), which one add or
// subtract brings into range; anything else takes the remainder (the same
// integer either way, without a division on the common path).
__host__ __device__ __forceinline__ int wrap_repeat(int i, int n) {
    if (i < 0) i += n;
    else if (i >= n) i -= n;
    if ((unsigned)i >= (unsigned)n) i = ((i % n) + n) % n;
    return i;
}

// Exact bilinear fetch, LINEAR filter with REPEAT addressing
// (src/RaytracingDescriptors.hpp:63, 70).
template <int NC, class Tex>
__device__ __forceinline__ void bilinear(const Tex& tex, uint32_t w, uint32_t h, float u, float v, float* out) {
    float x = u * (float)w - 0.5f;
    float y = v * (float)h - 0.5f;
    float fx0 = floorf(x), fy0 = floorf(y);
    float ax = x - fx0, ay = y - fy0;
    int i0 = (int)fx0, j0 = (int)fy0;
    int iw = (int)w, ih = (int)h;
    int i1 = i0 + 1, j1 = j0 + 1;
    i0 = wrap_repeat(i0, iw);
    i1 = wrap_repeat(i1, iw);
    j0 = wrap_repeat(j0, ih);
    j1 = wrap_repeat(j1, ih);
    float t00[NC], t10[NC], t01[NC], t11[NC];
    tex.fetch((size_t)j0 * w + i0, t00);
    tex.fetch((size_t)j0 * w + i1, t10);
    tex.fetch((size_t)j1 * w + i0, t01);
    tex.fetch((size_t)j1 * w + i1, t11);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        float top = t00[c] * (1.0f - ax) + t10[c] * ax;
        float bot = t01[c] * (1.0f - ax) + t11[c] * ax;
        out[c] = top * (1.0f - ay) + bot * ay;
    }
}

// bilinear() for a sample inside one probe tile of an atlas, as every
// lookup of sampleProbes makes: the texture coordinate keeps the sample at
// least half a texel inside the tile (the tile's border texels, filled by
// probesCopyBorders, surround the interior it addresses), so REPEAT
// addressing is the identity and the four texels are found without it; the
// indices are clamped into the atlas all the same, so a fetch never leaves
// it.  32-bit texel indices (atlases below 2^31 texels).
template <int NC, class Tex>
__device__ __forceinline__ void bilinear_tile(const Tex& tex, uint32_t w, uint32_t h, float u, float v, float* out) {
    float x = u * (float)w - 0.5f;
    float y = v * (float)h - 0.5f;
    float fx0 = floorf(x), fy0 = floorf(y);
    float ax = x - fx0, ay = y - fy0;
    const int iw = (int)w, ih = (int)h;
    const int i0 = max((int)fx0, 0), j0 = max((int)fy0, 0);
    const int i1 = min(i0 + 1, iw - 1), j1 = min(j0 + 1, ih - 1);
    const uint32_t r0 = (uint32_t)j0 * w, r1 = (uint32_t)j1 * w;
    float t00[NC], t10[NC], t01[NC], t11[NC];
    tex.fetch(r0 + (uint32_t)i0, t00);
    tex.fetch(r0 + (uint32_t)i1, t10);
    tex.fetch(r1 + (uint32_t)i0, t01);
    tex.fetch(r1 + (uint32_t)i1, t11);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        float top = t00[c] * (1.0f - ax) + t10[c] * ax;
        float bot = t01[c] * (1.0f - ax) + t11[c] * ax;
        out[c] = top * (1.0f - ay) + bot * ay;
    }
}

}  // namespace ddgi

// trace.cu — probe ray trace + hit shading.
//
// One thread per (probe slot, ray).  Replaces src/shaders/traceProbes.rgen
// (launch cell per probe x ray), the closest-hit program
// src/shaders/closesthit.glsl:133-289 with NO_REFLECTION, the miss program
// src/shaders/miss.rmiss:17-23 (constant sky) and the shadow query
// src/shaders/closesthit.glsl:270-281 + shadow.rmiss:6-9.
//
// Traversal walks the top-level LBVH in world space; at an instance leaf it
// pushes an EXIT marker, moves the ray into object space with the instance's
// world-to-object transform and continues in the mesh's LBVH; popping the
// marker restores the world ray.  Rays of a warp come from one probe and are
// binned by direction octant (the ray order table), so the warp's rays share
// their origin and roughly their direction.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "shade.cuh"

namespace ddgi {

namespace {

constexpr int kStack = 64;
constexpr int kExit = 0x7fffffff;
constexpr uint32_t kNoHit = 0xFFFFFFFFu;

struct HitRec {
    float t, b1, b2;
    uint32_t inst, prim;
    bool back;
};

// Fetch counters of the measurement variant (COUNT = true): inner nodes
// visited, triangles tested, instances entered, rays traced, shading bytes.
struct Fetches {
    uint32_t nodes = 0, tris = 0, insts = 0, rays = 0, shade_bytes = 0;
};

// Closest hit (ANY = false) or any hit (ANY = true) with t in [tmin, tmax];
// ties on t go to the lowest (instance, primitive).
template <bool ANY, bool COUNT = false>
__device__ __forceinline__ bool traverse(const DeviceScene& sc, float3 wo, float3 wd, float tmin, float tmax,
                                         uint32_t mask, HitRec* best, uint32_t* err, Fetches* fc = nullptr) {
    if (COUNT) fc->rays++;
    best->inst = kNoHit;
    best->prim = 0;
    best->t = tmax;
    best->b1 = best->b2 = 0.0f;
    best->back = false;
    if (sc.tlas_root < 0) return false;
    Ray r;
    ray_setup(r, wo, wd);
    int stack[kStack];
    int sp = 0;
    int ref = sc.tlas_root;
    bool in_blas = false;
    uint32_t inst_id = 0;
    float tcur = tmax;
    // A well-formed tree visits each node at most once per ray; the cap only
    // stops a malformed one from looping.
    for (uint32_t steps = 0;; ++steps) {
        if (steps > 4u * (sc.node_count + sc.tri_count + sc.instance_count) + 64u) {
            raise_error(err, DEV_BAD_INDEX);
            return best->inst != kNoHit;
        }
        if (ref >= 0) {
            if (COUNT) fc->nodes++;
            if ((uint32_t)ref >= sc.node_count) {
                raise_error(err, DEV_BAD_INDEX);
                return best->inst != kNoHit;
            }
            BvhNode n = load_node(sc.nodes, ref);
            bool h0, h1;
            float t0, t1;
            node_hit(r, n, tmin, tcur, &h0, &h1, &t0, &t1);
            if (h0 && h1) {
                int nearr = n.d.x, farr = n.d.y;
                if (t1 < t0) {
                    nearr = n.d.y;
                    farr = n.d.x;
                }
                if (sp >= kStack) {
                    raise_error(err, DEV_STACK_OVERFLOW);
                    return best->inst != kNoHit;
                }
                stack[sp++] = farr;
                ref = nearr;
                continue;
            }
            if (h0) {
                ref = n.d.x;
                continue;
            }
            if (h1) {
                ref = n.d.y;
                continue;
            }
        } else if (!in_blas) {
            // top-level leaf: one instance
            if ((uint32_t)((~ref) >> 3) >= sc.instance_count) {
                raise_error(err, DEV_BAD_INDEX);
                return best->inst != kNoHit;
            }
            const GpuInstance* gi = sc.instances + ((~ref) >> 3);
            int4 meta = __ldg(reinterpret_cast<const int4*>(gi) + 3);  // blas_root, custom, mask, id
            if (((uint32_t)meta.z & mask) != 0 && meta.x >= 0) {
                if (COUNT) fc->insts++;
                if (sp >= kStack) {
                    raise_error(err, DEV_STACK_OVERFLOW);
                    return best->inst != kNoHit;
                }
                stack[sp++] = kExit;
                float4 w[3] = {__ldg(&gi->w2o[0]), __ldg(&gi->w2o[1]), __ldg(&gi->w2o[2])};
                float3 oo, od;
                xform_exact(w, wo, wd, &oo, &od);
                ray_setup(r, oo, od);
                inst_id = (uint32_t)meta.w;
                in_blas = true;
                ref = meta.x;
                continue;
            }
        } else {
            int first = (~ref) >> 3, count = ((~ref) & 7) + 1;
            if ((uint32_t)first + (uint32_t)count > sc.tri_count) {
                raise_error(err, DEV_BAD_INDEX);
                return best->inst != kNoHit;
            }
            if (COUNT) fc->tris += count;
            for (int k = 0; k < count; ++k) {
                const float4* tp = reinterpret_cast<const float4*>(sc.tris + first + k);
                float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float t, b1, b2;
                bool back;
                if (tri_hit_exact(r, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), f3(c.x, c.y, c.z), tmin, tcur, &t, &b1, &b2,
                                  &back)) {
                    uint32_t prim = (uint32_t)__float_as_int(a.w);
                    bool better = ANY || best->inst == kNoHit || t < best->t ||
                                  (t == best->t && (inst_id < best->inst || (inst_id == best->inst && prim < best->prim)));
                    if (better) {
                        best->t = t;
                        best->inst = inst_id;
                        best->prim = prim;
                        best->b1 = b1;
                        best->b2 = b2;
                        best->back = back;
                        tcur = t;
                        if (ANY) return true;
                    }
                }
            }
        }
        // pop
        for (;;) {
            if (sp == 0) return best->inst != kNoHit;
            ref = stack[--sp];
            if (ref != kExit) break;
            in_blas = false;
            ray_setup(r, wo, wd);
        }
    }
}

// closesthit.glsl:133-289 (NO_REFLECTION, no textures) for a front-face hit.
template <class AV, bool COUNT>
__device__ float3 shade_front(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L,
                              const uint32_t* states, const AV& at, float3 origin, float3 dir, const HitRec& h,
                              uint32_t* err, Fetches* fc) {
    // instance record, offset entry, 3 indices, 3 normals, material, and per
    // sampleProbes call up to 8 probes x (4 colour + 4 depth texels + state)
    if (COUNT)
        fc->shade_bytes += 64 + 12 + 12 + 48 + 48 +
                           2 * 8 * (4 * decltype(at.color)::kBytes + 4 * decltype(at.depth)::kBytes + 4u);
    // hit position: product then sum, each rounded (shared with the shadow ray)
    float3 position = f3(__fadd_rn(__fmul_rn(dir.x, h.t), origin.x), __fadd_rn(__fmul_rn(dir.y, h.t), origin.y),
                         __fadd_rn(__fmul_rn(dir.z, h.t), origin.z));
    const GpuInstance* gi = sc.instances_by_id + h.inst;
    uint32_t custom = __ldg(&gi->custom);
    ddgi_offset_entry oe = sc.offsets[custom];
    uint32_t io = oe.index_offset + 3u * h.prim;
    uint32_t i0 = __ldg(sc.indices + io), i1 = __ldg(sc.indices + io + 1), i2 = __ldg(sc.indices + io + 2);
    uint32_t vb = oe.vertex_offset;
    if (vb + max(i0, max(i1, i2)) >= sc.vertex_count || oe.material_index >= sc.material_count) {
        raise_error(err, DEV_BAD_INDEX);
        return f3(0, 0, 0);
    }
    float4 n0 = __ldg(sc.normals + vb + i0), n1 = __ldg(sc.normals + vb + i1), n2 = __ldg(sc.normals + vb + i2);
    float b1 = h.b1, b2 = h.b2;
    float b0 = 1.0f - b1 - b2;
    float3 tsn = norm3(f3(n0.x * b0 + n1.x * b1 + n2.x * b2, n0.y * b0 + n1.y * b1 + n2.y * b2,
                          n0.z * b0 + n1.z * b1 + n2.z * b2));
    float4 w0 = __ldg(&gi->w2o[0]), w1 = __ldg(&gi->w2o[1]), w2 = __ldg(&gi->w2o[2]);
    // normal * gl_WorldToObjectEXT: transpose of the world-to-object 3x3
    float3 normal = norm3(f3(tsn.x * w0.x + tsn.y * w1.x + tsn.z * w2.x, tsn.x * w0.y + tsn.y * w1.y + tsn.z * w2.y,
                             tsn.x * w0.z + tsn.y * w1.z + tsn.z * w2.z));
    const ddgi_material& m = sc.materials[oe.material_index];
    float3 albedo = f3(m.base_color[0], m.base_color[1], m.base_color[2]);
    float metal = m.metallic, rough = m.roughness;
    float3 color = f3(m.emissive[0], m.emissive[1], m.emissive[2]);
    float3 diffuseColor = albedo * (1.0f - 0.04f) * (1.0f - metal);
    float3 specularColor = mix3(f3(0.04f, 0.04f, 0.04f), albedo, metal);
    float3 reflectDir = dir - normal * (2.0f * dot3(normal, dir));
    float3 reflection = sample_probes(position, reflectDir, -dir, g, states, at);
    color = color + specularColor * reflection;
    float3 indirect = sample_probes(position, normal, -dir, g, states, at);
    color = color + indirect * diffuseColor;
    HitRec sh;
    bool shadowed =
        traverse<true, COUNT>(sc, position, f3(L.dir[0], L.dir[1], L.dir[2]), 0.1f, 10000.0f, 0xFFu, &sh, err, fc);
    if (!shadowed) {
        color = color + pbr_metallic_roughness(normal, norm3(-dir), f3(L.color[0], L.color[1], L.color[2]),
                                               f3(L.dir[0], L.dir[1], L.dir[2]), albedo, metal, rough);
        if (L.dir[1] < 0.0f) color = color * (1.0f - clampf(-L.dir[1], 0.0f, 0.1f) / 0.1f);
    }
    return color;
}

__device__ __forceinline__ void flush_counters(const Fetches& fc, unsigned long long* c) {
    unsigned long long v[5] = {fc.nodes, fc.tris, fc.insts, fc.rays, fc.shade_bytes};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        unsigned long long x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(c + k, x);
    }
}

template <class AV, bool COUNT>
__global__ void __launch_bounds__(128) k_trace_shade(DeviceScene sc, DeviceGrid g, DeviceLight L,
                                                     const uint32_t* __restrict__ probe_list, uint32_t nprobes,
                                                     const float4* __restrict__ dirs,
                                                     const uint32_t* __restrict__ ray_order,
                                                     const uint32_t* __restrict__ states, AV at, float4* rays_out,
                                                     ddgi_hit* hits_out, uint32_t* err,
                                                     unsigned long long* counters) {
    Fetches fc;
    uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t R = g.rays;
    if (gid >= nprobes * R) {
        if (COUNT) flush_counters(fc, counters);
        return;
    }
    uint32_t slot = gid / R, j = gid - slot * R;
    uint32_t ray = __ldg(ray_order + j);
    uint32_t probe = probe_list ? __ldg(probe_list + slot) : slot;
    float3 o = probe_origin_exact(g, probe);
    float4 d4 = __ldg(dirs + ray);
    float3 d = f3(d4.x, d4.y, d4.z);
    HitRec h;
    bool hit = traverse<false, COUNT>(sc, o, d, 0.01f, g.tmax, 0x3u, &h, err, &fc);
    float4 rec;
    if (!hit) {
        rec = make_float4(L.sky[0], L.sky[1], L.sky[2], -1.0f);  // miss.rmiss:17-23
    } else if (h.back) {
        rec = make_float4(0.0f, 0.0f, 0.0f, h.t * 0.80f);  // closesthit.glsl:137-141
    } else {
        float3 c = shade_front<AV, COUNT>(sc, g, L, states, at, o, d, h, err, &fc);
        rec = make_float4(c.x, c.y, c.z, h.t);
    }
    size_t out = (size_t)slot * R + ray;
    rays_out[out] = rec;
    if (hits_out) {
        ddgi_hit hr;
        hr.instance = hit ? h.inst : kNoHit;
        hr.primitive = hit ? h.prim : 0u;
        hr.t = hit ? h.t : 0.0f;
        hr.backface = (hit && h.back) ? 1u : 0u;
        hits_out[out] = hr;
    }
    if (COUNT) {
        fc.shade_bytes += 16;  // ray record
        flush_counters(fc, counters);
    }
}

// Generic closest-hit / any-hit queries (parity tests of the traversal).
__global__ void k_trace_rays(DeviceScene sc, const float* origins, const float* dirs, uint32_t n, float tmin,
                             float tmax, uint32_t mask, int any, ddgi_hit* out, float* bary, uint32_t* err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 o = f3(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]);
    float3 d = f3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
    HitRec h;
    bool hit = any ? traverse<true>(sc, o, d, tmin, tmax, mask, &h, err)
                   : traverse<false>(sc, o, d, tmin, tmax, mask, &h, err);
    ddgi_hit hr;
    hr.instance = hit ? h.inst : kNoHit;
    hr.primitive = hit ? h.prim : 0u;
    hr.t = hit ? h.t : 0.0f;
    hr.backface = (hit && h.back) ? 1u : 0u;
    out[i] = hr;
    if (bary) {
        bary[2 * i] = hit ? h.b1 : 0.0f;
        bary[2 * i + 1] = hit ? h.b2 : 0.0f;
    }
}

}  // namespace

cudaError_t launch_trace_shade(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L,
                               const uint32_t* probe_list, uint32_t nprobes, const float4* dirs,
                               const uint32_t* ray_order, const uint32_t* states, const void* color,
                               const void* depth, bool fp16_atlas, float4* rays_out, ddgi_hit* hits_out,
                               uint32_t* err, cudaStream_t st, unsigned long long* counters) {
    uint64_t total = (uint64_t)nprobes * g.rays;
    if (total == 0) return cudaSuccess;
    const int T = 128;
    uint32_t blocks = (uint32_t)((total + T - 1) / T);
    if (fp16_atlas) {
        AtlasView<ColorTexF16, DepthTexF16> at{{static_cast<const uint2*>(color)},
                                               {static_cast<const uint32_t*>(depth)}};
        if (counters)
            k_trace_shade<decltype(at), true><<<blocks, T, 0, st>>>(sc, g, L, probe_list, nprobes, dirs, ray_order,
                                                                    states, at, rays_out, hits_out, err, counters);
        else
            k_trace_shade<decltype(at), false><<<blocks, T, 0, st>>>(sc, g, L, probe_list, nprobes, dirs, ray_order,
                                                                     states, at, rays_out, hits_out, err, nullptr);
    } else {
        AtlasView<ColorTexF32, DepthTexF32> at{{static_cast<const float4*>(color)},
                                               {static_cast<const float2*>(depth)}};
        if (counters)
            k_trace_shade<decltype(at), true><<<blocks, T, 0, st>>>(sc, g, L, probe_list, nprobes, dirs, ray_order,
                                                                    states, at, rays_out, hits_out, err, counters);
        else
            k_trace_shade<decltype(at), false><<<blocks, T, 0, st>>>(sc, g, L, probe_list, nprobes, dirs, ray_order,
                                                                     states, at, rays_out, hits_out, err, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_trace_rays(const DeviceScene& sc, const float* origins, const float* dirs, uint32_t n, float tmin,
                              float tmax, uint32_t mask, int any, ddgi_hit* out, float* bary, uint32_t* err,
                              cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const int T = 128;
    k_trace_rays<<<(n + T - 1) / T, T, 0, st>>>(sc, origins, dirs, n, tmin, tmax, mask, any, out, bary, err);
    return cudaGetLastError();
}

}  // namespace ddgi

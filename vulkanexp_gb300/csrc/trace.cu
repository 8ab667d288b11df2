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
#include "traverse.cuh"

namespace ddgi {

namespace {

// closesthit.glsl:133-289 (NO_REFLECTION, no textures) for a front-face hit,
// with the shadow query traced inline.
template <class AV, bool COUNT>
__device__ float3 shade_front(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L,
                              const uint32_t* states, const AV& at, float3 origin, float3 dir, const HitRec& h,
                              uint32_t* err, Fetches* fc) {
    // instance record, offset entry, 3 indices, 3 normals, material, and per
    // sampleProbes call up to 8 probes x (4 colour + 4 depth texels + state)
    if (COUNT)
        fc->shade_bytes += 64 + 12 + 12 + 48 + 48 +
                           2 * 8 * (4 * decltype(at.color)::kBytes + 4 * decltype(at.depth)::kBytes + 4u);
    SurfaceShade s;
    if (!shade_surface(sc, g, L, states, at, origin, dir, h.t, h.b1, h.b2, h.inst, h.prim, &s, err)) return s.base;
    HitRec sh;
    bool shadowed =
        traverse<true, COUNT>(sc, s.position, f3(L.dir[0], L.dir[1], L.dir[2]), 0.1f, 10000.0f, 0xFFu, &sh, err, fc);
    return shadowed ? s.base : lit_color(s);
}

__device__ __forceinline__ void flush_counters(const Fetches& fc, unsigned long long* c) {
    unsigned long long v[11] = {fc.nodes[0], fc.tris[0], fc.insts[0], fc.rays[0], fc.shade_bytes,
                                fc.nodes[1], fc.tris[1], fc.insts[1], fc.rays[1], fc.top_nodes[0], fc.top_nodes[1]};
#pragma unroll
    for (int k = 0; k < 11; ++k) {
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

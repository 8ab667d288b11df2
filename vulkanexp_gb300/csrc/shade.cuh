// shade.cuh — hit shading of a probe ray: sampleProbes (the infinite-bounce
// lookup into the previous atlas), the sun BRDF, and the closest-hit program
// of the reference with NO_REFLECTION.
#pragma once

#include <cuda_fp16.h>

#include "common.cuh"

namespace ddgi {

// Atlas views.  FP32 form: float4 colour (RGBA) and float2 depth texels;
// FP16 form: 4 x half colour and 2 x half depth texels.
struct ColorTexF32 {
    static constexpr uint32_t kBytes = 16;
    const float4* p;
    __device__ __forceinline__ void fetch(size_t i, float* o) const {
        float4 v = __ldg(p + i);
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
    }
};
struct DepthTexF32 {
    static constexpr uint32_t kBytes = 8;
    const float2* p;
    __device__ __forceinline__ void fetch(size_t i, float* o) const {
        float2 v = __ldg(p + i);
        o[0] = v.x;
        o[1] = v.y;
    }
};
struct ColorTexF16 {
    static constexpr uint32_t kBytes = 8;
    const uint2* p;  // 4 halves
    __device__ __forceinline__ void fetch(size_t i, float* o) const {
        uint2 v = __ldg(p + i);
        __half2 a = *reinterpret_cast<__half2*>(&v.x);
        __half2 b = *reinterpret_cast<__half2*>(&v.y);
        float2 fa = __half22float2(a), fb = __half22float2(b);
        o[0] = fa.x;
        o[1] = fa.y;
        o[2] = fb.x;
    }
};
struct DepthTexF16 {
    static constexpr uint32_t kBytes = 4;
    const uint32_t* p;  // 2 halves
    __device__ __forceinline__ void fetch(size_t i, float* o) const {
        uint32_t v = __ldg(p + i);
        float2 f = __half22float2(*reinterpret_cast<__half2*>(&v));
        o[0] = f.x;
        o[1] = f.y;
    }
};

// Either form, chosen per lookup at run time (the batched kernels, whose
// volumes may mix the forms): one copy of the shading code instead of one
// per form.
struct ColorTexDyn {
    const void* p;
    bool half;
    __device__ __forceinline__ void fetch(size_t i, float* o) const {
        if (half) ColorTexF16{static_cast<const uint2*>(p)}.fetch(i, o);
        else ColorTexF32{static_cast<const float4*>(p)}.fetch(i, o);
    }
};
struct DepthTexDyn {
    const void* p;
    bool half;
    __device__ __forceinline__ void fetch(size_t i, float* o) const {
        if (half) DepthTexF16{static_cast<const uint32_t*>(p)}.fetch(i, o);
        else DepthTexF32{static_cast<const float2*>(p)}.fetch(i, o);
    }
};

template <class CT, class DT>
struct AtlasView {
    CT color;
    DT depth;
};

__device__ __forceinline__ float3 grid_probe_pos(const DeviceGrid& g, int x, int y, int z) {
    return f3((float)x * g.cell[0] + g.mn[0], (float)y * g.cell[1] + g.mn[1], (float)z * g.cell[2] + g.mn[2]);
}

// sampleProbes (src/shaders/irradiance.glsl:145-237) for NQ lookups at one
// position that differ in the direction argument (`normal`): the closest-hit
// program makes two (reflection and diffuse), which share the eight probes'
// states, positions, directions and trilinear weights.  Each lookup's
// arithmetic is the reference's.
template <int NQ, class AV>
__device__ void sample_probes_n(float3 position, const float3 (&normal)[NQ], float3 toCamera, const DeviceGrid& g,
                                const uint32_t* states, const AV& at, float3 (&result)[NQ]) {
    float3 cs = abs3(f3(g.cell[0], g.cell[1], g.cell[2]));
    float3 gridCoords = (position - f3(g.mn[0], g.mn[1], g.mn[2])) / cs;
    // (written so that NaN also returns 0)
    if (!(gridCoords.x >= 0.0f && gridCoords.y >= 0.0f && gridCoords.z >= 0.0f)) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) result[q] = f3(0, 0, 0);
        return;
    }
    float3 biasedPosition[NQ];
    float2 nuv[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        biasedPosition[q] = position + (normal[q] + toCamera) * g.bias;
        nuv[q] = sphere_to_oct_uv(normal[q]);
    }
    // the clamp only matters beyond 2^24 cells, where every corner is off-grid
    int fx = (int)fminf(gridCoords.x, 16777216.0f), fy = (int)fminf(gridCoords.y, 16777216.0f),
        fz = (int)fminf(gridCoords.z, 16777216.0f);
    float3 alpha = (position - grid_probe_pos(g, fx, fy, fz)) / cs;
    alpha = f3(clampf(alpha.x, 0.0f, 1.0f), clampf(alpha.y, 0.0f, 1.0f), clampf(alpha.z, 0.0f, 1.0f));

    float3 finalColor[NQ], fallbackColor[NQ];
    float totalWeight[NQ], totalFallbackWeight[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        finalColor[q] = fallbackColor[q] = f3(0, 0, 0);
        totalWeight[q] = totalFallbackWeight[q] = 0.0f;
    }
    const float uvsx = (float)(g.res[0] * g.res[1]), uvsy = (float)g.res[2];
    const float cr = (float)g.color_res, dr = (float)g.depth_res;
    const float cscale = (float)(g.color_res - 2) / cr;
    const float dscale = (float)(g.depth_res - 2) / dr;

#pragma unroll 1
    for (int i = 0; i < 8; ++i) {
        int ox = i & 1, oy = (i >> 1) & 1, oz = (i >> 2) & 1;
        int px = fx + ox, py = fy + oy, pz = fz + oz;
        if (px > g.res[0] - 1 || py > g.res[1] - 1 || pz > g.res[2] - 1) continue;
        uint32_t lin = (uint32_t)(px + g.res[0] * py + g.res[0] * g.res[1] * pz);
        if (__ldg(states + lin) == 0) continue;
        float3 probePosition = grid_probe_pos(g, px, py, pz);
        float3 directionToProbe = norm3(probePosition - position);
        int tile = py * g.res[0] + px;
        const float ctile = (float)((int)g.color_res * tile + 1) / cr, cpz = (float)((int)g.color_res * pz + 1) / cr;
        const float dtile = (float)((int)g.depth_res * tile + 1) / dr, dpz = (float)((int)g.depth_res * pz + 1) / dr;
        float3 tri = f3(ox ? alpha.x : 1.0f - alpha.x, oy ? alpha.y : 1.0f - alpha.y, oz ? alpha.z : 1.0f - alpha.z);
        float triw = tri.x * tri.y * tri.z + 0.001f;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            float3 biasedDirectionToProbe = probePosition - biasedPosition[q];
            float2 duv = sphere_to_oct_uv(-norm3(biasedDirectionToProbe));
            float cu = (ctile + cscale * nuv[q].x) / uvsx;
            float cv = (cpz + cscale * nuv[q].y) / uvsy;
            float du = (dtile + dscale * duv.x) / uvsx;
            float dv = (dpz + dscale * duv.y) / uvsy;
            float weight = 1.0f;
            float bfw = fmaxf(0.0001f, (dot3(directionToProbe, normal[q]) + 1.0f) * 0.5f);
            weight *= bfw * bfw + 0.2f;
            float fallbackWeight = weight;
            float depth[2];
            bilinear_tile<2>(at.depth, g.depth_w, g.depth_h, du, dv, depth);
            float mean = depth[0];
            float variance = fabsf(depth[0] * depth[0] - depth[1]);
            float dist = len3(probePosition - biasedPosition[q]);
            float dm = fmaxf(dist - mean, 0.0001f);
            float cheb = variance / (variance + dm * dm);
            cheb = fmaxf(cheb * cheb * cheb, 0.0f);
            weight *= (dist <= mean) ? 1.0f : cheb;
            weight = fmaxf(0.000001f, weight);
            const float crush = 0.2f;
            if (weight < crush) weight *= weight * weight * (1.0f / (crush * crush));
            weight *= triw;
            fallbackWeight *= triw;
            float col[3];
            bilinear_tile<3>(at.color, g.color_w, g.color_h, cu, cv, col);
            float3 color = f3(sqrtf(col[0]), sqrtf(col[1]), sqrtf(col[2]));
            finalColor[q] = finalColor[q] + color * weight;
            totalWeight[q] += weight;
            fallbackColor[q] = fallbackColor[q] + color * fallbackWeight;
            totalFallbackWeight[q] += fallbackWeight;
        }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        float3 fc = finalColor[q], fb = fallbackColor[q];
        if (totalWeight[q] > 1e-3f) fc = fc * (1.0f / totalWeight[q]);
        if (totalFallbackWeight[q] > 1e-3f) fb = fb * (1.0f / totalFallbackWeight[q]);
        fc = fc * fc;
        fb = fb * fb;
        result[q] = mix3(fb, fc, 8.0f * clampf(totalWeight[q], 0.0f, 1.0f / 8.0f));
    }
}

template <class AV>
__device__ __forceinline__ float3 sample_probes(float3 position, float3 normal, float3 toCamera, const DeviceGrid& g,
                                                const uint32_t* states, const AV& at) {
    const float3 n[1] = {normal};
    float3 r[1];
    sample_probes_n<1>(position, n, toCamera, g, states, at, r);
    return r[0];
}

// pbrMetallicRoughness (src/shaders/pbrMetallicRoughness.glsl:43-84)
__device__ __forceinline__ float3 pbr_metallic_roughness(float3 n, float3 v, float3 lightColor, float3 lightDir,
                                                         float3 albedo, float metal, float rough) {
    const float pi = DDGI_PI;
    float3 diffuseColor = albedo * (1.0f - 0.04f) * (1.0f - metal);
    float alphaRoughness = rough * rough;
    float3 specularColor = mix3(f3(0.04f, 0.04f, 0.04f), albedo, metal);
    float reflectance = fmaxf(fmaxf(specularColor.x, specularColor.y), specularColor.z);
    float reflectance90 = clampf(reflectance * 25.0f, 0.0f, 1.0f);
    float3 R0 = specularColor;
    float3 R90 = f3(reflectance90, reflectance90, reflectance90);
    float3 l = norm3(lightDir);
    float3 h = norm3(l + v);
    float NdotL = clampf(dot3(n, l), 0.001f, 1.0f);
    float NdotV = clampf(fabsf(dot3(n, v)), 0.001f, 1.0f);
    float NdotH = clampf(dot3(n, h), 0.0f, 1.0f);
    float VdotH = clampf(dot3(v, h), 0.0f, 1.0f);
    float x = clampf(1.0f - VdotH, 0.0f, 1.0f);
    float x2 = x * x;
    float p5 = x2 * x2 * x;
    float3 F = R0 + (R90 - R0) * p5;
    float a2 = alphaRoughness * alphaRoughness;
    float attL = 2.0f * NdotL / (NdotL + sqrtf(a2 + (1.0f - a2) * (NdotL * NdotL)));
    float attV = 2.0f * NdotV / (NdotV + sqrtf(a2 + (1.0f - a2) * (NdotV * NdotV)));
    float G = attL * attV;
    float a = NdotH * alphaRoughness;
    float k = alphaRoughness / ((1.0f - NdotH * NdotH) + a * a);
    float D = clampf(k * k * (1.0f / pi), 0.0f, 4.0f);
    float3 diffuseContrib = (f3(1, 1, 1) - F) * diffuseColor * (1.0f / pi);
    float3 specContrib = F * (G * D / (4.0f * NdotL * NdotV));
    return lightColor * (diffuseContrib + specContrib) * NdotL;
}

// Front-face hit shading of src/shaders/closesthit.glsl:143-286 (NO_REFLECTION,
// no textures), split around the shadow query: `base` is emissive + specular
// bounce + diffuse bounce, `sun` the unshadowed sun term and `fade` the
// night fade (1 when the sun is above the horizon).  The shaded colour is
// base if the shadow ray hits, else (base + sun) * fade, which is the
// reference's `color += pbr; if (dir.y < 0) color *= fade`.
struct SurfaceShade {
    float3 base, sun, position;
    float fade;
};

// Geometry and material at a front-face hit (closesthit.glsl:143-190, no
// textures).
struct Surface {
    float3 position, normal, albedo, emissive;
    float metal, rough;
    uint32_t material;
};

__device__ __forceinline__ bool surface_at(const DeviceScene& sc, float3 origin, float3 dir, float t, float b1,
                                           float b2, uint32_t inst, uint32_t prim, Surface* s, uint32_t* err) {
    // hit position: product then sum, each rounded (shared with the shadow ray)
    s->position = f3(__fadd_rn(__fmul_rn(dir.x, t), origin.x), __fadd_rn(__fmul_rn(dir.y, t), origin.y),
                     __fadd_rn(__fmul_rn(dir.z, t), origin.z));
    const GpuInstance* gi = sc.instances_by_id + inst;
    uint32_t custom = __ldg(&gi->custom);
    ddgi_offset_entry oe = sc.offsets[custom];
    uint32_t io = oe.index_offset + 3u * prim;
    uint32_t i0 = __ldg(sc.indices + io), i1 = __ldg(sc.indices + io + 1), i2 = __ldg(sc.indices + io + 2);
    uint32_t vb = oe.vertex_offset;
    if (vb + max(i0, max(i1, i2)) >= sc.vertex_count || oe.material_index >= sc.material_count) {
        raise_error(err, DEV_BAD_INDEX);
        return false;
    }
    float4 n0 = __ldg(sc.normals + vb + i0), n1 = __ldg(sc.normals + vb + i1), n2 = __ldg(sc.normals + vb + i2);
    float b0 = 1.0f - b1 - b2;
    float3 tsn = norm3(f3(n0.x * b0 + n1.x * b1 + n2.x * b2, n0.y * b0 + n1.y * b1 + n2.y * b2,
                          n0.z * b0 + n1.z * b1 + n2.z * b2));
    float4 w0 = __ldg(&gi->w2o[0]), w1 = __ldg(&gi->w2o[1]), w2 = __ldg(&gi->w2o[2]);
    // normal * gl_WorldToObjectEXT: transpose of the world-to-object 3x3
    s->normal = norm3(f3(tsn.x * w0.x + tsn.y * w1.x + tsn.z * w2.x, tsn.x * w0.y + tsn.y * w1.y + tsn.z * w2.y,
                         tsn.x * w0.z + tsn.y * w1.z + tsn.z * w2.z));
    const ddgi_material& m = sc.materials[oe.material_index];
    s->albedo = f3(m.base_color[0], m.base_color[1], m.base_color[2]);
    s->emissive = f3(m.emissive[0], m.emissive[1], m.emissive[2]);
    s->metal = m.metallic;
    s->rough = m.roughness;
    s->material = oe.material_index;
    return true;
}

template <class AV>
__device__ __forceinline__ bool shade_surface(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L,
                                              const uint32_t* states, const AV& at, float3 origin, float3 dir,
                                              float t, float b1, float b2, uint32_t inst, uint32_t prim,
                                              SurfaceShade* out, uint32_t* err) {
    Surface s;
    if (!surface_at(sc, origin, dir, t, b1, b2, inst, prim, &s, err)) {
        out->position = s.position;
        out->base = out->sun = f3(0, 0, 0);
        out->fade = 1.0f;
        return false;
    }
    out->position = s.position;
    const float3 position = s.position, normal = s.normal, albedo = s.albedo;
    const float metal = s.metal, rough = s.rough;
    float3 color = s.emissive;
    float3 diffuseColor = albedo * (1.0f - 0.04f) * (1.0f - metal);
    float3 specularColor = mix3(f3(0.04f, 0.04f, 0.04f), albedo, metal);
    float3 reflectDir = dir - normal * (2.0f * dot3(normal, dir));
    const float3 lookups[2] = {reflectDir, normal};
    float3 sampled[2];  // reflection, indirect
    sample_probes_n<2>(position, lookups, -dir, g, states, at, sampled);
    color = color + specularColor * sampled[0];
    color = color + sampled[1] * diffuseColor;
    out->base = color;
    out->sun = pbr_metallic_roughness(normal, norm3(-dir), f3(L.color[0], L.color[1], L.color[2]),
                                      f3(L.dir[0], L.dir[1], L.dir[2]), albedo, metal, rough);
    out->fade = L.dir[1] < 0.0f ? 1.0f - clampf(-L.dir[1], 0.0f, 0.1f) / 0.1f : 1.0f;
    return true;
}

__device__ __forceinline__ float3 lit_color(const SurfaceShade& s) { return (s.base + s.sun) * s.fade; }

}  // namespace ddgi

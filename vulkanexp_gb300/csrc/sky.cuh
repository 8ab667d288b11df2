// sky.cuh — the atmospheric sky of the miss program, an optional mode
// (ddgi_set_sky_mode(DDGI_SKY_ATMOSPHERE)); the default is a constant sky
// radiance.
//
// src/shaders/sky.glsl:60-127 (single-scattering atmosphere after O'Neil,
// GPU Gems 2 ch. 16, "Accurate Atmospheric Scattering"), called by
// src/shaders/miss.rmiss:22 with the light's direction, colour and colour.a
// as brightness, showSun = true, and by src/shaders/FinalGather.frag:56 with
// brightness 1.  The planet's surface is 100 m below y = 0; its radius and
// the atmosphere's depth, the Rayleigh/Mie constants, the wavelengths and
// the 64 samples are the shader's.  Every addition, multiplication,
// division and square root is rounded separately (__fadd_rn, ...), as the
// CPU checker computes them, so the two agree to the exp/pow rounding.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace ddgi {
namespace sky {

constexpr float kPi = 3.1415926538f;  // common.glsl:4
constexpr float kInnerRadius = 100000.0f;
constexpr float kOuterRadius = 2500.0f + kInnerRadius;
constexpr float kDensityAltitude = 0.25f;
constexpr float kKr = 0.0025f, kKm = 0.0010f, kG = -0.990f;
constexpr uint32_t kSamples = 64;

__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float dv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
__device__ __forceinline__ float len3(float3 a) { return __fsqrt_rn(dot3(a, a)); }
__device__ __forceinline__ float3 sc3(float3 a, float s) { return f3(mul(a.x, s), mul(a.y, s), mul(a.z, s)); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return f3(add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return f3(sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)); }
__device__ __forceinline__ float3 nrm3(float3 a) {  // times the reciprocal length, as the shading code normalises
    const float inv = dv(1.0f, len3(a));
    return f3(mul(a.x, inv), mul(a.y, inv), mul(a.z, inv));
}

// traceSphereOutside around the origin (sky.glsl:14-31).
__device__ __forceinline__ float sphere_outside(float radius, float3 o, float3 d) {
    const float a = dot3(d, d), b = dot3(d, o), c = sub(dot3(o, o), mul(radius, radius));
    const float g = sub(mul(b, b), mul(a, c));
    if (g > 0.0f) {
        const float dis = dv(sub(-__fsqrt_rn(g), b), a);
        if (dis > 0.0f) return dis;
    }
    return -1.0f;
}

// traceSphereInside around the origin (sky.glsl:34-43).
__device__ __forceinline__ float sphere_inside(float radius, float3 o, float3 d) {
    const float3 oc = f3(-o.x, -o.y, -o.z);
    const float docdir = dot3(oc, d);
    const float3 pc = add3(o, sc3(d, docdir));
    const float lc = len3(pc);
    const float dist = __fsqrt_rn(sub(mul(radius, radius), mul(lc, lc)));
    const float lo = len3(sub3(pc, o));
    return docdir > 0.0f ? sub(dist, lo) : add(dist, lo);
}

// scale() of sky.glsl:45-49.
__device__ __forceinline__ float scale_fn(float c) {
    const float x = sub(1.0f, c);
    float p = add(-6.80f, mul(x, 5.25f));
    p = add(3.83f, mul(x, p));
    p = add(0.459f, mul(x, p));
    p = add(-0.00287f, mul(x, p));
    return mul(kDensityAltitude, expf(p));
}

// sky() with showSun = true.
static __device__ __noinline__ float3 atmosphere(float3 ray_origin, float3 ray_dir, float3 sun_pos, float3 sun_color,
                                          float brightness) {
    const float scale = dv(1.0f, sub(kOuterRadius, kInnerRadius));
    const float3 inv_wl = f3(dv(1.0f, powf(0.650f, 4.0f)), dv(1.0f, powf(0.570f, 4.0f)), dv(1.0f, powf(0.475f, 4.0f)));
    const float kr4pi = mul(mul(kKr, 4.0f), kPi), km4pi = mul(mul(kKm, 4.0f), kPi);
    sun_color = sc3(sun_color, brightness);
    float3 position = sub3(ray_origin, f3(0.0f, sub(-kInnerRadius, 100.0f), 0.0f));
    float height = len3(position);
    const float3 light_dir = nrm3(sun_pos);
    if (fabsf(sub(height, kInnerRadius)) < 1e-3f) {  // on the surface
        position = add3(position, sc3(nrm3(position), 1e-2f));
        height = len3(position);
    }
    if (height < kOuterRadius) {
        if (height > kInnerRadius) {
            const float pd = sphere_outside(kInnerRadius, position, ray_dir);
            if (pd >= 0.0f) {
                const float l = fmaxf(0.1f, dot3(light_dir, nrm3(add3(position, sc3(ray_dir, pd)))));
                return f3(mul(l, 0.05f), mul(l, 0.05f), mul(l, 0.05f));
            }
        } else {
            return f3(0.0f, 0.0f, 0.0f);
        }
        const float ray_depth = sphere_inside(kOuterRadius, position, ray_dir);
        if (isinf(ray_depth) || isnan(ray_depth)) return f3(0.0f, 0.0f, 0.0f);
        const float k = dv(scale, kDensityAltitude);
        const float depth = expf(mul(k, sub(kInnerRadius, height)));
        const float start_angle = dv(dot3(ray_dir, position), height);
        const float start_offset = mul(depth, scale_fn(start_angle));
        const float sample_len = dv(ray_depth, (float)kSamples);
        const float scaled_len = mul(sample_len, scale);
        const float3 sample_ray = sc3(ray_dir, sample_len);
        float3 p = add3(position, sc3(sample_ray, 0.5f));
        float3 color = f3(0.0f, 0.0f, 0.0f);
        for (uint32_t i = 0; i < kSamples; ++i) {
            const float h = len3(p);
            const float dep = expf(mul(k, sub(kInnerRadius, h)));
            const float light_angle = dv(dot3(light_dir, p), h);
            const float camera_angle = dv(dot3(ray_dir, p), h);
            const float scatter = add(start_offset, mul(dep, sub(scale_fn(light_angle), scale_fn(camera_angle))));
            const float3 att = f3(expf(mul(-scatter, add(mul(inv_wl.x, kr4pi), km4pi))),
                                  expf(mul(-scatter, add(mul(inv_wl.y, kr4pi), km4pi))),
                                  expf(mul(-scatter, add(mul(inv_wl.z, kr4pi), km4pi))));
            if (isinf(att.x) || isinf(att.y) || isinf(att.z) || isnan(att.x) || isnan(att.y) || isnan(att.z))
                continue;  // sky.glsl:103 (the sample point does not advance either)
            color = add3(color, sc3(att, mul(dep, scaled_len)));
            p = add3(p, sample_ray);
        }
        const float3 secondary = f3(mul(mul(color.x, kKm), sun_color.x), mul(mul(color.y, kKm), sun_color.y),
                                    mul(mul(color.z, kKm), sun_color.z));
        color = f3(mul(color.x, mul(mul(inv_wl.x, kKr), sun_color.x)), mul(color.y, mul(mul(inv_wl.y, kKr), sun_color.y)),
                   mul(color.z, mul(mul(inv_wl.z, kKr), sun_color.z)));
        const float mie_cos = dot3(light_dir, f3(-ray_dir.x, -ray_dir.y, -ray_dir.z));
        const float g2 = mul(kG, kG);
        const float num = mul(mul(1.5f, dv(sub(1.0f, g2), add(2.0f, g2))), add(1.0f, mul(mie_cos, mie_cos)));
        const float den = powf(fmaxf(1e-3f, sub(add(1.0f, g2), mul(mul(2.0f, kG), mie_cos))), 1.5f);
        const float phase = dv(num, den);
        color = add3(color, sc3(secondary, phase));
        if (!(isinf(color.x) || isinf(color.y) || isinf(color.z))) return color;
    } else {
        const float d = sphere_outside(kOuterRadius, position, ray_dir);
        if (d > 0.0f) {
            const float l = mul(dot3(light_dir, nrm3(add3(position, sc3(ray_dir, d)))), 0.5f);
            return f3(mul(l, 0.5294117647f), mul(l, 0.80784313725f), mul(l, 0.92156862745f));
        }
    }
    return f3(0.0f, 0.0f, 0.0f);
}

}  // namespace sky
}  // namespace ddgi

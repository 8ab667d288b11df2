// glsl_rt.hpp — what the reference's probe-trace ray-tracing shaders
// (src/shaders/traceProbes.rgen, closesthit_noreflection.rchit through
// closesthit.glsl, miss.rmiss, shadow.rmiss; the pipeline of
// src/IrradianceProbes.cpp:205-262) need beyond glsl_compute.hpp to run on
// the host: the ray-tracing built-ins, ray payloads passed between stages,
// hit attributes and traceRayEXT.  Test infrastructure: built by
// oracle/build_ref_glsl.py into oracle/_ref/, loaded only by tests and the
// fixture generator.
//
// traceRayEXT finds the hit through a traversal function the caller
// supplies (the shaders hand that job to the Vulkan implementation, whose
// acceleration structures are not part of the reference's code), then runs
// the stages of the reference's shader binding table on it: the closest-hit
// stage for a hit (unless gl_RayFlagsSkipClosestHitShaderEXT), miss stage
// `missIndex` for a miss.  The pipeline has no any-hit stage, so every
// triangle is opaque.  Built-ins of the calling stage are saved and restored
// around a nested call.  Payloads are copied into the callee's
// rayPayloadInEXT variable and back, as the stages share them by location.
#pragma once

#include <stdint.h>
#include <string.h>

#include "glsl_compute.hpp"

namespace glsl {

struct accelerationStructureEXT {};

const uint gl_RayFlagsNoneEXT = 0u;
const uint gl_RayFlagsOpaqueEXT = 1u;
const uint gl_RayFlagsNoOpaqueEXT = 2u;
const uint gl_RayFlagsTerminateOnFirstHitEXT = 4u;
const uint gl_RayFlagsSkipClosestHitShaderEXT = 8u;
const uint gl_HitKindFrontFacingTriangleEXT = 0xFEu;
const uint gl_HitKindBackFacingTriangleEXT = 0xFFu;

// Not reached on the probe path's scenes (no material has a texture).
inline vec4 textureGrad(const sampler2D& s, const vec2& uv, const vec2&, const vec2&) {
    return s.texels ? textureLod(s, uv, 0.0f) : vec4(1.0f);
}
inline vec4 texture(const sampler2D& s, const vec2& uv) { return textureGrad(s, uv, vec2(), vec2()); }

// One closest hit (or, for a query that ends at the first hit, any hit) as
// the traversal reports it; instance ~0u = miss.
struct RtHit {
    uint32_t instance, primitive;
    float t;
    uint32_t backface;
};
// Traversal: n rays from origins/dirs (3 floats each) over [tmin, tmax]
// against instances whose mask shares a bit with `mask`; any_hit != 0 ends
// at the first hit.  Barycentrics (u, v) of each hit into bary.
typedef void (*RtTraverse)(const void* ctx, const float* origins, const float* dirs, uint32_t n, float tmin,
                           float tmax, uint32_t mask, int any_hit, RtHit* out, float* bary, int nthreads);

struct RtScene {
    const void* ctx;
    RtTraverse traverse;
    const float* object_to_world;  // 12 floats per instance, row-major 3x4
    const float* world_to_object;  // 12 floats per instance, row-major 3x4
    const uint32_t* custom_index;  // per instance
};
inline RtScene g_rt_scene;

typedef void (*RtStage)(void* payload);
inline RtStage g_rt_miss[2] = {nullptr, nullptr};
inline RtStage g_rt_closest_hit = nullptr;

struct RtBuiltins {
    uvec3 launch_id, launch_size;
    vec3 world_origin, world_direction;
    float tmin, tmax, hit_t;
    uint hit_kind;
    int custom_index, primitive_id, instance_id;
    mat4x3 object_to_world, world_to_object;
    vec2 bary;
};
inline thread_local RtBuiltins rt_builtins;
inline thread_local int rt_depth = 0;
inline thread_local float* rt_record = nullptr;  // the launch's first traceRayEXT arguments

#define gl_LaunchIDEXT (::glsl::rt_builtins.launch_id)
#define gl_LaunchSizeEXT (::glsl::rt_builtins.launch_size)
#define gl_WorldRayOriginEXT (::glsl::rt_builtins.world_origin)
#define gl_WorldRayDirectionEXT (::glsl::rt_builtins.world_direction)
#define gl_RayTminEXT (::glsl::rt_builtins.tmin)
#define gl_RayTmaxEXT (::glsl::rt_builtins.tmax)
#define gl_HitTEXT (::glsl::rt_builtins.hit_t)
#define gl_HitKindEXT (::glsl::rt_builtins.hit_kind)
#define gl_InstanceCustomIndexEXT (::glsl::rt_builtins.custom_index)
#define gl_InstanceID (::glsl::rt_builtins.instance_id)
#define gl_PrimitiveID (::glsl::rt_builtins.primitive_id)
#define gl_ObjectToWorldEXT (::glsl::rt_builtins.object_to_world)
#define gl_WorldToObjectEXT (::glsl::rt_builtins.world_to_object)

inline mat4x3 rt_matrix(const float* m) {  // row-major 3x4 -> 4 columns of 3
    mat4x3 r;
    for (int c = 0; c < 4; ++c) r.c[c] = vec3(m[c], m[4 + c], m[8 + c]);
    return r;
}

inline void rt_trace(uint flags, uint mask, uint miss_index, const vec3& origin, float tmin, const vec3& dir,
                     float tmax, void* payload) {
    if (rt_depth == 0 && rt_record) {
        const float rec[8] = {origin.x, origin.y, origin.z, dir.x, dir.y, dir.z, tmin, tmax};
        memcpy(rt_record, rec, sizeof(rec));
    }
    const RtBuiltins saved = rt_builtins;
    ++rt_depth;
    const float o[3] = {origin.x, origin.y, origin.z}, d[3] = {dir.x, dir.y, dir.z};
    RtHit h;
    float bary[2] = {0.0f, 0.0f};
    g_rt_scene.traverse(g_rt_scene.ctx, o, d, 1, tmin, tmax, mask & 0xFFu,
                        (flags & gl_RayFlagsTerminateOnFirstHitEXT) ? 1 : 0, &h, bary, 1);
    rt_builtins.world_origin = origin;
    rt_builtins.world_direction = dir;
    rt_builtins.tmin = tmin;
    rt_builtins.tmax = tmax;
    if (h.instance == 0xFFFFFFFFu) {
        g_rt_miss[miss_index](payload);
    } else if (!(flags & gl_RayFlagsSkipClosestHitShaderEXT)) {
        rt_builtins.hit_t = h.t;
        rt_builtins.hit_kind = h.backface ? gl_HitKindBackFacingTriangleEXT : gl_HitKindFrontFacingTriangleEXT;
        rt_builtins.instance_id = (int)h.instance;
        rt_builtins.custom_index = (int)g_rt_scene.custom_index[h.instance];
        rt_builtins.primitive_id = (int)h.primitive;
        rt_builtins.object_to_world = rt_matrix(g_rt_scene.object_to_world + 12 * (size_t)h.instance);
        rt_builtins.world_to_object = rt_matrix(g_rt_scene.world_to_object + 12 * (size_t)h.instance);
        rt_builtins.bary = vec2(bary[0], bary[1]);
        g_rt_closest_hit(payload);
    }
    --rt_depth;
    rt_builtins = saved;
}

}  // namespace glsl

// Declarations of a stage's ray-tracing variables, as build_ref_glsl.py
// rewrites them; each stage's unit defines rt_payload_slot[] before
// including its shader.
//   layout(location = L) rayPayloadEXT T name;  -> RT_PAYLOAD(L, T, name)
//   layout(location = L) rayPayloadInEXT T name; -> RT_PAYLOAD_IN(L, T, name)
//   hitAttributeEXT T name;                       -> RT_HIT_ATTRIBUTE(T, name)
#define RT_PAYLOAD(loc, T, name) \
    thread_local T name;         \
    const bool rt_reg_##name = (rt_payload_slot[loc] = [] { return (void*)&name; }, true);
#define RT_PAYLOAD_IN(loc, T, name)                      \
    thread_local T name;                                 \
    void* rt_incoming() { return (void*)&name; }         \
    const size_t rt_incoming_bytes = sizeof(T);
#define RT_HIT_ATTRIBUTE(T, name) \
    thread_local T name;          \
    void rt_set_hit_attribute() { name = ::glsl::rt_builtins.bary; }

// A stage's traceRayEXT: the payload at `location` of the calling stage.
#define RT_STAGE_PROLOGUE                                                                                         \
    void* (*rt_payload_slot[4])() = {nullptr, nullptr, nullptr, nullptr};                                         \
    void traceRayEXT(const accelerationStructureEXT&, uint flags, uint mask, uint, uint, uint miss_index,        \
                     const vec3& origin, float tmin, const vec3& dir, float tmax, int location) {                 \
        rt_trace(flags, mask, miss_index, origin, tmin, dir, tmax, rt_payload_slot[location]());                  \
    }

// A called stage's entry: payload in, main(), payload out.
#define RT_STAGE_ENTRY(fn, set_attribute)                    \
    void fn(void* payload) {                                 \
        using namespace glsl;                                \
        memcpy(rt_incoming(), payload, rt_incoming_bytes);   \
        set_attribute;                                       \
        main();                                              \
        memcpy(payload, rt_incoming(), rt_incoming_bytes);   \
    }

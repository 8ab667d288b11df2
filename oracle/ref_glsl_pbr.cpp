// ref_glsl_pbr.cpp — the reference's src/shaders/pbrMetallicRoughness.glsl
// (with common.glsl) compiled as C++ over glsl_shim.hpp.  Test
// infrastructure: built by oracle/build_ref_glsl.py into oracle/_ref/.
#include "glsl_shim.hpp"

namespace glsl {
namespace {  // internal linkage: common.glsl is in every unit
#define in  // the GLSL parameter qualifier (by value here)
#include "pbrMetallicRoughness.glsl"
#undef in
}  // namespace
}  // namespace glsl

extern "C" void ref_pbr(const float* n, const float* v, const float* light_color, const float* light_dir,
                        const float* albedo4, float metalness, float roughness, float* out4) {
    const glsl::vec4 c = glsl::pbrMetallicRoughness(
        glsl::vec3(n[0], n[1], n[2]), glsl::vec3(v[0], v[1], v[2]),
        glsl::vec3(light_color[0], light_color[1], light_color[2]), glsl::vec3(light_dir[0], light_dir[1], light_dir[2]),
        glsl::vec4(albedo4[0], albedo4[1], albedo4[2], albedo4[3]), metalness, roughness);
    out4[0] = c.x, out4[1] = c.y, out4[2] = c.z, out4[3] = c.w;
}

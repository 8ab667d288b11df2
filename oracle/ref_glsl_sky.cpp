// ref_glsl_sky.cpp — the reference's src/shaders/sky.glsl compiled as C++
// over glsl_shim.hpp, after common.glsl (which defines pi for it, as in the
// miss shader).  Test infrastructure: built by oracle/build_ref_glsl.py into
// oracle/_ref/.
#include "glsl_shim.hpp"

namespace glsl {
namespace {  // internal linkage: common.glsl is in every unit
#define in  // the GLSL parameter qualifier (by value here)
#include "common.glsl"
#include "sky.glsl"
#undef in
}  // namespace
}  // namespace glsl

extern "C" void ref_sky(const float* origin, const float* dir, const float* sun_pos, const float* sun_color,
                        float brightness, int show_sun, float* out3) {
    const glsl::vec3 c =
        glsl::sky(glsl::vec3(origin[0], origin[1], origin[2]), glsl::vec3(dir[0], dir[1], dir[2]),
                  glsl::vec3(sun_pos[0], sun_pos[1], sun_pos[2]), glsl::vec3(sun_color[0], sun_color[1], sun_color[2]),
                  brightness, show_sun != 0);
    out3[0] = c.x, out3[1] = c.y, out3[2] = c.z;
}

// ref_glsl_miss.cpp — the reference's miss stages of the probe trace,
// src/shaders/miss.rmiss (the sky) and shadow.rmiss, compiled as C++ over
// glsl_rt.hpp.  Test infrastructure: built by oracle/build_ref_glsl.py from
// the reference's files into oracle/_ref/.
#include "glsl_rt.hpp"
#include "ref_glsl_trace.h"

namespace glsl {
namespace miss {
namespace {
RT_STAGE_PROLOGUE
#define in  // the GLSL parameter qualifier (by value here)
#include "miss.rmiss"
#undef in
}  // namespace
}  // namespace miss
namespace shadow_miss {
namespace {
RT_STAGE_PROLOGUE
#include "shadow.rmiss"
}  // namespace
}  // namespace shadow_miss
}  // namespace glsl

namespace glsl_stages {

void bind_miss(const RefTraceInputs& r) {
    using namespace glsl::miss;
    DirectionalLight.direction =
        glsl::vec4(r.light_direction[0], r.light_direction[1], r.light_direction[2], r.light_direction[3]);
    DirectionalLight.color = glsl::vec4(r.light_color[0], r.light_color[1], r.light_color[2], r.light_color[3]);
}

void entry_miss(void* payload) {
    using namespace glsl::miss;
    memcpy(rt_incoming(), payload, rt_incoming_bytes);
    glsl::miss::main();
    memcpy(payload, rt_incoming(), rt_incoming_bytes);
}

void entry_shadow_miss(void* payload) {
    using namespace glsl::shadow_miss;
    memcpy(rt_incoming(), payload, rt_incoming_bytes);
    glsl::shadow_miss::main();
    memcpy(payload, rt_incoming(), rt_incoming_bytes);
}

}  // namespace glsl_stages

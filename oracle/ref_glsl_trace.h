// ref_glsl_trace.h — the resources the reference's probe-trace stages read
// (the descriptor set of src/IrradianceProbes.cpp and RaytracingDescriptors),
// handed to each stage's unit of oracle/ref_glsl_*.cpp.  Test
// infrastructure: built by oracle/build_ref_glsl.py into oracle/_ref/.
#pragma once

#include <stdint.h>

#include "../include/ddgi.h"

struct RefTraceInputs {
    const ddgi_grid_desc* grid;
    float light_direction[4], light_color[4];  // LightBuffer: direction, colour (a = sky brightness)
    const float* vertices;                     // 16 floats per vertex (4 vec4, Vertex.glsl)
    const uint32_t* indices;
    const uint32_t* offsets;    // material, vertex offset, index offset per instance custom index
    const uint32_t* materials;  // 12 words per material (unpackMaterial.glsl)
    uint32_t* states;           // probe states
    const float* color;         // previous colour atlas, 4 floats per texel
    const float* depth;         // previous depth atlas, 2 floats per texel
};

namespace glsl_stages {
void bind_closest_hit(const RefTraceInputs& in);
void bind_miss(const RefTraceInputs& in);
void entry_closest_hit(void* payload);
void entry_miss(void* payload);
void entry_shadow_miss(void* payload);
}  // namespace glsl_stages

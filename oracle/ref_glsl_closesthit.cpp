// ref_glsl_closesthit.cpp — the reference's closest-hit stage of the probe
// trace, src/shaders/closesthit_noreflection.rchit (closesthit.glsl with
// NO_REFLECTION), compiled as C++ over glsl_rt.hpp.  Test infrastructure:
// built by oracle/build_ref_glsl.py from the reference's files into
// oracle/_ref/.
#include "glsl_rt.hpp"
#include "ref_glsl_trace.h"

namespace glsl {
namespace {  // internal linkage: each stage is its own unit
RT_STAGE_PROLOGUE
#define in  // the GLSL parameter qualifier (by value here)
#include "closesthit_noreflection.rchit"
#undef in
}  // namespace
}  // namespace glsl

namespace glsl_stages {

void bind_closest_hit(const RefTraceInputs& r) {
    using namespace glsl;
    const ddgi_grid_desc* d = r.grid;
    grid = make_probe_grid<ProbeGrid>(d);
    Probes = r.states;
    Vertices = reinterpret_cast<vec4*>(const_cast<float*>(r.vertices));
    indices.i = const_cast<uint*>(r.indices);
    offsets.o = const_cast<uint*>(r.offsets);
    Materials = const_cast<uint*>(r.materials);
    textures = nullptr;
    const int r01 = (int)d->resolution[0] * (int)d->resolution[1], r2 = (int)d->resolution[2];
    irradianceColor = sampler2D{r.color, (int)d->color_res * r01, (int)d->color_res * r2, 4};
    irradianceDepth = sampler2D{r.depth, (int)d->depth_res * r01, (int)d->depth_res * r2, 2};
    DirectionalLight.direction =
        vec4(r.light_direction[0], r.light_direction[1], r.light_direction[2], r.light_direction[3]);
    DirectionalLight.color = vec4(r.light_color[0], r.light_color[1], r.light_color[2], r.light_color[3]);
}

RT_STAGE_ENTRY(entry_closest_hit, rt_set_hit_attribute())

}  // namespace glsl_stages

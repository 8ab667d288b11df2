// ref_glsl_irradiance.cpp — the reference's src/shaders/irradiance.glsl
// (with common.glsl and ProbeGrid.glsl) compiled as C++ over glsl_shim.hpp,
// exported for the checks of the oracle's restatements.  Test
// infrastructure: built by oracle/build_ref_glsl.py from the reference's
// files into oracle/_ref/.
#include <stdint.h>

#include "../include/ddgi.h"
#include "glsl_shim.hpp"

namespace glsl {
namespace {  // internal linkage: common.glsl is in every unit
// the probe-state buffer sampleProbes reads (closesthit.glsl:19's Probes[])
static uint* Probes = nullptr;
#define in  // the GLSL parameter qualifier (by value here)
#include "irradiance.glsl"
#undef in
}  // namespace
}  // namespace glsl

namespace {
glsl::ProbeGrid to_grid(const ddgi_grid_desc* d) {
    glsl::ProbeGrid g;
    g.extentMin = glsl::vec3(d->extent_min[0], d->extent_min[1], d->extent_min[2]);
    g.depthSharpness = d->depth_sharpness;
    g.extentMax = glsl::vec3(d->extent_max[0], d->extent_max[1], d->extent_max[2]);
    g.hysteresis = d->hysteresis;
    g.resolution = glsl::ivec3((int)d->resolution[0], (int)d->resolution[1], (int)d->resolution[2]);
    g.raysPerProbe = d->rays_per_probe;
    g.colorRes = d->color_res;
    g.depthRes = d->depth_res;
    g.shadowBias = d->shadow_bias;
    g.padding[0] = 0;
    return g;
}
}  // namespace

extern "C" {

void ref_spherical_fibonacci(float i, float n, float* out3) {
    const glsl::vec3 v = glsl::sphericalFibonacci(i, n);
    out3[0] = v.x, out3[1] = v.y, out3[2] = v.z;
}

void ref_oct_encode(const float* v3, float* out2) {
    const glsl::vec2 o = glsl::octEncode(glsl::vec3(v3[0], v3[1], v3[2]));
    out2[0] = o.x, out2[1] = o.y;
}

void ref_oct_decode(float x, float y, float* out3) {
    const glsl::vec3 v = glsl::octDecode(glsl::vec2(x, y));
    out3[0] = v.x, out3[1] = v.y, out3[2] = v.z;
}

void ref_sphere_to_oct_uv(const float* d3, float* out2) {
    const glsl::vec2 uv = glsl::spherePointToOctohedralUV(glsl::vec3(d3[0], d3[1], d3[2]));
    out2[0] = uv.x, out2[1] = uv.y;
}

void ref_probe_world_position(const ddgi_grid_desc* d, uint32_t index, float* out3) {
    const glsl::vec3 p = glsl::probeIndexToWorldPosition((glsl::uint)index, to_grid(d));
    out3[0] = p.x, out3[1] = p.y, out3[2] = p.z;
}

// sampleProbes over row-major atlases (colour 4 floats, depth 2 floats per
// texel) of the grid's sizes.
void ref_sample_probes(const ddgi_grid_desc* d, const uint32_t* states, const float* color, const float* depth,
                       const float* pos, const float* nrm, const float* view, float* out3) {
    const glsl::ProbeGrid g = to_grid(d);
    const int cw = (int)(d->color_res * d->resolution[0] * d->resolution[1]), ch = (int)(d->color_res * d->resolution[2]);
    const int dw = (int)(d->depth_res * d->resolution[0] * d->resolution[1]), dh = (int)(d->depth_res * d->resolution[2]);
    glsl::Probes = const_cast<glsl::uint*>(states);
    const glsl::sampler2D ctex{color, cw, ch, 4}, dtex{depth, dw, dh, 2};
    const glsl::vec3 c = glsl::sampleProbes(glsl::vec3(pos[0], pos[1], pos[2]), glsl::vec3(nrm[0], nrm[1], nrm[2]),
                                            glsl::vec3(view[0], view[1], view[2]), g, ctex, dtex);
    out3[0] = c.x, out3[1] = c.y, out3[2] = c.z;
}

}  // extern "C"

// ref_glsl_copy_borders.cpp — the reference's border copy
// (src/shaders/probesCopyBorders.comp) compiled as C++ over
// glsl_compute.hpp, and the whole reference update after the trace in
// IrradianceProbes::update's order (src/IrradianceProbes.cpp:514-529):
// irradiance pass, depth pass, border copy.  Test infrastructure: built by
// oracle/build_ref_glsl.py from the reference's files into oracle/_ref/.
#include <stdint.h>

#include <vector>

#include "../include/ddgi.h"
#include "glsl_compute.hpp"

namespace glsl {
namespace {  // internal linkage: each pass is its own unit
#define in   // the GLSL parameter qualifier (by value here)
#include "probesCopyBorders.comp"
#undef in
}  // namespace
}  // namespace glsl

extern "C" {

void ref_update_irradiance(const ddgi_grid_desc* d, const uint32_t* list, uint32_t count, uint32_t* states,
                           float* rays, int ray_columns, float* dirs, float* atlas);
void ref_update_depth(const ddgi_grid_desc* d, const uint32_t* list, uint32_t count, uint32_t* states, float* rays,
                      int ray_columns, float* dirs, float* atlas);

// color: 4 floats per texel, depth: 2 floats per texel (row-major atlases of
// the grid's sizes).
void ref_copy_borders(const ddgi_grid_desc* d, const uint32_t* list, uint32_t count, uint32_t* states, float* color,
                      float* depth) {
    using namespace glsl;
    grid = make_probe_grid<ProbeGrid>(d);
    Probes = states;
    indices = const_cast<uint*>(list);
    const int r01 = (int)d->resolution[0] * (int)d->resolution[1], r2 = (int)d->resolution[2];
    bind_image(irradiance, color, (int)d->color_res * r01, (int)d->color_res * r2, 4);
    bind_image(glsl::depth, depth, (int)d->depth_res * r01, (int)d->depth_res * r2, 2);
    dispatch(count, gl_WorkGroupSize, &glsl::main);
}

// The reference's update of the listed probes from traced rays: rays holds
// raysPerProbe records (r, g, b, hit distance) per listed probe, dirs the
// raysPerProbe directions (x, y, z, w) the trace used.  The ray images are
// laid out as the reference's (column = position in the list, row = ray).
void ref_probes_update(const ddgi_grid_desc* d, const uint32_t* list, uint32_t count, const float* rays,
                       const float* dirs, uint32_t* states, float* color, float* depth) {
    const uint32_t R = d->rays_per_probe;
    std::vector<float> img((size_t)count * R * 4), dimg(dirs, dirs + (size_t)R * 4);
    for (uint32_t s = 0; s < count; ++s)
        for (uint32_t i = 0; i < R; ++i)
            for (int c = 0; c < 4; ++c) img[((size_t)i * count + s) * 4 + c] = rays[((size_t)s * R + i) * 4 + c];
    ref_update_irradiance(d, list, count, states, img.data(), (int)count, dimg.data(), color);
    ref_update_depth(d, list, count, states, img.data(), (int)count, dimg.data(), depth);
    ref_copy_borders(d, list, count, states, color, depth);
}

}  // extern "C"

// ref_glsl_final_gather.cpp — the reference's final gather, the atlas's
// consumer: src/shaders/FinalGather.frag compiled as C++ over
// glsl_compute.hpp and run once per pixel, the G-buffer subpass inputs read
// at the pixel and fragPosition at its centre.  Test infrastructure: built
// by oracle/build_ref_glsl.py from the reference's files into oracle/_ref/.
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "../include/ddgi.h"
#include "glsl_rt.hpp"

namespace glsl {
namespace final_gather {
namespace {
#define in  // the GLSL parameter qualifier (by value here)
#include "FinalGather.frag"
#undef in
}  // namespace
}  // namespace final_gather
}  // namespace glsl

extern "C" {

// width x height pixels, row-major; every G-buffer input 4 floats per pixel
// (position + depth, normal + metalness, albedo + roughness, emissive,
// direct light in .r); reflection: the reflection image (4 floats per
// pixel); view, proj: column-major 4x4; light: direction and colour (4 each);
// atlases: colour 4 floats, depth 2 floats per texel.  out: 4 floats per
// pixel.
void ref_final_gather(const ddgi_grid_desc* d, const float* light_direction4, const float* light_color4,
                      const uint32_t* states, const float* color, const float* depth, int width, int height,
                      const float* position_depth, const float* normal_metalness, const float* albedo_roughness,
                      const float* emissive, const float* direct_light, const float* reflection, const float* view,
                      const float* proj, float* out, int nthreads) {
    using namespace glsl;
    using namespace glsl::final_gather;
    grid = make_probe_grid<ProbeGrid>(d);
    Probes = const_cast<uint*>(states);
    const int r01 = (int)d->resolution[0] * (int)d->resolution[1], r2 = (int)d->resolution[2];
    irradianceColor = sampler2D{color, (int)d->color_res * r01, (int)d->color_res * r2, 4};
    irradianceDepth = sampler2D{depth, (int)d->depth_res * r01, (int)d->depth_res * r2, 2};
    inputReflection = sampler2D{reflection, width, height, 4};
    inputPositionDepth.texels = position_depth;
    inputNormalMetalness.texels = normal_metalness;
    inputAlbedoRoughness.texels = albedo_roughness;
    inputEmissive.texels = emissive;
    inputDirectLight.texels = direct_light;
    DirectionalLight.direction = vec4(light_direction4[0], light_direction4[1], light_direction4[2], light_direction4[3]);
    DirectionalLight.color = vec4(light_color4[0], light_color4[1], light_color4[2], light_color4[3]);
    for (int c = 0; c < 4; ++c) {
        ubo.view.c[c] = vec4(view[4 * c], view[4 * c + 1], view[4 * c + 2], view[4 * c + 3]);
        ubo.proj.c[c] = vec4(proj[4 * c], proj[4 * c + 1], proj[4 * c + 2], proj[4 * c + 3]);
    }
    const size_t pixels = (size_t)width * height;
    std::atomic<size_t> next{0};
    auto worker = [&] {
        for (;;) {
            const size_t p = next.fetch_add(1);
            if (p >= pixels) break;
            gl_current_pixel = p;
            fragPosition = vec2(((float)(p % width) + 0.5f) / (float)width, ((float)(p / width) + 0.5f) / (float)height);
            final_gather::main();
            out[4 * p] = glsl::final_gather::color.x;
            out[4 * p + 1] = glsl::final_gather::color.y;
            out[4 * p + 2] = glsl::final_gather::color.z;
            out[4 * p + 3] = glsl::final_gather::color.w;
        }
    };
    const int nt = std::max(1, std::min(nthreads, 64));
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
}

}  // extern "C"

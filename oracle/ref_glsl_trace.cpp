// ref_glsl_trace.cpp — the reference's probe trace run on the host: the
// ray-generation stage src/shaders/traceProbes.rgen compiled as C++ over
// glsl_rt.hpp, launched over (listed probes x raysPerProbe) as
// IrradianceProbes::update does (src/IrradianceProbes.cpp:486-487), with
// the pipeline's shader binding table (src/IrradianceProbes.cpp:205-262):
// miss 0 = miss.rmiss, miss 1 = shadow.rmiss, hit group 0 =
// closesthit_noreflection.rchit, no any-hit stage.  Test infrastructure:
// built by oracle/build_ref_glsl.py from the reference's files into
// oracle/_ref/.
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "../include/ddgi_exact.h"
#include "glsl_rt.hpp"
#include "ref_glsl_trace.h"

namespace glsl {
namespace {  // internal linkage: each stage is its own unit
RT_STAGE_PROLOGUE
#define in  // the GLSL parameter qualifier (by value here)
#include "traceProbes.rgen"
#undef in
}  // namespace
}  // namespace glsl

extern "C" {

// The reference's trace + shade of the listed probes' rays.  orientation:
// the row-major 3x3 rotation M of the update (the push constant's mat4 holds
// it as columns); instances: the scene's ddgi_instance records;
// traverse/traverse_ctx: the traversal (see glsl_rt.hpp).  Outputs, per
// listed probe s and ray i: rays[(s R + i) 4 ...] = the ray-result image's
// texel (r, g, b, hit distance); records[(s R + i) 8 ...] = the arguments of
// the stage's traceRayEXT (origin, direction, tmin, tmax); dirs[4 i ...] =
// the ray-direction image's row i (written by the launch whose probe
// position equals i, so rows i >= count stay as given).
void ref_trace_probes(const ddgi_grid_desc* d, const float* light_direction4, const float* light_color4,
                      const float* vertices, const uint32_t* indices, const uint32_t* offsets,
                      const uint32_t* materials, const ddgi_instance* instances, uint32_t instance_count,
                      uint32_t* states, const float* color, const float* depth, const float orientation[9],
                      const uint32_t* list, uint32_t count, glsl::RtTraverse traverse, const void* traverse_ctx,
                      float* rays, float* records, float* dirs, int nthreads) {
    using namespace glsl;
    RefTraceInputs in{};
    in.grid = d;
    for (int k = 0; k < 4; ++k) in.light_direction[k] = light_direction4[k], in.light_color[k] = light_color4[k];
    in.vertices = vertices;
    in.indices = indices;
    in.offsets = offsets;
    in.materials = materials;
    in.states = states;
    in.color = color;
    in.depth = depth;
    glsl_stages::bind_closest_hit(in);
    glsl_stages::bind_miss(in);

    std::vector<float> o2w(12 * (size_t)instance_count), w2o(12 * (size_t)instance_count);
    std::vector<uint32_t> custom(instance_count);
    for (uint32_t i = 0; i < instance_count; ++i) {
        memcpy(&o2w[12 * (size_t)i], instances[i].transform, 12 * sizeof(float));
        if (!ddgi_affine_inverse(instances[i].transform, &w2o[12 * (size_t)i]))
            memset(&w2o[12 * (size_t)i], 0, 12 * sizeof(float));
        custom[i] = instances[i].custom_index & 0xFFFFFFu;
    }
    g_rt_scene = RtScene{traverse_ctx, traverse, o2w.data(), w2o.data(), custom.data()};
    g_rt_miss[0] = &glsl_stages::entry_miss;
    g_rt_miss[1] = &glsl_stages::entry_shadow_miss;
    g_rt_closest_hit = &glsl_stages::entry_closest_hit;

    const uint32_t R = d->rays_per_probe;
    grid = make_probe_grid<ProbeGrid>(d);
    Probes = states;
    glsl::indices = const_cast<uint*>(list);
    for (int c = 0; c < 4; ++c)
        push.randomOrientation.c[c] =
            c < 3 ? vec4(orientation[c], orientation[3 + c], orientation[6 + c], 0.0f) : vec4(0.0f, 0.0f, 0.0f, 1.0f);
    std::vector<float> image((size_t)count * R * 4, 0.0f);
    bind_image(rayIrradianceDepth, image.data(), (int)count, (int)R, 4);
    bind_image(rayDirection, dirs, 1, (int)R, 4);

    const size_t launches = (size_t)count * R;
    std::atomic<size_t> next{0};
    auto worker = [&] {
        for (;;) {
            const size_t k = next.fetch_add(1);
            if (k >= launches) break;
            const uint32_t x = (uint32_t)(k / R), y = (uint32_t)(k % R);
            rt_builtins = RtBuiltins{};
            rt_builtins.launch_id = uvec3(x, y, 0u);
            rt_builtins.launch_size = uvec3(count, R, 1u);
            rt_record = records + 8 * k;
            glsl::main();
            rt_record = nullptr;
        }
    };
    const int nt = std::max(1, std::min(nthreads, 64));
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
    for (uint32_t s = 0; s < count; ++s)
        for (uint32_t i = 0; i < R; ++i)
            memcpy(rays + ((size_t)s * R + i) * 4, &image[((size_t)i * count + s) * 4], 4 * sizeof(float));
}

}  // extern "C"

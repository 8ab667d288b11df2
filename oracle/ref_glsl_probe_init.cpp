// ref_glsl_probe_init.cpp — the reference's probe classification run on the
// host: src/shaders/probesInit.rgen compiled as C++ over glsl_rt.hpp with
// the init pipeline's shader binding table (src/IrradianceProbes.cpp:
// 155-200): miss 0 = probeInitMiss.rmiss, hit group 0 = backfaceTest.rchit,
// launched over the probe grid.  Test infrastructure: built by
// oracle/build_ref_glsl.py from the reference's files into oracle/_ref/.
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "../include/ddgi.h"
#include "../include/ddgi_exact.h"
#include "glsl_rt.hpp"

namespace glsl {
namespace probe_init {
namespace {
RT_STAGE_PROLOGUE
#define in  // the GLSL parameter qualifier (by value here)
#include "probesInit.rgen"
#undef in
}  // namespace
}  // namespace probe_init
namespace probe_init_miss {
namespace {
RT_STAGE_PROLOGUE
#include "probeInitMiss.rmiss"
}  // namespace
}  // namespace probe_init_miss
namespace backface_test {
namespace {
RT_STAGE_PROLOGUE
#include "backfaceTest.rchit"
}  // namespace
}  // namespace backface_test
}  // namespace glsl

namespace {
void entry_init_miss(void* payload) {
    using namespace glsl::probe_init_miss;
    memcpy(rt_incoming(), payload, rt_incoming_bytes);
    glsl::probe_init_miss::main();
    memcpy(payload, rt_incoming(), rt_incoming_bytes);
}
void entry_backface_test(void* payload) {
    using namespace glsl::backface_test;
    memcpy(rt_incoming(), payload, rt_incoming_bytes);
    glsl::backface_test::main();
    memcpy(payload, rt_incoming(), rt_incoming_bytes);
}
}  // namespace

extern "C" {

// The reference's probe classification of every probe of the grid: states
// receives 0 (off), 1 (near geometry) or 8 per probe.  orientation: the
// row-major 3x3 rotation of the push constant; instances and traverse as
// for ref_trace_probes.
void ref_init_probes(const ddgi_grid_desc* d, const ddgi_instance* instances, uint32_t instance_count,
                     const float orientation[9], glsl::RtTraverse traverse, const void* traverse_ctx, uint32_t* states,
                     int nthreads) {
    using namespace glsl;
    std::vector<float> o2w(12 * (size_t)instance_count), w2o(12 * (size_t)instance_count);
    std::vector<uint32_t> custom(instance_count);
    for (uint32_t i = 0; i < instance_count; ++i) {
        memcpy(&o2w[12 * (size_t)i], instances[i].transform, 12 * sizeof(float));
        if (!ddgi_affine_inverse(instances[i].transform, &w2o[12 * (size_t)i]))
            memset(&w2o[12 * (size_t)i], 0, 12 * sizeof(float));
        custom[i] = instances[i].custom_index & 0xFFFFFFu;
    }
    g_rt_scene = RtScene{traverse_ctx, traverse, o2w.data(), w2o.data(), custom.data()};
    g_rt_miss[0] = &entry_init_miss;
    g_rt_closest_hit = &entry_backface_test;
    probe_init::grid = make_probe_grid<probe_init::ProbeGrid>(d);
    probe_init::Probes = states;
    for (int c = 0; c < 4; ++c)
        probe_init::push.randomOrientation.c[c] =
            c < 3 ? vec4(orientation[c], orientation[3 + c], orientation[6 + c], 0.0f) : vec4(0.0f, 0.0f, 0.0f, 1.0f);
    const uint32_t rx = (uint32_t)d->resolution[0], ry = (uint32_t)d->resolution[1], rz = (uint32_t)d->resolution[2];
    const size_t launches = (size_t)rx * ry * rz;
    std::atomic<size_t> next{0};
    auto worker = [&] {
        for (;;) {
            const size_t k = next.fetch_add(1);
            if (k >= launches) break;
            rt_builtins = RtBuiltins{};
            rt_builtins.launch_id = uvec3((uint32_t)(k % rx), (uint32_t)((k / rx) % ry), (uint32_t)(k / ((size_t)rx * ry)));
            rt_builtins.launch_size = uvec3(rx, ry, rz);
            probe_init::main();
        }
    };
    const int nt = std::max(1, std::min(nthreads, 64));
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
}

}  // extern "C"

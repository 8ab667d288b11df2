/*
 * irradiance_probes.hpp — the C++ class VulkanExp's renderer calls, over the
 * C ABI of ddgi.h.
 *
 * Keeps the name, public fields and methods of `IrradianceProbes`
 * (src/IrradianceProbes.hpp:16-129) so the editor's call sites
 * (src/Editor.cpp:226-229, src/UI.cpp:312-316 and 991-1000,
 * src/VulkanLifecycle.cpp:133 and 239) keep their shape:
 *
 *   reference                                   here
 *   init(device, transferQF, computeQF, min, max) init(min, max)      -> ddgi_create
 *   writeDescriptorSet(renderer, lightBuffer)   writeDescriptorSet(scene, light) -> ddgi_scene_build
 *                                                                         + ddgi_set_light
 *   setLightBuffer(buffer)                      setLightBuffer(light)  -> ddgi_set_light
 *   updateUniforms()                            updateUniforms()       -> ddgi_set_grid
 *   initProbes(queue)                           initProbes(stream)     -> ddgi_init_probes
 *   update(scene, queue)                        update(stream)         -> ddgi_update_scheduled
 *   createPipeline / destroyPipeline            (nothing to build: kernels are compiled in)
 *   destroy()                                   destroy()              -> ddgi_destroy
 *   getProbeCount()                             getProbeCount()
 *   getIrradianceView() / getDepthView()        getIrradiance() / getDepth(): device pointers
 *   getComputeTimes() ...                       getComputeTimes() ...: per-stage ms of the last
 *                                               update when timing is on (the reference keeps
 *                                               rolling buffers of the same stages)
 *   GridParameters, TargetHysteresis,           the same public fields; TargetHysteresis and the
 *   ProbesPerUpdate, MaxRaysPerProbe            ramp of update() run in the library
 *                                               (ddgi_set_target_hysteresis)
 *
 * update() and initProbes() draw the ray-set rotation like the reference
 * (a random unit Z, genBasis, rows X, Y, Z: src/IrradianceProbes.cpp:347-355,
 * 455-460) from a generator seeded by the caller (the reference's
 * glm::sphericalRand is unseeded); overloads take the rotation explicitly.
 * Errors throw std::runtime_error with the library's message, as the
 * reference's VK_CHECK throws (src/vulkan/VkTools.hpp:39-47).  One host
 * thread per object, as in the reference.
 */
#ifndef DDGI_IRRADIANCE_PROBES_HPP
#define DDGI_IRRADIANCE_PROBES_HPP

#include <cmath>
#include <cstdint>
#include <random>
#include <stdexcept>
#include <string>

#include "ddgi.h"

namespace ddgi {

class IrradianceProbes {
public:
    static const uint32_t MaxRaysPerProbe = DDGI_MAX_RAYS_PER_PROBE;

    uint32_t ProbesPerUpdate = 0;  // 0: as many as the schedule selects
    float TargetHysteresis = 0.98f;

    // GridInfo defaults (src/IrradianceProbes.hpp:49-60); the last word is the
    // blend precision (ddgi_precision) where the reference has padding
    ddgi_grid_desc GridParameters{{0.0f, 0.0f, 0.0f}, 12.0f, {0.0f, 0.0f, 0.0f}, 0.0f, {32, 16, 32}, 192, 8, 16,
                                  0.3f, DDGI_PRECISION_FP32};

    explicit IrradianceProbes(uint64_t seed = 0) : _rng(seed) {}
    IrradianceProbes(const IrradianceProbes&) = delete;
    IrradianceProbes& operator=(const IrradianceProbes&) = delete;
    ~IrradianceProbes() { destroy(); }

    void init(const float extentMin[3], const float extentMax[3]) {
        destroy();
        for (int k = 0; k < 3; ++k) {
            GridParameters.extent_min[k] = extentMin[k];
            GridParameters.extent_max[k] = extentMax[k];
        }
        check(ddgi_create(&GridParameters, &_ctx), "ddgi_create");
        _shadow = GridParameters.hysteresis;
        _target = TargetHysteresis;
        check(ddgi_set_target_hysteresis(_ctx, _target), "ddgi_set_target_hysteresis");
    }

    // Scene and light binding (the reference binds the TLAS, vertex, index,
    // offset-table and material buffers through its descriptor set).
    void writeDescriptorSet(const ddgi_scene_desc& scene, const ddgi_light& light, ddgi_stream stream = nullptr) {
        check(ddgi_scene_build(ctx(), &scene, stream), "ddgi_scene_build");
        setLightBuffer(light);
    }
    void setLightBuffer(const ddgi_light& light) { check(ddgi_set_light(ctx(), &light), "ddgi_set_light"); }

    // The ramp moves the hysteresis inside the library, so GridParameters.
    // hysteresis here is only current after syncHysteresis().  Uploading keeps
    // the ramp's value unless the caller changed the field since it was last
    // in step with the library (the editor's hysteresis slider does that).
    void updateUniforms() {
        if (GridParameters.hysteresis == _shadow) GridParameters.hysteresis = currentHysteresis();
        check(ddgi_set_grid(ctx(), &GridParameters), "ddgi_set_grid");
        _shadow = GridParameters.hysteresis;
    }
    // Reads the ramp's current value into GridParameters.hysteresis.
    void syncHysteresis(ddgi_stream stream = nullptr) { _shadow = GridParameters.hysteresis = currentHysteresis(stream); }

    void initProbes(ddgi_stream stream = nullptr) {
        float m[9];
        randomOrientation(m);
        initProbes(m, stream);
    }
    void initProbes(const float orientation[9], ddgi_stream stream) {
        GridParameters.hysteresis = 0.0f;  // src/IrradianceProbes.cpp:358; the library zeroes the ramp's copy
        _shadow = 0.0f;
        check(ddgi_init_probes(ctx(), orientation, stream), "ddgi_init_probes");
    }

    void update(ddgi_stream stream = nullptr) {
        float m[9];
        randomOrientation(m);
        update(m, stream);
    }
    void update(const float orientation[9], ddgi_stream stream) {
        syncTarget();
        check(ddgi_update_scheduled(ctx(), orientation, ProbesPerUpdate, stream), "ddgi_update_scheduled");
    }
    // An update of the listed probes (or all with list = nullptr), for
    // callers that pick probes themselves.
    void update(const float orientation[9], const uint32_t* list, uint32_t count, ddgi_stream stream) {
        syncTarget();
        check(ddgi_update(ctx(), orientation, list, count, stream), "ddgi_update");
    }

    void destroy() {
        if (_ctx) ddgi_destroy(_ctx);
        _ctx = nullptr;
    }

    uint32_t getProbeCount() const {
        return (uint32_t)GridParameters.resolution[0] * (uint32_t)GridParameters.resolution[1] *
               (uint32_t)GridParameters.resolution[2];
    }

    // Device pointers of the current atlases (FP32: float4 / float2 texels;
    // BF16 form: half4 / half2).
    void* getIrradiance() const { return atlas(DDGI_ATLAS_COLOR); }
    void* getDepth() const { return atlas(DDGI_ATLAS_DEPTH); }

    // The hysteresis the last update blended with, and the ramp's host-side
    // value (the reference's GridParameters.hysteresis after the update).
    float blendedHysteresis(ddgi_stream stream = nullptr) {
        float b = 0.0f;
        check(ddgi_get_hysteresis(ctx(), &b, nullptr, nullptr, stream), "ddgi_get_hysteresis");
        return b;
    }
    float currentHysteresis(ddgi_stream stream = nullptr) {
        float p = 0.0f;
        check(ddgi_get_hysteresis(ctx(), nullptr, &p, nullptr, stream), "ddgi_get_hysteresis");
        return p;
    }

    // Stage timings of the last update (ddgi_enable_timing on): the
    // reference's compute, trace, update, border-copy and copy times.
    void enableTimings(bool on) { check(ddgi_enable_timing(ctx(), on ? 1 : 0), "ddgi_enable_timing"); }
    float getComputeTimes() const { return timings().total_ms; }
    float getTraceTimes() const { return timings().trace_ms; }
    float getUpdateTimes() const { return timings().blend_ms; }
    float getBorderCopyTimes() const { return timings().border_ms; }
    float getCopyTimes() const { return timings().copy_ms; }

    ddgi_ctx* context() const { return _ctx; }

    // genBasis (src/IrradianceProbes.cpp:347-355) in float with GLM's
    // operation order: b1 = (n.x > 0.9 ? y : x) - n dot(b1, n), normalised
    // as b1 * (1 / sqrt(dot(b1, b1))), b2 = cross(n, b1); dot sums left to
    // right.
    static void genBasis(const float n[3], float b1[3], float b2[3]) {
        b1[0] = n[0] > 0.9f ? 0.0f : 1.0f;
        b1[1] = n[0] > 0.9f ? 1.0f : 0.0f;
        b1[2] = 0.0f;
        const float d = b1[0] * n[0] + b1[1] * n[1] + b1[2] * n[2];
        for (int k = 0; k < 3; ++k) b1[k] -= n[k] * d;
        const float il = 1.0f / std::sqrt(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
        for (int k = 0; k < 3; ++k) b1[k] *= il;
        b2[0] = n[1] * b1[2] - b1[1] * n[2];
        b2[1] = n[2] * b1[0] - b1[2] * n[0];
        b2[2] = n[0] * b1[1] - b1[0] * n[1];
    }

    // A rotation as the reference draws one: Z uniform on the unit sphere,
    // genBasis, rows X, Y, Z of transpose(mat3(X, Y, Z)).
    void randomOrientation(float m[9]) {
        std::uniform_real_distribution<double> u(-1.0, 1.0), a(0.0, 6.283185307179586);
        const double z = u(_rng), phi = a(_rng);
        const double r = std::sqrt(z * z < 1.0 ? 1.0 - z * z : 0.0);
        const float Z[3] = {(float)(r * std::cos(phi)), (float)(r * std::sin(phi)), (float)z};
        float X[3], Y[3];
        genBasis(Z, X, Y);
        for (int k = 0; k < 3; ++k) {
            m[k] = X[k];
            m[3 + k] = Y[k];
            m[6 + k] = Z[k];
        }
    }

private:
    ddgi_ctx* _ctx = nullptr;
    float _target = 0.98f;
    float _shadow = 0.0f;  // GridParameters.hysteresis when it last matched the library's ramp value
    std::mt19937_64 _rng;

    ddgi_ctx* ctx() const {
        if (!_ctx) throw std::runtime_error("IrradianceProbes: init() first");
        return _ctx;
    }
    void check(ddgi_status s, const char* what) const {
        if (s != DDGI_OK)
            throw std::runtime_error(std::string(what) + ": " + ddgi_status_string(s) + ": " +
                                     (_ctx ? ddgi_last_error(_ctx) : ""));
    }
    // TargetHysteresis is a plain field, as in the reference; a change
    // reaches the library before the next update.
    void syncTarget() {
        if (TargetHysteresis != _target) {
            check(ddgi_set_target_hysteresis(ctx(), TargetHysteresis), "ddgi_set_target_hysteresis");
            _target = TargetHysteresis;
        }
    }
    void* atlas(ddgi_atlas_kind k) const {
        void* p = nullptr;
        check(ddgi_atlas_device_ptr(ctx(), k, &p), "ddgi_atlas_device_ptr");
        return p;
    }
    ddgi_timings timings() const {
        ddgi_timings t{};
        check(ddgi_get_timings(ctx(), &t), "ddgi_get_timings");
        return t;
    }
};

}  // namespace ddgi

#endif  // DDGI_IRRADIANCE_PROBES_HPP

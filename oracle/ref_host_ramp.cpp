// ref_host_ramp.cpp — the reference's hysteresis ramp, the block of
// IrradianceProbes::update at src/IrradianceProbes.cpp:462-476 ("Get closer
// to the target hysteresis"), compiled from its own source text:
// oracle/build_ref_glsl.py copies the block into
// oracle/_ref/src/hysteresisRamp.inc, and it compiles here inside a
// stand-in member function with the members it reads.  updateUniforms()
// records the value it would upload.  The block's counter is a
// function-local static, as in the reference, so a process's calls form one
// sequence.  Test infrastructure: built into oracle/_ref/libref_glsl.so.
#include <stdint.h>

#include <cmath>

namespace refhost {

struct RampHost {
    struct {
        float hysteresis;
    } GridParameters;
    float TargetHysteresis = 0.98f;
    uint32_t probe_total = 0;
    float uniform = 0.0f;  // the hysteresis of the last updateUniforms()
    uint32_t getProbeCount() const { return probe_total; }
    void updateUniforms() { uniform = GridParameters.hysteresis; }
    void step(uint32_t probeCount) {
#include "hysteresisRamp.inc"
    }
};

}  // namespace refhost

extern "C" {

// K successive updates of counts[k] probes each on a grid of P probes,
// starting from GridParameters.hysteresis = h0 (also the uploaded value):
// uniform[k] = the hysteresis the update's shaders read, param[k] =
// GridParameters.hysteresis after it.
void ref_ramp_sequence(float h0, float target, uint32_t P, const uint32_t* counts, uint32_t K, float* uniform,
                       float* param) {
    refhost::RampHost r;
    r.GridParameters.hysteresis = h0;
    r.uniform = h0;
    r.TargetHysteresis = target;
    r.probe_total = P;
    for (uint32_t k = 0; k < K; ++k) {
        r.step(counts[k]);
        uniform[k] = r.uniform;
        param[k] = r.GridParameters.hysteresis;
    }
}

}  // extern "C"

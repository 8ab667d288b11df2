// kernels.h — host-side launchers of the DDGI kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace ddgi {

// trace.cu
cudaError_t launch_trace_shade(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L,
                               const uint32_t* probe_list, uint32_t nprobes, const float4* dirs,
                               const uint32_t* ray_order, const uint32_t* states, const void* color,
                               const void* depth, bool fp16_atlas, float4* rays_out, ddgi_hit* hits_out,
                               uint32_t* err, cudaStream_t st, unsigned long long* counters = nullptr);
cudaError_t launch_trace_rays(const DeviceScene& sc, const float* origins, const float* dirs, uint32_t n, float tmin,
                              float tmax, uint32_t mask, int any, ddgi_hit* out, float* bary, uint32_t* err,
                              cudaStream_t st);

// wavefront.cu
struct WaveHits {
    float4* thit;    // (t, b1, b2, instance bits) per ray
    uint32_t* prim;  // primitive | backface << 31
};
struct ShadowQueue {
    uint32_t* idx;   // ray record index
    float4* pos;     // shadow-ray origin (hit position)
    float4* sun;     // unshadowed sun term (xyz) and night fade (w)
    uint32_t* count;
};
cudaError_t launch_wavefront(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L,
                             const uint32_t* probe_list, uint32_t nprobes, const float4* dirs,
                             const uint32_t* ray_order, const uint32_t* states, const void* color, const void* depth,
                             bool fp16_atlas, WaveHits hits, ShadowQueue q, uint32_t* counters, float4* rays_out,
                             ddgi_hit* hits_out, int stack_cap, uint32_t* err, cudaStream_t st,
                             cudaEvent_t after_primary);

// adjoint.cu
cudaError_t launch_replay_update(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L, const float4* dirs,
                                 uint32_t* states, float4* color, float2* depth, const float4* thit,
                                 const uint32_t* prim, float4* rays, uint32_t* err, cudaStream_t st);
cudaError_t launch_adjoint_step(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L, const float4* dirs,
                                const uint32_t* states, const float4* color_prev, const float2* depth_prev,
                                const float4* thit, const uint32_t* prim, float4* gk, float4* gprev, float4* gx,
                                double* grad, uint32_t* err, cudaStream_t st);

// blend_tc.cu
size_t tc_weight_bytes(uint32_t rays, uint32_t color_res, uint32_t depth_res);
bool tc_blend_supported(uint32_t color_res, uint32_t depth_res);
cudaError_t launch_blend_tc(const DeviceGrid& g, const uint32_t* probe_list, uint32_t nprobes, const float4* rays,
                            const float4* dirs, uint8_t* wbuf, float* rowsum, uint32_t* states, void* color,
                            void* depth, float4* acc_color, float2* acc_depth, uint32_t* err, cudaStream_t st);

// blend.cu
cudaError_t launch_blend_fp32(const DeviceGrid& g, const uint32_t* probe_list, uint32_t nprobes, const float4* rays,
                              const float4* dirs, uint32_t* states, float4* color, float2* depth, cudaStream_t st);

}  // namespace ddgi

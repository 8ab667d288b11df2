// gather.cu — the consumer of the probe atlas: a headless final gather.
//
// src/shaders/FinalGather.frag:39-80 per pixel of a G-buffer held in device
// memory instead of subpass attachments:
//   miss (depth <= 0): the sky radiance (the constant sky that replaces
//     sky.glsl, as on the probe rays' miss);
//   else  direct * pbrMetallicRoughness(sun)            (direct = the shadow
//         + mix(0.004, albedo, metal) * reflection        term's .r)
//         + sampleProbes(position, normal, view) * albedo * (1 - 0.004) * (1 - metal)
//         + emissive,
// with view = normalize(camera - position).  The bounce lookup is the same
// sample_probes the probe update uses, on the context's current atlas and
// probe states.  One thread per pixel, coalesced 16-byte loads.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "sky.cuh"
#include "shade.cuh"

namespace ddgi {

namespace {

template <class AV>
__global__ void __launch_bounds__(256) k_final_gather(GatherArgs a, AV at) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.pixels) return;
    const float4 pd = __ldg(a.position_depth + i);
    float4 out;
    if (!(pd.w > 0.0f)) {  // FinalGather.frag:55-57
        out = make_float4(a.L.sky[0], a.L.sky[1], a.L.sky[2], 1.0f);
        if (a.L.sky_mode == DDGI_SKY_ATMOSPHERE) {  // view direction in position.xyz, brightness 1
            const float3 c = sky::atmosphere(a.origin, sky::nrm3(f3(pd.x, pd.y, pd.z)),
                                             f3(a.L.dir[0], a.L.dir[1], a.L.dir[2]),
                                             f3(a.L.color[0], a.L.color[1], a.L.color[2]), 1.0f);
            out = make_float4(c.x, c.y, c.z, 1.0f);
        }
    } else {
        const float4 nm = __ldg(a.normal_metalness + i);
        const float4 ar = __ldg(a.albedo_roughness + i);
        const float4 em = __ldg(a.emissive + i);
        const float direct = __ldg(a.direct_light + i);
        const float4 refl = a.reflection ? __ldg(a.reflection + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float3 position = f3(pd.x, pd.y, pd.z);
        const float3 normal = norm3(f3(nm.x, nm.y, nm.z));
        const float metal = nm.w, rough = ar.w;
        const float3 albedo = f3(ar.x, ar.y, ar.z);
        const float3 view = norm3(a.origin - position);
        float3 c = pbr_metallic_roughness(normal, view, f3(a.L.color[0], a.L.color[1], a.L.color[2]),
                                          f3(a.L.dir[0], a.L.dir[1], a.L.dir[2]), albedo, metal, rough) *
                   direct;
        const float f0 = 0.004f;
        const float3 diffuse = albedo * (1.0f - f0) * (1.0f - metal);
        const float3 specular = mix3(f3(f0, f0, f0), albedo, metal);
        c = c + specular * f3(refl.x, refl.y, refl.z);
        const float3 indirect = sample_probes(position, normal, view, a.g, a.states, at);
        c = c + indirect * diffuse;
        c = c + f3(em.x, em.y, em.z);
        out = make_float4(c.x, c.y, c.z, 1.0f);
    }
    a.out[i] = out;
}

}  // namespace

cudaError_t launch_final_gather(const GatherArgs& a, const void* color, const void* depth, bool fp16_atlas,
                                cudaStream_t st) {
    if (a.pixels == 0) return cudaSuccess;
    const uint32_t blocks = (a.pixels + 255) / 256;
    if (fp16_atlas) {
        AtlasView<ColorTexF16, DepthTexF16> at{{static_cast<const uint2*>(color)},
                                               {static_cast<const uint32_t*>(depth)}};
        k_final_gather<<<blocks, 256, 0, st>>>(a, at);
    } else {
        AtlasView<ColorTexF32, DepthTexF32> at{{static_cast<const float4*>(color)},
                                               {static_cast<const float2*>(depth)}};
        k_final_gather<<<blocks, 256, 0, st>>>(a, at);
    }
    return cudaGetLastError();
}

}  // namespace ddgi

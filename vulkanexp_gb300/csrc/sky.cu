// sky.cu — miss records shaded with the atmospheric sky (optional mode).
//
// With ddgi_set_sky_mode(DDGI_SKY_ATMOSPHERE) the miss program's radiance is
// sky() of src/shaders/sky.glsl:60-127 (miss.rmiss:22) instead of the
// constant sky radiance.  The traces write misses with the constant sky as
// before (depth -1); this pass, run after them and before the blend, replaces
// the radiance of every miss record with the atmospheric sky seen from the
// probe along the ray.  Record i of an update belongs to slot i / R, ray
// i % R (the direction table's index).
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "sky.cuh"

namespace ddgi {

namespace {

__global__ void __launch_bounds__(128) k_shade_sky(DeviceGrid g, DeviceLight L, uint32_t total,
                                                   const uint32_t* dev_count, const uint32_t* probe_list,
                                                   const float4* __restrict__ dirs, float4* rays) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (dev_count) total = min(total, *dev_count * g.rays);
    if (i >= total) return;
    const float4 r = rays[i];
    if (r.w != -1.0f) return;  // a hit
    const uint32_t slot = i / g.rays, ray = i - slot * g.rays;
    const uint32_t probe = probe_list ? probe_list[slot] : slot;
    const float3 o = probe_origin_exact(g, probe);
    const float4 d = __ldg(dirs + ray);
    const float3 c = sky::atmosphere(o, f3(d.x, d.y, d.z), f3(L.dir[0], L.dir[1], L.dir[2]),
                                     f3(L.color[0], L.color[1], L.color[2]), L.sun_brightness);
    rays[i] = make_float4(c.x, c.y, c.z, -1.0f);
}

}  // namespace

cudaError_t launch_shade_sky(const DeviceGrid& g, const DeviceLight& L, uint32_t nprobes, const uint32_t* dev_count,
                             const uint32_t* probe_list, const float4* dirs, float4* rays, cudaStream_t st) {
    const uint32_t total = nprobes * g.rays;
    if (total == 0) return cudaSuccess;
    k_shade_sky<<<(total + 127) / 128, 128, 0, st>>>(g, L, total, dev_count, probe_list, dirs, rays);
    return cudaGetLastError();
}

}  // namespace ddgi

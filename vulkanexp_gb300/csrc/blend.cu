// blend.cu — plain FP32 atlas blend with the border copy fused in.
//
// One block per updated probe, one thread per interior texel of both atlases
// (36 colour + 196 depth for 8/16 tiles), as the reference's two dispatches
// do (src/shaders/probesUpdate.glsl:49-121: WG 1x6x6 and 1x14x14, one
// workgroup per probe).  The probe's ray records and the shared direction
// table are staged in shared memory; each texel sums its cosine (colour) or
// cosine^sharpness (depth) weighted rays in ray order, normalises, applies
// hysteresis against the previous texel in place, and the block then copies
// the octahedral border (src/shaders/probesCopyBorders.comp:21-245,
// generalised to any tile side) and updates the probe state
// (probesUpdate.glsl:104-120, with the max-change taken over all texels).
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"

namespace ddgi {

namespace {

// Blend of one probe by the whole block: `pr` = its R ray records.
// `hy` is the hysteresis of this update (the grid's, or the ramp's value).
__device__ __forceinline__ void blend_probe_fp32(const DeviceGrid& g, uint32_t probe, const float4* __restrict__ pr,
                                                 const float4* __restrict__ dirs, uint32_t* states, float4* color,
                                                 float2* depth, const float hy) {
    extern __shared__ float4 smem[];
    const uint32_t R = g.rays;
    float4* s_rays = smem;
    float4* s_dirs = smem + R;
    __shared__ uint32_t s_max_change;
    __shared__ uint32_t s_out_of_range;

    if (threadIdx.x == 0) {
        s_max_change = 0u;
        s_out_of_range = 0u;
    }
    __syncthreads();
    uint32_t oor = 0;
    for (uint32_t r = threadIdx.x; r < R; r += blockDim.x) {
        float4 v = pr[r];
        s_rays[r] = v;
        s_dirs[r] = dirs[r];
        if (v.w < 0.0f || v.w > g.cell_len) ++oor;
    }
    if (oor) atomicAdd(&s_out_of_range, oor);
    __syncthreads();

    const uint32_t rx = (uint32_t)g.res[0], rxy = (uint32_t)(g.res[0] * g.res[1]);
    const int ix = (int)(probe % rx), iy = (int)((probe % rxy) / rx), iz = (int)(probe / rxy);
    const int tile = iy * g.res[0] + ix;
    const int nc = (int)g.color_res - 2, nd = (int)g.depth_res - 2;
    const int ncol = nc * nc, ntex = ncol + nd * nd;

    for (int t = threadIdx.x; t < ntex; t += blockDim.x) {
        if (t < ncol) {
            int tx = t % nc, ty = t / nc;
            float sc = texel_scale((uint32_t)nc), ce = 0.5f * (float)(nc - 1);
            float3 td = oct_decode(sc * ((float)tx - ce), sc * ((float)ty - ce));
            float a0 = 0.f, a1 = 0.f, a2 = 0.f, aw = 0.f;
            for (uint32_t r = 0; r < R; ++r) {
                float4 d = s_dirs[r];
                float4 v = s_rays[r];
                float w = fmaxf(0.0f, td.x * d.x + td.y * d.y + td.z * d.z);
                a0 += w * v.x;
                a1 += w * v.y;
                a2 += w * v.z;
                aw += w;
            }
            if (aw > 1e-3f) {
                a0 /= aw;
                a1 /= aw;
                a2 /= aw;
            }
            size_t px = (size_t)((int)g.color_res * tile + 1 + tx), py = (size_t)((int)g.color_res * iz + 1 + ty);
            float4* texel = color + py * g.color_w + px;
            float4 prev = *texel;
            float mc = fmaxf(fmaxf(fabsf(a0 - prev.x), fabsf(a1 - prev.y)), fabsf(a2 - prev.z));
            atomicMax(&s_max_change, __float_as_uint(mc));
            *texel = store_color(g, a0 * (1.0f - hy) + prev.x * hy, a1 * (1.0f - hy) + prev.y * hy,
                                 a2 * (1.0f - hy) + prev.z * hy);
        } else {
            int u = t - ncol;
            int tx = u % nd, ty = u / nd;
            float sc = texel_scale((uint32_t)nd), ce = 0.5f * (float)(nd - 1);
            float3 td = oct_decode(sc * ((float)tx - ce), sc * ((float)ty - ce));
            float a0 = 0.f, a1 = 0.f, aw = 0.f;
            const float cl = g.cell_len;
            for (uint32_t r = 0; r < R; ++r) {
                float4 d = s_dirs[r];
                float dep = fminf(cl, s_rays[r].w);
                if (dep < 0.0f) dep = cl;
                float w = powf(fmaxf(0.0f, td.x * d.x + td.y * d.y + td.z * d.z), g.sharp);
                a0 += w * dep;
                a1 += w * dep * dep;
                aw += w;
            }
            if (aw > 1e-3f) {
                a0 /= aw;
                a1 /= aw;
            }
            size_t px = (size_t)((int)g.depth_res * tile + 1 + tx), py = (size_t)((int)g.depth_res * iz + 1 + ty);
            float2* texel = depth + py * g.depth_w + px;
            float2 prev = *texel;
            *texel = store_depth(g, a0 * (1.0f - hy) + prev.x * hy, a1 * (1.0f - hy) + prev.y * hy);
        }
    }
    __syncthreads();

    // border copy (probesCopyBorders.comp), generalised
    const int nbc = 4 + 4 * nc, nbd = 4 + 4 * nd;
    for (int e = threadIdx.x; e < nbc + nbd; e += blockDim.x) {
        if (e < nbc) {
            int4 b = border_entry(e, (int)g.color_res);
            size_t ox = (size_t)g.color_res * tile, oy = (size_t)g.color_res * iz;
            color[(oy + b.y) * g.color_w + ox + b.x] = color[(oy + b.w) * g.color_w + ox + b.z];
        } else {
            int4 b = border_entry(e - nbc, (int)g.depth_res);
            size_t ox = (size_t)g.depth_res * tile, oy = (size_t)g.depth_res * iz;
            depth[(oy + b.y) * g.depth_w + ox + b.x] = depth[(oy + b.w) * g.depth_w + ox + b.z];
        }
    }

    if (threadIdx.x == 0) {  // probesUpdate.glsl:110-119
        uint32_t s = states[probe];
        if (s_out_of_range >= R) {
            s = 8;
        } else {
            float mc = __uint_as_float(s_max_change);
            float sf = (float)s;
            if (mc < 0.02f / sf) s = min(s + 1u, 8u);
            else if (mc > 0.04f / sf) s = max(s - 1u, 1u);
            else if (mc > 0.25f) s = 1;
        }
        states[probe] = s;
    }
}

__global__ void __launch_bounds__(256) k_blend_fp32(DeviceGrid g, const uint32_t* __restrict__ probe_list,
                                                    const float4* __restrict__ rays, const float4* __restrict__ dirs,
                                                    uint32_t* states, float4* color, float2* depth,
                                                    const uint32_t* dev_count, const float* hyst_dev) {
    const uint32_t slot = blockIdx.x;
    if (dev_count && slot >= *dev_count) return;  // whole block
    const uint32_t probe = probe_list ? probe_list[slot] : slot;
    blend_probe_fp32(g, probe, rays + (size_t)slot * g.rays, dirs, states, color, depth,
                     hyst_dev ? *hyst_dev : g.hyst);
}

// Batched form: block b blends probe (b - tile_base[i]) of volume list[i];
// the block that finishes a volume's last probe stamps its completion time.
__global__ void __launch_bounds__(256) k_batch_blend_fp32(BatchTables bt, BatchBlendList bl,
                                                          const float4* __restrict__ rays) {
    uint32_t lo = 0, hi = bl.n;  // tile_base[lo] <= b < tile_base[hi]
    const uint32_t b = blockIdx.x;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(bl.tile_base + mid) <= b) lo = mid;
        else hi = mid;
    }
    const uint32_t v = __ldg(bl.list + lo);
    const BatchVolume& vol = bt.vols[v];
    const uint32_t probe = b - __ldg(bl.tile_base + lo);
    blend_probe_fp32(vol.g, probe, rays + vol.ray_base + (size_t)probe * vol.g.rays, bt.dirs + vol.dir_base,
                     vol.states, static_cast<float4*>(vol.color), static_cast<float2*>(vol.depth), vol.g.hyst);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t items = __ldg(bl.tile_base + lo + 1) - __ldg(bl.tile_base + lo);
        if (atomicAdd(bt.done + v, 1u) == items - 1u) bt.clock[1 + v] = globaltimer_ns();
    }
}

}  // namespace

cudaError_t launch_blend_fp32(const DeviceGrid& g, const uint32_t* probe_list, uint32_t nprobes, const float4* rays,
                              const float4* dirs, uint32_t* states, float4* color, float2* depth, cudaStream_t st,
                              const uint32_t* dev_count, const float* hyst_dev) {
    if (nprobes == 0) return cudaSuccess;
    size_t smem = sizeof(float4) * 2 * g.rays;
    k_blend_fp32<<<nprobes, 256, smem, st>>>(g, probe_list, rays, dirs, states, color, depth, dev_count, hyst_dev);
    return cudaGetLastError();
}

cudaError_t launch_batch_blend_fp32(const BatchTables& bt, const BatchBlendList& bl, uint32_t max_rays,
                                    const float4* rays, uint32_t threads, cudaStream_t st) {
    if (bl.ntiles == 0) return cudaSuccess;
    threads = threads < 32 ? 32 : (threads > 256 ? 256 : threads / 32 * 32);
    size_t smem = sizeof(float4) * 2 * max_rays;
    k_batch_blend_fp32<<<bl.ntiles, threads, smem, st>>>(bt, bl, rays);
    return cudaGetLastError();
}

}  // namespace ddgi

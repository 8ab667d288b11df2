// blend_shared.cu — FP32 atlas blend with the blend weights computed once per
// update instead of once per probe.
//
// Every probe of an update traces the same direction table, so the weight of
// ray r in interior texel t (max(0, n_t . d_r) for colour, its depth-sharpness
// power for depth: src/shaders/probesUpdate.glsl:71-98) and each texel's
// weight sum are the same for all probes.  k_fp32_weights computes them once
// (W[r][t], texel-contiguous, and the sums in ray order); the blend then is a
// product of each probe's ray records with W, done for kProbesPerBlock probes
// per block so that each W row is read once per block.  Arithmetic and
// accumulation order per (probe, texel) are those of blend.cu's per-probe
// kernel (same weight expressions, sums in ray order, the same normalisation,
// hysteresis, border copy and probe-state rule), which remains the plain
// reference-like form.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ddgi.h"
#include "common.cuh"
#include "kernels.h"

namespace ddgi {

namespace {

constexpr uint32_t kProbesPerBlock = 8;
constexpr uint32_t kBlendThreads = 256;

// Weights of one texel over all rays (thread t of the grid = texel t).
__device__ __forceinline__ void texel_weights(const DeviceGrid& g, const float4* __restrict__ dirs, uint32_t t,
                                              float* __restrict__ W, float* __restrict__ wsum) {
    const int nc = (int)g.color_res - 2, nd = (int)g.depth_res - 2;
    const uint32_t ncol = (uint32_t)(nc * nc), ntex = ncol + (uint32_t)(nd * nd);
    if (t >= ntex) return;
    const uint32_t R = g.rays;
    float aw = 0.0f;
    if (t < ncol) {
        int tx = (int)t % nc, ty = (int)t / nc;
        float sc = texel_scale((uint32_t)nc), ce = 0.5f * (float)(nc - 1);
        float3 td = oct_decode(sc * ((float)tx - ce), sc * ((float)ty - ce));
        for (uint32_t r = 0; r < R; ++r) {
            float4 d = __ldg(dirs + r);
            float w = fmaxf(0.0f, td.x * d.x + td.y * d.y + td.z * d.z);
            W[(size_t)r * ntex + t] = w;
            aw += w;
        }
    } else {
        int u = (int)(t - ncol);
        int tx = u % nd, ty = u / nd;
        float sc = texel_scale((uint32_t)nd), ce = 0.5f * (float)(nd - 1);
        float3 td = oct_decode(sc * ((float)tx - ce), sc * ((float)ty - ce));
        for (uint32_t r = 0; r < R; ++r) {
            float4 d = __ldg(dirs + r);
            float w = powf(fmaxf(0.0f, td.x * d.x + td.y * d.y + td.z * d.z), g.sharp);
            W[(size_t)r * ntex + t] = w;
            aw += w;
        }
    }
    wsum[t] = aw;
}

__global__ void __launch_bounds__(128) k_fp32_weights(DeviceGrid g, const float4* __restrict__ dirs, float* W,
                                                      float* wsum) {
    texel_weights(g, dirs, blockIdx.x * blockDim.x + threadIdx.x, W, wsum);
}

// Blend of probes p0 .. p0 + np - 1 (slots of `rays`) by one block.
__device__ __forceinline__ void blend_probes_shared(const DeviceGrid& g, const uint32_t* __restrict__ probe_list,
                                                    uint32_t p0, uint32_t np, const float4* __restrict__ rays,
                                                    const float* __restrict__ W, const float* __restrict__ wsum,
                                                    uint32_t* states, float4* color, float2* depth, const float hy) {
    extern __shared__ float4 s_rec[];  // [kProbesPerBlock][R]: colour xyz, clamped depth w
    __shared__ uint32_t s_max_change[kProbesPerBlock], s_out_of_range[kProbesPerBlock], s_probe[kProbesPerBlock];
    const uint32_t R = g.rays;
    const float cl = g.cell_len;
    if (threadIdx.x < kProbesPerBlock) {
        s_max_change[threadIdx.x] = 0u;
        s_out_of_range[threadIdx.x] = 0u;
        s_probe[threadIdx.x] = threadIdx.x < np ? (probe_list ? probe_list[p0 + threadIdx.x] : p0 + threadIdx.x) : 0u;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < np * R; i += blockDim.x) {
        const uint32_t p = i / R;
        float4 v = rays[(size_t)p0 * R + i];
        if (v.w < 0.0f || v.w > cl) atomicAdd(&s_out_of_range[p], 1u);
        float dep = fminf(cl, v.w);
        if (dep < 0.0f) dep = cl;
        s_rec[i] = make_float4(v.x, v.y, v.z, dep);
    }
    __syncthreads();

    const uint32_t rx = (uint32_t)g.res[0], rxy = (uint32_t)(g.res[0] * g.res[1]);
    const int nc = (int)g.color_res - 2, nd = (int)g.depth_res - 2;
    const uint32_t ncol = (uint32_t)(nc * nc), ntex = ncol + (uint32_t)(nd * nd);
    for (uint32_t t = threadIdx.x; t < ntex; t += blockDim.x) {
        const float aw = wsum[t];
        if (t < ncol) {
            float a[kProbesPerBlock][3];
#pragma unroll
            for (uint32_t p = 0; p < kProbesPerBlock; ++p) a[p][0] = a[p][1] = a[p][2] = 0.0f;
            for (uint32_t r = 0; r < R; ++r) {
                const float w = __ldg(W + (size_t)r * ntex + t);
#pragma unroll
                for (uint32_t p = 0; p < kProbesPerBlock; ++p) {
                    if (p < np) {
                        const float4 v = s_rec[p * R + r];
                        a[p][0] += w * v.x;
                        a[p][1] += w * v.y;
                        a[p][2] += w * v.z;
                    }
                }
            }
            const int tx = (int)t % nc, ty = (int)t / nc;
#pragma unroll
            for (uint32_t p = 0; p < kProbesPerBlock; ++p) {
                if (p >= np) continue;
                float a0 = a[p][0], a1 = a[p][1], a2 = a[p][2];
                if (aw > 1e-3f) {
                    a0 /= aw;
                    a1 /= aw;
                    a2 /= aw;
                }
                const uint32_t probe = s_probe[p];
                const int ix = (int)(probe % rx), iy = (int)((probe % rxy) / rx), iz = (int)(probe / rxy);
                const int tile = iy * g.res[0] + ix;
                size_t px = (size_t)((int)g.color_res * tile + 1 + tx), py = (size_t)((int)g.color_res * iz + 1 + ty);
                float4* texel = color + py * g.color_w + px;
                float4 prev = *texel;
                float mc = fmaxf(fmaxf(fabsf(a0 - prev.x), fabsf(a1 - prev.y)), fabsf(a2 - prev.z));
                atomicMax(&s_max_change[p], __float_as_uint(mc));
                *texel = store_color(g, a0 * (1.0f - hy) + prev.x * hy, a1 * (1.0f - hy) + prev.y * hy,
                                     a2 * (1.0f - hy) + prev.z * hy);
            }
        } else {
            float a[kProbesPerBlock][2];
#pragma unroll
            for (uint32_t p = 0; p < kProbesPerBlock; ++p) a[p][0] = a[p][1] = 0.0f;
            for (uint32_t r = 0; r < R; ++r) {
                const float w = __ldg(W + (size_t)r * ntex + t);
#pragma unroll
                for (uint32_t p = 0; p < kProbesPerBlock; ++p) {
                    if (p < np) {
                        const float dep = s_rec[p * R + r].w;
                        a[p][0] += w * dep;
                        a[p][1] += w * dep * dep;
                    }
                }
            }
            const int u = (int)(t - ncol), tx = u % nd, ty = u / nd;
#pragma unroll
            for (uint32_t p = 0; p < kProbesPerBlock; ++p) {
                if (p >= np) continue;
                float a0 = a[p][0], a1 = a[p][1];
                if (aw > 1e-3f) {
                    a0 /= aw;
                    a1 /= aw;
                }
                const uint32_t probe = s_probe[p];
                const int ix = (int)(probe % rx), iy = (int)((probe % rxy) / rx), iz = (int)(probe / rxy);
                const int tile = iy * g.res[0] + ix;
                size_t px = (size_t)((int)g.depth_res * tile + 1 + tx), py = (size_t)((int)g.depth_res * iz + 1 + ty);
                float2* texel = depth + py * g.depth_w + px;
                float2 prev = *texel;
                *texel = store_depth(g, a0 * (1.0f - hy) + prev.x * hy, a1 * (1.0f - hy) + prev.y * hy);
            }
        }
    }
    __syncthreads();

    // border copy (probesCopyBorders.comp, generalised) of each probe
    const int nbc = 4 + 4 * nc, nbd = 4 + 4 * nd;
    for (uint32_t i = threadIdx.x; i < np * (uint32_t)(nbc + nbd); i += blockDim.x) {
        const uint32_t p = i / (uint32_t)(nbc + nbd);
        const int e = (int)(i % (uint32_t)(nbc + nbd));
        const uint32_t probe = s_probe[p];
        const int ix = (int)(probe % rx), iy = (int)((probe % rxy) / rx), iz = (int)(probe / rxy);
        const int tile = iy * g.res[0] + ix;
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

    if (threadIdx.x < np) {  // probesUpdate.glsl:110-119
        const uint32_t p = threadIdx.x, probe = s_probe[p];
        uint32_t s = states[probe];
        if (s_out_of_range[p] >= R) {
            s = 8;
        } else {
            float mc = __uint_as_float(s_max_change[p]);
            float sf = (float)s;
            if (mc < 0.02f / sf) s = min(s + 1u, 8u);
            else if (mc > 0.04f / sf) s = max(s - 1u, 1u);
            else if (mc > 0.25f) s = 1;
        }
        states[probe] = s;
    }
}

__global__ void __launch_bounds__(kBlendThreads) k_blend_fp32_shared(DeviceGrid g, const uint32_t* probe_list,
                                                                     uint32_t nprobes, const float4* rays,
                                                                     const float* W, const float* wsum,
                                                                     uint32_t* states, float4* color, float2* depth,
                                                                     const uint32_t* dev_count,
                                                                     const float* hyst_dev) {
    const uint32_t n = dev_count ? min(*dev_count, nprobes) : nprobes;
    const uint32_t p0 = blockIdx.x * kProbesPerBlock;
    if (p0 >= n) return;  // whole block
    blend_probes_shared(g, probe_list, p0, min(kProbesPerBlock, n - p0), rays, W, wsum, states, color, depth,
                        hyst_dev ? *hyst_dev : g.hyst);
}

// Batched form: weights per FP32 volume (grid y = position in the list),
// then block b blends tile (b - tile_base[i]) of kProbesPerBlock probes of
// volume list[i]; the block finishing a volume's last tile stamps its
// completion time.
__global__ void __launch_bounds__(128) k_batch_fp32_weights(BatchTables bt, BatchBlendList bl) {
    const BatchVolume& vol = bt.vols[__ldg(bl.list + blockIdx.y)];
    texel_weights(vol.g, bt.dirs + vol.dir_base, blockIdx.x * blockDim.x + threadIdx.x,
                  reinterpret_cast<float*>(vol.wbuf), vol.rowsum);
}

__global__ void __launch_bounds__(kBlendThreads) k_batch_blend_fp32_shared(BatchTables bt, BatchBlendList bl,
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
    const uint32_t P = (uint32_t)vol.g.res[0] * (uint32_t)vol.g.res[1] * (uint32_t)vol.g.res[2];
    const uint32_t p0 = (b - __ldg(bl.tile_base + lo)) * kProbesPerBlock;
    if (p0 < P)
        blend_probes_shared(vol.g, nullptr, p0, min(kProbesPerBlock, P - p0), rays + vol.ray_base,
                            reinterpret_cast<const float*>(vol.wbuf), vol.rowsum, vol.states,
                            static_cast<float4*>(vol.color), static_cast<float2*>(vol.depth), vol.g.hyst);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t items = __ldg(bl.tile_base + lo + 1) - __ldg(bl.tile_base + lo);
        if (atomicAdd(bt.done + v, 1u) == items - 1u) bt.clock[1 + v] = globaltimer_ns();
    }
}

}  // namespace

size_t fp32_weight_bytes(uint32_t rays, uint32_t color_res, uint32_t depth_res) {
    const size_t ntex = (size_t)(color_res - 2) * (color_res - 2) + (size_t)(depth_res - 2) * (depth_res - 2);
    return ntex * rays * sizeof(float);
}

uint32_t fp32_shared_tiles(uint32_t nprobes) { return (nprobes + kProbesPerBlock - 1) / kProbesPerBlock; }

// Record staging of kProbesPerBlock probes at up to DDGI_MAX_RAYS_PER_PROBE
// rays, on the current device.
cudaError_t set_shared_smem_limit() {
    const int bytes = (int)(sizeof(float4) * kProbesPerBlock * DDGI_MAX_RAYS_PER_PROBE);
    cudaError_t e = ensure_dynamic_smem(k_blend_fp32_shared, bytes);
    if (e == cudaSuccess) e = ensure_dynamic_smem(k_batch_blend_fp32_shared, bytes);
    return e;
}

cudaError_t launch_blend_fp32_shared(const DeviceGrid& g, const uint32_t* probe_list, uint32_t nprobes,
                                     const float4* rays, const float4* dirs, float* W, float* wsum, uint32_t* states,
                                     float4* color, float2* depth, cudaStream_t st, const uint32_t* dev_count,
                                     const float* hyst_dev) {
    if (nprobes == 0) return cudaSuccess;
    cudaError_t e = set_shared_smem_limit();
    if (e != cudaSuccess) return e;
    const uint32_t ntex = (g.color_res - 2) * (g.color_res - 2) + (g.depth_res - 2) * (g.depth_res - 2);
    k_fp32_weights<<<(ntex + 127) / 128, 128, 0, st>>>(g, dirs, W, wsum);
    const size_t smem = sizeof(float4) * kProbesPerBlock * g.rays;
    k_blend_fp32_shared<<<fp32_shared_tiles(nprobes), kBlendThreads, smem, st>>>(g, probe_list, nprobes, rays, W,
                                                                               wsum, states, color, depth,
                                                                               dev_count, hyst_dev);
    return cudaGetLastError();
}

cudaError_t launch_batch_blend_fp32_shared(const BatchTables& bt, const BatchBlendList& bl, uint32_t max_ntex,
                                           uint32_t max_rays, const float4* rays, cudaStream_t st) {
    if (bl.ntiles == 0) return cudaSuccess;
    cudaError_t e = set_shared_smem_limit();
    if (e != cudaSuccess) return e;
    k_batch_fp32_weights<<<dim3((max_ntex + 127) / 128, bl.n), 128, 0, st>>>(bt, bl);
    const size_t smem = sizeof(float4) * kProbesPerBlock * max_rays;
    k_batch_blend_fp32_shared<<<bl.ntiles, kBlendThreads, smem, st>>>(bt, bl, rays);
    return cudaGetLastError();
}

}  // namespace ddgi

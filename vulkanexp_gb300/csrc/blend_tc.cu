// blend_tc.cu — the atlas blend as a BF16 tensor-core contraction (tcgen05).
//
// Within one update every probe uses the same ray directions (one rotation
// per update, src/IrradianceProbes.cpp:455-460), so the blend weights of
// src/shaders/probesUpdate.glsl:70-83 form two matrices shared by all probes:
//   W_c[t][r] = max(0, dot(texelDir_t, dir_r))               (colour texels)
//   W_d[t][r] = max(0, dot(texelDir_t, dir_r))^depthSharpness (depth texels)
// and the blend of every probe is a product with its ray records:
//   colour[t][c] = sum_r W_c[t][r] * rgb_r[c]            c = r, g, b
//   depth[t][c]  = sum_r W_d[t][r] * (d_r, d_r^2)[c]
// normalised by the row sums sum_r W[t][r] (the reference's result.w, the
// same for every probe, so it is computed once per update).
//
// Tiling: a CTA takes 32 probes; each probe owns 4 rows of the A operand
// (r, g, b, 0 for colour; d, d^2, 0, 0 for depth), so A is M = 128 rows x K
// rays, K-major, and the weights are B (N = texels, padded to 16) x K.
// K is processed in chunks of 64 rays staged in shared memory as BF16
// (radiance scaled per probe by 1 / max radiance, depth by 1 / |cell|);
// one thread issues tcgen05.mma (M = 128, K = 16 per instruction) into two
// FP32 accumulators in tensor memory (colour at column 0, depth at 256).
// Both operands are split into a BF16 high part and a BF16 remainder
// (x = hi + lo) and three products hi*hi + hi*lo + lo*hi are accumulated,
// which brings the contraction to ~16 mantissa bits; the MMAs are a small
// part of this memory-bound kernel, and it keeps the atlas error against an
// FP64 blend below 1e-3 (the FP16 atlas store dominates what is left).
// The epilogue reads the accumulators with tcgen05.ld, undoes the scaling,
// normalises, applies hysteresis in FP32 against the FP16 atlas, stores FP16
// texels, copies the borders and updates the probe states.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "tc.cuh"

namespace ddgi {

namespace {

constexpr int kTileProbes = 32;  // 128 A rows
constexpr int kKChunk = 64;      // rays per shared-memory stage
constexpr int kThreads = 256;
constexpr uint32_t kSBO = (kKChunk / 8) * 128;  // bytes between 8-row groups
constexpr uint32_t kLBO = 128;                  // bytes between K-adjacent core matrices
constexpr uint32_t kDepthCol = 256;             // TMEM column of the depth accumulator
constexpr uint32_t kTmemCols = 512;
// Every CTA allocates all 512 tensor-memory columns of its SM, so no two
// CTAs may share an SM: the shared-memory request is at least this much
// (two of them exceed the SM's 228 KB).
constexpr size_t kMinSmem = 120 * 1024;

struct TcArgs {
    DeviceGrid g;
    const uint32_t* probe_list;
    uint32_t nprobes;
    const float4* rays;
    // per chunk: high parts B_d (Nd rows), B_c (Nc rows), then the remainders
    // in the same order; core-matrix layout
    const uint4* wchunks;
    const float* rowsum;   // Nd depth sums then Nc colour sums (of the BF16 weights)
    uint32_t nc, nd;       // interior sides
    uint32_t Nc, Nd;       // texel counts padded to 16
    uint32_t nchunks;
    uint32_t* states;
    uint2* color;        // published atlas: 4 x half per texel
    uint32_t* depth;     // 2 x half per texel
    float4* acc_color;   // FP32 hysteresis accumulators (interior texels)
    float2* acc_depth;
    uint32_t* err;
    const uint32_t* dev_count;  // listed probes, read on the device (NULL: nprobes)
    uint32_t stall;             // test hook: issue no MMA and no commit, so the completion wait runs out
    const float* hyst_dev;      // hysteresis of this update in device memory (the ramp's), or NULL: g.hyst
};

// Limit of one tensor-core completion wait (the MMAs of a chunk take
// microseconds).  The limits count global (wall-clock) time, so time the
// CTA spends preempted or time-sliced with another context's work counts
// too; the first limit is generous for that reason.  After it runs out the
// CTA records the error and waits once more, up to kDrainLimitNs, for MMAs
// that may still be in flight, before it releases its tensor memory.
constexpr uint64_t kWaitLimitNs = 500ull * 1000 * 1000;
constexpr uint64_t kDrainLimitNs = 4000ull * 1000 * 1000;

// Byte offset of (row, 8-element K group) in a K-chunk operand.
__host__ __device__ __forceinline__ uint32_t canon_off(uint32_t row, uint32_t kgroup) {
    return (row >> 3) * kSBO + kgroup * 128u + (row & 7u) * 16u;
}

// Two floats as BF16 high parts (returned) and BF16 remainders (*lo); a in
// the low half (lower address).
__device__ __forceinline__ uint32_t pack2(float a, float b, uint32_t* lo) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    float2 hf = __bfloat1622float2(h);
    __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    *lo = *reinterpret_cast<uint32_t*>(&l);
    return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ int4 border_entry(int e, int n) {
    int m = n - 2;
    if (e == 0) return make_int4(0, 0, n - 2, n - 2);
    if (e == 1) return make_int4(0, n - 1, n - 2, 1);
    if (e == 2) return make_int4(n - 1, 0, 1, n - 2);
    if (e == 3) return make_int4(n - 1, n - 1, 1, 1);
    e -= 4;
    int side = e / m, j = e % m + 1;
    if (side == 0) return make_int4(0, j, 1, n - 1 - j);
    if (side == 1) return make_int4(n - 1, j, n - 2, n - 1 - j);
    if (side == 2) return make_int4(j, 0, n - 1 - j, 1);
    return make_int4(j, n - 1, n - 1 - j, n - 2);
}

__device__ __forceinline__ uint2 float4_to_half4(float a, float b, float c, float d) {
    __half2 x = __floats2half2_rn(a, b), y = __floats2half2_rn(c, d);
    return make_uint2(*reinterpret_cast<uint32_t*>(&x), *reinterpret_cast<uint32_t*>(&y));
}

// Row `row` of the weight matrices of one update in the B-operand layout
// (depth rows first, then colour rows), plus its row sum; one warp per row.
// Lane g builds the 16-byte core-matrix rows of 8-ray groups g, g + 32, ...
// (high and low BF16 parts); the row sum adds the parts group by group and
// then across lanes in a fixed shuffle order, so it is deterministic.
__device__ __forceinline__ void tc_weight_row(uint32_t row, uint32_t lane, const float4* dirs, uint32_t R,
                                              uint32_t nc, uint32_t nd, float sharp, uint32_t Nc, uint32_t Nd,
                                              uint32_t nchunks, uint8_t* wout, float* rowsum) {
    if (row >= Nd + Nc) return;  // warp-uniform
    const bool colour = row >= Nd;
    const uint32_t t = colour ? row - Nd : row;
    const uint32_t n = colour ? nc : nd;
    const bool valid = t < n * n;
    float3 td = f3(0, 0, 0);
    if (valid) {
        float sc = texel_scale(n), ce = 0.5f * (float)(n - 1);
        td = oct_decode(sc * ((float)(t % n) - ce), sc * ((float)(t / n) - ce));
    }
    const size_t part_bytes = (size_t)(Nd + Nc) * 128;  // one chunk of one part
    const uint32_t groups = nchunks * (kKChunk / 8);
    float sum = 0.0f;
    for (uint32_t gidx = lane; gidx < groups; gidx += 32) {
        uint32_t hw[4], lw[4];
        float part = 0.0f;
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
            float w2[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t r = gidx * 8 + e + h;
                float w = 0.0f;
                if (valid && r < R) {
                    float4 d = dirs[r];
                    float c = fmaxf(0.0f, td.x * d.x + td.y * d.y + td.z * d.z);
                    w = colour ? c : powf(c, sharp);
                }
                w2[h] = w;
            }
            __nv_bfloat162 hi = __floats2bfloat162_rn(w2[0], w2[1]);
            float2 hf = __bfloat1622float2(hi);
            __nv_bfloat162 lo = __floats2bfloat162_rn(w2[0] - hf.x, w2[1] - hf.y);
            float2 lf = __bfloat1622float2(lo);
            part += hf.x + lf.x;
            part += hf.y + lf.y;
            hw[e / 2] = *reinterpret_cast<uint32_t*>(&hi);
            lw[e / 2] = *reinterpret_cast<uint32_t*>(&lo);
        }
        sum += part;
        const uint32_t c = gidx / (kKChunk / 8), kg = gidx % (kKChunk / 8);
        const size_t off = (size_t)c * 2 * part_bytes + (colour ? (size_t)Nd * 128 : 0) + canon_off(t, kg);
        *reinterpret_cast<uint4*>(wout + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4*>(wout + off + part_bytes) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) rowsum[row] = sum;
}

// One warp per row, four rows per block.
__global__ void k_tc_weights(const float4* dirs, uint32_t R, uint32_t nc, uint32_t nd, float sharp, uint32_t Nc,
                             uint32_t Nd, uint32_t nchunks, uint8_t* wout, float* rowsum) {
    tc_weight_row(blockIdx.x * 4 + (threadIdx.x >> 5), threadIdx.x & 31, dirs, R, nc, nd, sharp, Nc, Nd, nchunks,
                  wout, rowsum);
}

// Blend of the 32-probe tile starting at probe slot p0 (< nprobes) by the
// whole CTA.
// Scale of a probe's colour records before the BF16 split: the power of two
// 2^e >= the largest radiance (so scaled records are <= 1 and the scaling
// is exact), e clamped to [-100, 100]; a probe whose largest radiance is
// below 2^-100 (zero, denormal) keeps scale 1, so the reciprocal is always
// finite and a zero record never meets an infinite one (0 x inf = NaN).
__device__ __forceinline__ float radiance_scale(float mx) {
    if (!(mx >= 0x1p-100f)) return 1.0f;  // also NaN
    int e = 100;
    if (mx < 0x1p100f) frexpf(mx, &e);
    return ldexpf(1.0f, e);
}

__device__ __forceinline__ void blend_tc_tile(const TcArgs& a, const uint32_t p0, const uint32_t nprobes) {
    extern __shared__ __align__(1024) uint8_t smem[];
    // A operands (128 x 64 BF16 = 16 KB each): colour hi/lo, depth hi/lo;
    // then B: high parts of (Nd + Nc) x 64, then the remainders
    uint8_t* sA_c = smem;
    uint8_t* sA_cl = smem + 16384;
    uint8_t* sA_d = smem + 32768;
    uint8_t* sA_dl = smem + 49152;
    uint8_t* sB = smem + 65536;
    __shared__ uint64_t s_bar;
    __shared__ uint32_t s_tmem;
    __shared__ float s_max[kTileProbes];  // per-probe colour scale (radiance_scale)
    __shared__ uint32_t s_oor[kTileProbes], s_maxc[kTileProbes];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t np = min((uint32_t)kTileProbes, nprobes - p0);
    const uint32_t R = a.g.rays;
    const float cell = a.g.cell_len;

    if (warp == 0) tc::tmem_alloc(&s_tmem, kTmemCols);
    if (tid == 0) tc::mbar_init(&s_bar, 1);
    if (tid < kTileProbes) s_maxc[tid] = 0u;
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = s_tmem;

    // pass 1: per-probe radiance maximum and out-of-range count
    for (int q = 0; q < kTileProbes / 8; ++q) {
        uint32_t pl = warp * (kTileProbes / 8) + q;
        float mx = 0.0f;
        uint32_t oor = 0;
        if (pl < np) {
            const float4* pr = a.rays + (size_t)(p0 + pl) * R;
#pragma unroll 8
            for (uint32_t r = lane; r < R; r += 32) {  // unrolled: eight loads in flight per lane
                float4 v = pr[r];
                mx = fmaxf(mx, fmaxf(v.x, fmaxf(v.y, v.z)));
                if (v.w < 0.0f || v.w > cell) ++oor;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            oor += __shfl_xor_sync(0xffffffffu, oor, o);
        }
        if (lane == 0) {
            s_max[pl] = radiance_scale(mx);
            s_oor[pl] = oor;
        }
    }
    __syncthreads();

    const uint32_t idc = tc::idesc_bf16_f32(128, a.Nc), idd = tc::idesc_bf16_f32(128, a.Nd);
    const size_t chunk16 = 2 * (size_t)(a.Nd + a.Nc) * 128 / 16;  // both parts
    bool ok = true;
    uint32_t phase = 0;
    for (uint32_t c = 0; c < a.nchunks; ++c) {
        {   // B: this chunk of both weight matrices, copied while A is built
            // (the previous chunk's MMAs have completed: its wait ended the
            // last iteration)
            const uint4* src = a.wchunks + (size_t)c * chunk16;
            uint4* dst = reinterpret_cast<uint4*>(sB);
            for (uint32_t i = tid; i < chunk16; i += kThreads) tc::cp_async16(dst + i, src + i);
        }
        {   // A: thread = (probe, group of 8 rays); one 16-byte core-matrix row per operand row
            const uint32_t pl = (uint32_t)tid >> 3, j = (uint32_t)tid & 7u;
            const float inv = 1.0f / s_max[pl];  // a power of two: exact
            const float cinv = 1.0f / cell;
            // [row][hi/lo][4 words of 2 BF16]: rows r, g, b (colour), d, d^2 (depth)
            uint32_t w[5][2][4];
#pragma unroll
            for (int e = 0; e < 8; e += 2) {
                float4 v[2];
                float dn[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint32_t r = c * kKChunk + j * 8 + e + h;
                    bool valid = pl < np && r < R;
                    v[h] = valid ? a.rays[(size_t)(p0 + pl) * R + r] : make_float4(0, 0, 0, 0);
                    float dep = fminf(cell, v[h].w);
                    if (dep < 0.0f) dep = cell;
                    dn[h] = valid ? dep * cinv : 0.0f;
                }
                w[0][0][e / 2] = pack2(v[0].x * inv, v[1].x * inv, &w[0][1][e / 2]);
                w[1][0][e / 2] = pack2(v[0].y * inv, v[1].y * inv, &w[1][1][e / 2]);
                w[2][0][e / 2] = pack2(v[0].z * inv, v[1].z * inv, &w[2][1][e / 2]);
                w[3][0][e / 2] = pack2(dn[0], dn[1], &w[3][1][e / 2]);
                w[4][0][e / 2] = pack2(dn[0] * dn[0], dn[1] * dn[1], &w[4][1][e / 2]);
            }
            const uint4 z = make_uint4(0, 0, 0, 0);
#pragma unroll
            for (int part = 0; part < 2; ++part) {
                uint8_t* ac = part ? sA_cl : sA_c;
                uint8_t* ad = part ? sA_dl : sA_d;
#pragma unroll
                for (int ch = 0; ch < 3; ++ch)
                    *reinterpret_cast<uint4*>(ac + canon_off(pl * 4 + ch, j)) =
                        make_uint4(w[ch][part][0], w[ch][part][1], w[ch][part][2], w[ch][part][3]);
                *reinterpret_cast<uint4*>(ac + canon_off(pl * 4 + 3, j)) = z;
                *reinterpret_cast<uint4*>(ad + canon_off(pl * 4 + 0, j)) =
                    make_uint4(w[3][part][0], w[3][part][1], w[3][part][2], w[3][part][3]);
                *reinterpret_cast<uint4*>(ad + canon_off(pl * 4 + 1, j)) =
                    make_uint4(w[4][part][0], w[4][part][1], w[4][part][2], w[4][part][3]);
                *reinterpret_cast<uint4*>(ad + canon_off(pl * 4 + 2, j)) = z;
                *reinterpret_cast<uint4*>(ad + canon_off(pl * 4 + 3, j)) = z;
            }
        }
        tc::cp_async_wait_all();
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0 && !a.stall) {
            tc::fence_after_sync();
            const uint32_t part = (a.Nd + a.Nc) * 128;
            const uint32_t aC = tc::smem_u32(sA_c), aCl = tc::smem_u32(sA_cl);
            const uint32_t aD = tc::smem_u32(sA_d), aDl = tc::smem_u32(sA_dl);
            const uint32_t bD = tc::smem_u32(sB), bC = bD + a.Nd * 128;
            // hi*hi + hi*lo + lo*hi, K = 16 per instruction
            const uint32_t ac_[3] = {aC, aC, aCl}, ad_[3] = {aD, aD, aDl};
            const uint32_t bo_[3] = {0u, part, 0u};
#pragma unroll
            for (uint32_t ks = 0; ks < kKChunk / 16; ++ks) {
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    uint32_t acc = (c > 0 || ks > 0 || q > 0) ? 1u : 0u;
                    tc::mma_bf16(tmem + 0, tc::smem_desc(ac_[q] + ks * 256, kLBO, kSBO),
                                 tc::smem_desc(bC + bo_[q] + ks * 256, kLBO, kSBO), idc, acc);
                    tc::mma_bf16(tmem + kDepthCol, tc::smem_desc(ad_[q] + ks * 256, kLBO, kSBO),
                                 tc::smem_desc(bD + bo_[q] + ks * 256, kLBO, kSBO), idd, acc);
                }
            }
            tc::commit(&s_bar);
        }
        __syncwarp();
        bool done = tc::mbar_wait(&s_bar, phase, kWaitLimitNs);
        phase ^= 1u;
        tc::fence_after_sync();
        if (!__syncthreads_and(done)) {
            ok = false;
            break;
        }
    }

    if (!ok) {
        // the MMAs did not complete in time: record it, give them one more,
        // longer bounded wait (a stall of the issuing thread means no MMA is
        // in flight; a preempted CTA's MMAs finish once it runs again), then
        // release the tensor memory: a CTA must not exit holding it
        if (tid == 0) raise_error(a.err, DEV_WAIT_TIMEOUT);
        if (!a.stall) tc::mbar_wait(&s_bar, phase ^ 1u, kDrainLimitNs);  // the stall hook issued none
    } else {
        // epilogue 1: accumulators -> shared staging (the operand buffers are free now)
        float* S_c = reinterpret_cast<float*>(smem);                        // [32][nc*nc][3]
        float* S_d = S_c + kTileProbes * a.nc * a.nc * 3;                    // [32][nd*nd][2]
        const uint32_t quarter = (uint32_t)warp & 3u;
        const uint32_t row = quarter * 32u + (uint32_t)lane;
        const uint32_t pl = row >> 2, ch = row & 3u;
        const uint32_t lane_base = tmem + ((quarter * 32u) << 16);
        const float scale_c = s_max[pl];
        if (warp < 4) {
            const uint32_t ntex = a.nc * a.nc;
            for (uint32_t col0 = 0; col0 < a.Nc; col0 += 16) {
                float v[16];
                tc::tmem_ld16(lane_base + col0, v);
                if (ch < 3 && pl < np) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        uint32_t t = col0 + i;
                        if (t < ntex) {
                            float s = a.rowsum[a.Nd + t];
                            float val = v[i] * scale_c;
                            if (s > 1e-3f) val /= s;
                            S_c[(pl * ntex + t) * 3 + ch] = val;
                        }
                    }
                }
            }
        } else {
            const uint32_t ntex = a.nd * a.nd;
            const float unscale = ch == 0 ? cell : cell * cell;
            for (uint32_t col0 = 0; col0 < a.Nd; col0 += 16) {
                float v[16];
                tc::tmem_ld16(lane_base + kDepthCol + col0, v);
                if (ch < 2 && pl < np) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        uint32_t t = col0 + i;
                        if (t < ntex) {
                            float s = a.rowsum[t];
                            float val = v[i] * unscale;
                            if (s > 1e-3f) val /= s;
                            S_d[(pl * ntex + t) * 2 + ch] = val;
                        }
                    }
                }
            }
        }
        __syncthreads();

        // epilogue 2: hysteresis in the FP32 accumulator, FP16 publish
        const float hy = a.hyst_dev ? *a.hyst_dev : a.g.hyst;
        const uint32_t rx = (uint32_t)a.g.res[0], rxy = (uint32_t)(a.g.res[0] * a.g.res[1]);
        const uint32_t ntc = a.nc * a.nc, ntd = a.nd * a.nd;
        const uint32_t nprobes_grid = rxy * (uint32_t)a.g.res[2];
        for (uint32_t i = tid; i < np * (ntc + ntd); i += kThreads) {
            uint32_t pl2 = i / (ntc + ntd), t = i % (ntc + ntd);
            uint32_t probe = a.probe_list ? a.probe_list[p0 + pl2] : p0 + pl2;
            if (probe >= nprobes_grid) {  // a probe list entry outside the grid
                raise_error(a.err, DEV_BAD_INDEX);
                continue;
            }
            int ix = (int)(probe % rx), iy = (int)((probe % rxy) / rx), iz = (int)(probe / rxy);
            int tile = iy * a.g.res[0] + ix;
            if (t < ntc) {
                uint32_t tx = t % a.nc, ty = t / a.nc;
                size_t px = (size_t)((int)a.g.color_res * tile + 1 + (int)tx);
                size_t py = (size_t)((int)a.g.color_res * iz + 1 + (int)ty);
                size_t ti = py * a.g.color_w + px;
                float4 prev = a.acc_color[ti];
                const float* res = S_c + (pl2 * ntc + t) * 3;
                float mc = fmaxf(fmaxf(fabsf(res[0] - prev.x), fabsf(res[1] - prev.y)), fabsf(res[2] - prev.z));
                atomicMax(&s_maxc[pl2], __float_as_uint(mc));
                float4 nv = make_float4(res[0] * (1.0f - hy) + prev.x * hy, res[1] * (1.0f - hy) + prev.y * hy,
                                        res[2] * (1.0f - hy) + prev.z * hy, 1.0f);
                a.acc_color[ti] = nv;
                a.color[ti] = float4_to_half4(nv.x, nv.y, nv.z, nv.w);
            } else {
                uint32_t u = t - ntc, tx = u % a.nd, ty = u / a.nd;
                size_t px = (size_t)((int)a.g.depth_res * tile + 1 + (int)tx);
                size_t py = (size_t)((int)a.g.depth_res * iz + 1 + (int)ty);
                size_t ti = py * a.g.depth_w + px;
                float2 prev = a.acc_depth[ti];
                const float* res = S_d + (pl2 * ntd + u) * 2;
                float2 nv = make_float2(res[0] * (1.0f - hy) + prev.x * hy, res[1] * (1.0f - hy) + prev.y * hy);
                a.acc_depth[ti] = nv;
                __half2 o = __floats2half2_rn(nv.x, nv.y);
                a.depth[ti] = *reinterpret_cast<uint32_t*>(&o);
            }
        }
        __syncthreads();

        // border copy (probesCopyBorders.comp, generalised) and probe state
        const int ncr = (int)a.g.color_res, ndr = (int)a.g.depth_res;
        const uint32_t nbc = 4 + 4 * (uint32_t)(ncr - 2), nbd = 4 + 4 * (uint32_t)(ndr - 2);
        for (uint32_t i = tid; i < np * (nbc + nbd); i += kThreads) {
            uint32_t pl2 = i / (nbc + nbd), e = i % (nbc + nbd);
            uint32_t probe = a.probe_list ? a.probe_list[p0 + pl2] : p0 + pl2;
            if (probe >= nprobes_grid) continue;
            int ix = (int)(probe % rx), iy = (int)((probe % rxy) / rx), iz = (int)(probe / rxy);
            int tile = iy * a.g.res[0] + ix;
            if (e < nbc) {
                int4 b = border_entry((int)e, ncr);
                size_t ox = (size_t)ncr * tile, oy = (size_t)ncr * iz;
                a.color[(oy + b.y) * a.g.color_w + ox + b.x] = a.color[(oy + b.w) * a.g.color_w + ox + b.z];
            } else {
                int4 b = border_entry((int)(e - nbc), ndr);
                size_t ox = (size_t)ndr * tile, oy = (size_t)ndr * iz;
                a.depth[(oy + b.y) * a.g.depth_w + ox + b.x] = a.depth[(oy + b.w) * a.g.depth_w + ox + b.z];
            }
        }
        uint32_t probe_t = (uint32_t)tid < np ? (a.probe_list ? a.probe_list[p0 + tid] : p0 + tid) : nprobes_grid;
        if (probe_t < nprobes_grid) {  // probesUpdate.glsl:110-119
            uint32_t probe = probe_t;
            uint32_t s = a.states[probe];
            if (s_oor[tid] >= R) {
                s = 8;
            } else {
                float mc = __uint_as_float(s_maxc[tid]);
                float sf = (float)s;
                if (mc < 0.02f / sf) s = min(s + 1u, 8u);
                else if (mc > 0.04f / sf) s = max(s - 1u, 1u);
                else if (mc > 0.25f) s = 1;
            }
            a.states[probe] = s;
        }
    }

    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, kTmemCols);
    }
}

__global__ void __launch_bounds__(kThreads) k_blend_tc(TcArgs a) {
    const uint32_t n = a.dev_count ? *a.dev_count : a.nprobes;
    const uint32_t p0 = blockIdx.x * kTileProbes;
    if (p0 >= n) return;  // whole CTA, before any tensor-memory allocation
    blend_tc_tile(a, p0, n);
}

// Interior sides, padded texel counts and ray chunks of a grid.
struct TcShape {
    uint32_t nc, nd, Nc, Nd, nchunks;
};
__host__ __device__ __forceinline__ TcShape tc_shape(const DeviceGrid& g) {
    TcShape t;
    t.nc = g.color_res - 2;
    t.nd = g.depth_res - 2;
    t.Nc = (t.nc * t.nc + 15) / 16 * 16;
    t.Nd = (t.nd * t.nd + 15) / 16 * 16;
    t.nchunks = (g.rays + kKChunk - 1) / kKChunk;
    return t;
}

// Batched weights: blockIdx.y picks the volume of the list.
__global__ void k_batch_tc_weights(BatchTables bt, BatchBlendList bl) {
    const BatchVolume& vol = bt.vols[__ldg(bl.list + blockIdx.y)];
    const TcShape t = tc_shape(vol.g);
    tc_weight_row(blockIdx.x * 4 + (threadIdx.x >> 5), threadIdx.x & 31, bt.dirs + vol.dir_base, vol.g.rays, t.nc,
                  t.nd, vol.g.sharp, t.Nc, t.Nd, t.nchunks, vol.wbuf, vol.rowsum);
}

// Batched blend: CTA b takes tile (b - tile_base[i]) of volume list[i]; the
// CTA that finishes a volume's last tile stamps its completion time.
__global__ void __launch_bounds__(kThreads) k_batch_blend_tc(BatchTables bt, BatchBlendList bl,
                                                             const float4* __restrict__ rays) {
    __shared__ TcArgs s_args;
    __shared__ uint32_t s_v, s_tile, s_items;
    if (threadIdx.x == 0) {
        uint32_t lo = 0, hi = bl.n;  // tile_base[lo] <= b < tile_base[hi]
        const uint32_t b = blockIdx.x;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (__ldg(bl.tile_base + mid) <= b) lo = mid;
            else hi = mid;
        }
        const uint32_t v = __ldg(bl.list + lo);
        const BatchVolume& vol = bt.vols[v];
        const TcShape t = tc_shape(vol.g);
        TcArgs& a = s_args;
        a.g = vol.g;
        a.probe_list = nullptr;
        a.nprobes = (uint32_t)vol.g.res[0] * (uint32_t)vol.g.res[1] * (uint32_t)vol.g.res[2];
        a.rays = rays + vol.ray_base;
        a.wchunks = reinterpret_cast<const uint4*>(vol.wbuf);
        a.rowsum = vol.rowsum;
        a.nc = t.nc;
        a.nd = t.nd;
        a.Nc = t.Nc;
        a.Nd = t.Nd;
        a.nchunks = t.nchunks;
        a.states = vol.states;
        a.color = static_cast<uint2*>(vol.color);
        a.depth = static_cast<uint32_t*>(vol.depth);
        a.acc_color = vol.acc_color;
        a.acc_depth = vol.acc_depth;
        a.err = bt.err;
        a.dev_count = nullptr;
        a.stall = 0;
        a.hyst_dev = nullptr;
        s_v = v;
        s_tile = b - __ldg(bl.tile_base + lo);
        s_items = __ldg(bl.tile_base + lo + 1) - __ldg(bl.tile_base + lo);
    }
    __syncthreads();
    blend_tc_tile(s_args, s_tile * kTileProbes, s_args.nprobes);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(bt.done + s_v, 1u) == s_items - 1u) bt.clock[1 + s_v] = globaltimer_ns();
    }
}

// Shared-memory limit of both blend kernels on the current device.
cudaError_t set_tc_smem_limit() {
    cudaError_t e = ensure_dynamic_smem(k_blend_tc, 200 * 1024);
    if (e == cudaSuccess) e = ensure_dynamic_smem(k_batch_blend_tc, 200 * 1024);
    return e;
}

}  // namespace

size_t tc_weight_bytes(uint32_t rays, uint32_t color_res, uint32_t depth_res) {
    uint32_t nc = color_res - 2, nd = depth_res - 2;
    uint32_t Nc = (nc * nc + 15) / 16 * 16, Nd = (nd * nd + 15) / 16 * 16;
    uint32_t nchunks = (rays + kKChunk - 1) / kKChunk;
    return (size_t)nchunks * 2 * (Nc + Nd) * 128;
}

bool tc_blend_supported(uint32_t color_res, uint32_t depth_res) {
    uint32_t nc = color_res - 2, nd = depth_res - 2;
    return nc * nc <= 256 && nd * nd <= 256 && nc >= 1 && nd >= 1;
}

cudaError_t launch_blend_tc(const DeviceGrid& g, const uint32_t* probe_list, uint32_t nprobes, const float4* rays,
                            const float4* dirs, uint8_t* wbuf, float* rowsum, uint32_t* states, void* color,
                            void* depth, float4* acc_color, float2* acc_depth, uint32_t* err, cudaStream_t st,
                            const uint32_t* dev_count, bool stall, const float* hyst_dev) {
    if (nprobes == 0) return cudaSuccess;
    const uint32_t nc = g.color_res - 2, nd = g.depth_res - 2;
    const uint32_t Nc = (nc * nc + 15) / 16 * 16, Nd = (nd * nd + 15) / 16 * 16;
    const uint32_t nchunks = (g.rays + kKChunk - 1) / kKChunk;
    k_tc_weights<<<(Nd + Nc + 3) / 4, 128, 0, st>>>(dirs, g.rays, nc, nd, g.sharp, Nc, Nd, nchunks, wbuf, rowsum);
    TcArgs a;
    a.g = g;
    a.probe_list = probe_list;
    a.nprobes = nprobes;
    a.rays = rays;
    a.wchunks = reinterpret_cast<const uint4*>(wbuf);
    a.rowsum = rowsum;
    a.nc = nc;
    a.nd = nd;
    a.Nc = Nc;
    a.Nd = Nd;
    a.nchunks = nchunks;
    a.states = states;
    a.color = static_cast<uint2*>(color);
    a.depth = static_cast<uint32_t*>(depth);
    a.acc_color = acc_color;
    a.acc_depth = acc_depth;
    a.err = err;
    a.dev_count = dev_count;
    a.stall = stall ? 1u : 0u;
    a.hyst_dev = hyst_dev;
    // operand stage (A 64 KB + B up to 128 KB), reused by the epilogue staging
    size_t stage = 65536 + 2 * (size_t)(Nd + Nc) * 128;
    size_t staging = (size_t)kTileProbes * (nc * nc * 3 + nd * nd * 2) * sizeof(float);
    size_t smem = stage > staging ? stage : staging;
    if (smem < kMinSmem) smem = kMinSmem;
    cudaError_t e = set_tc_smem_limit();
    if (e != cudaSuccess) return e;
    uint32_t blocks = (nprobes + kTileProbes - 1) / kTileProbes;
    k_blend_tc<<<blocks, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

uint32_t tc_tiles(uint32_t nprobes) { return (nprobes + kTileProbes - 1) / kTileProbes; }

cudaError_t prepare_batch_kernels() {
    cudaError_t e = set_tc_smem_limit();
    return e == cudaSuccess ? set_shared_smem_limit() : e;
}

size_t batch_tc_smem(uint32_t color_res, uint32_t depth_res) {
    const uint32_t nc = color_res - 2, nd = depth_res - 2;
    const uint32_t Nc = (nc * nc + 15) / 16 * 16, Nd = (nd * nd + 15) / 16 * 16;
    size_t stage = 65536 + 2 * (size_t)(Nd + Nc) * 128;
    size_t staging = (size_t)kTileProbes * (nc * nc * 3 + nd * nd * 2) * sizeof(float);
    size_t smem = stage > staging ? stage : staging;
    return smem < kMinSmem ? kMinSmem : smem;
}

cudaError_t launch_batch_tc_weights(const BatchTables& bt, const BatchBlendList& bl, uint32_t max_rows,
                                    cudaStream_t st) {
    if (bl.n == 0) return cudaSuccess;
    k_batch_tc_weights<<<dim3((max_rows + 3) / 4, bl.n), 128, 0, st>>>(bt, bl);
    return cudaGetLastError();
}

cudaError_t launch_batch_blend_tc(const BatchTables& bt, const BatchBlendList& bl, const float4* rays, size_t smem,
                                  cudaStream_t st) {
    if (bl.ntiles == 0) return cudaSuccess;
    cudaError_t e = set_tc_smem_limit();
    if (e != cudaSuccess) return e;
    k_batch_blend_tc<<<bl.ntiles, kThreads, smem, st>>>(bt, bl, rays);
    return cudaGetLastError();
}

}  // namespace ddgi

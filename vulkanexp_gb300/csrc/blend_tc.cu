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
// Tiling: a CTA takes up to 25 probes (the launch picks the tile size that
// fills the SMs' CTA slots best); each probe owns 5 rows of the A operand
// (its ray records' r, g, b, clamped depth d and d^2), so A is M = 128 rows
// (the rest zero) x K rays, K-major, and the weights are B: the depth rows then the
// colour rows (each texel count padded to 16), N = Nd + Nc <= 256 in one
// accumulator at tensor-memory column 0 (wider tiles: depth at 0, colour at
// 256, in two MMAs).  Only the row x column pairs of matching kind are read
// back; the rest of the product is the price of one MMA per K step, cheap in
// this memory-bound kernel.  K is processed in chunks of 16 rays (one MMA K
// step) staged as BF16 in a ring of four shared-memory stages; both operands
// are split into a BF16 high part and a BF16 remainder (x = hi + lo) and
// three products hi*hi + hi*lo + lo*hi are accumulated (~16 mantissa bits,
// below the FP16 atlas store's rounding; BF16 keeps FP32's exponent range,
// so no scaling is needed).  One thread issues tcgen05.mma (M = 128,
// K = 16); while a chunk's MMAs run, the next chunks' weights arrive by
// cp.async and their records into registers.  With 256 accumulator columns
// two CTAs share an SM.  The epilogue reads the accumulators with
// tcgen05.ld, normalises (times the reciprocal row sums) through shared
// memory into texel order, applies hysteresis in the FP32 accumulators
// (previous values loaded eight per thread at a time), stores FP16 texels
// together with the border texels that copy them, and updates the probe
// states.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "tc.cuh"

namespace ddgi {

namespace {

constexpr int kTileProbes = 25;    // 5 A rows per probe: (r, g, b, d, d^2); at most 25 (128 rows)
constexpr int kRowsPerProbe = 5;
constexpr int kKChunk = 16;        // rays per shared-memory stage (one K step)
constexpr int kStages = 4;         // operand stages in the ring
constexpr int kThreads = 256;
constexpr uint32_t kSBO = (kKChunk / 8) * 128;  // bytes between 8-row groups
constexpr uint32_t kLBO = 128;                  // bytes between K-adjacent core matrices
constexpr uint32_t kAPart = 128 * kKChunk * 2;  // one BF16 part of the A stage (128 rows)
// A CTA whose texels need more than 256 accumulator columns allocates all
// 512 of its SM's: its shared-memory request is then at least this much, so
// no second CTA shares the SM (two exceed the SM's 228 KB).
constexpr size_t kOneCtaSmem = 120 * 1024;

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
    uint32_t tile;              // probes per CTA (1 .. kTileProbes)
    uint32_t smem_bytes;        // dynamic shared memory of the launch
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
    const size_t part_bytes = (size_t)(Nd + Nc) * (kKChunk * 2);  // one chunk of one part
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
        const size_t off = (size_t)c * 2 * part_bytes + (colour ? (size_t)Nd * (kKChunk * 2) : 0) + canon_off(t, kg);
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

// Calls put(bx, by) for each border texel of a tile of side n that copies
// interior texel (x, y), 1 <= x, y <= n - 2 (probesCopyBorders.comp:21-245,
// generalised: the inverse of border_entry in common.cuh); up to 8 for n = 3,
// 3 otherwise.
template <class F>
__device__ __forceinline__ void for_border_targets(int x, int y, int n, F put) {
    if (x == 1) put(0, n - 1 - y);
    if (x == n - 2) put(n - 1, n - 1 - y);
    if (y == 1) put(n - 1 - x, 0);
    if (y == n - 2) put(n - 1 - x, n - 1);
    if (x == n - 2 && y == n - 2) put(0, 0);
    if (x == n - 2 && y == 1) put(0, n - 1);
    if (x == 1 && y == n - 2) put(n - 1, 0);
    if (x == 1 && y == 1) put(n - 1, n - 1);
}

// Shared-memory layout of a tile: a ring of kStages operand stages, each the
// A operand of one chunk (hi part, lo part) then its B operand (hi, lo);
// chunk c uses stage c % kStages.  The epilogue staging reuses the ring.
__host__ __device__ __forceinline__ size_t tc_b_bytes(uint32_t Nd, uint32_t Nc) { return 2 * (size_t)(Nd + Nc) * (kKChunk * 2); }
__host__ __device__ __forceinline__ size_t tc_stage_bytes(uint32_t Nd, uint32_t Nc) {
    return 2 * (size_t)kAPart + tc_b_bytes(Nd, Nc);
}

// Dynamic shared memory of a tile: the operand ring or the epilogue
// staging, whichever is larger; with more than 256 accumulator columns at
// least kOneCtaSmem (one CTA per SM).
__host__ __device__ __forceinline__ size_t tc_staging_bytes(uint32_t nc, uint32_t nd) {
    return ((size_t)kTileProbes * (nc * nc * 3 + nd * nd * 2) * sizeof(float) + 15) / 16 * 16;
}
// The published FP16 tiles of the CTA's probes, border texels included,
// assembled after the staging so that they leave in whole rows.
__host__ __device__ __forceinline__ size_t tc_color_tiles_bytes(uint32_t nc) {
    return ((size_t)kTileProbes * (nc + 2) * (nc + 2) * 8 + 15) / 16 * 16;
}
__host__ __device__ __forceinline__ size_t tc_tiles_bytes(uint32_t nc, uint32_t nd) {
    return tc_color_tiles_bytes(nc) + (size_t)kTileProbes * (nd + 2) * (nd + 2) * 4;
}
// Largest request that still lets two CTAs share an SM (228 KB, of which
// each CTA also holds ~3 KB of static shared memory and 1 KB reserved).
constexpr size_t kTwoCtaSmem = 108 * 1024;

__host__ __device__ __forceinline__ size_t tc_smem_bytes(uint32_t nc, uint32_t nd, uint32_t Nc, uint32_t Nd) {
    const size_t ring = kStages * tc_stage_bytes(Nd, Nc);
    const size_t staging = tc_staging_bytes(nc, nd), with_tiles = staging + tc_tiles_bytes(nc, nd);
    const bool wide = Nd + Nc > 256;
    size_t smem = ring > staging ? ring : staging;
    // the tile images where they fit without losing the second CTA per SM
    // (or beside a wide tile's single CTA)
    if (with_tiles > smem && with_tiles <= (wide ? (size_t)200 * 1024 : kTwoCtaSmem)) smem = with_tiles;
    if (wide && smem < kOneCtaSmem) smem = kOneCtaSmem;
    return smem;
}

// Blend of the tile of a.tile probe slots starting at p0 (< nprobes) by the
// whole CTA.  Iteration c fills stage c % kStages with chunk c (weights
// by cp.async, ray operands from registers loaded two iterations before) and
// issues the MMAs of chunk c - 1, whose weights were copied one iteration
// before; a stage is refilled once the MMAs that read it (kStages chunks
// earlier) have signalled its barrier.
__device__ __forceinline__ void blend_tc_tile(const TcArgs& a, const uint32_t p0, const uint32_t nprobes) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t s_bar[kStages];
    __shared__ uint32_t s_tmem;
    __shared__ uint32_t s_oor[kTileProbes], s_maxc[kTileProbes];
    __shared__ float s_rinv[512];       // 1 / row sum of the weights (1 where the sum is <= 1e-3)
    __shared__ int2 s_org[kTileProbes];  // atlas tile (x, y) of each probe, in tiles; x < 0: none

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t np = min(a.tile, nprobes - p0);
    const uint32_t R = a.g.rays;
    const float cell = a.g.cell_len;
    const bool split = a.Nd + a.Nc > 256;        // two accumulators: depth at column 0, colour at 256
    const uint32_t cols = split ? 512u : 256u;
    const uint32_t cbase = split ? 256u : a.Nd;  // first colour column
    const size_t bbytes = tc_b_bytes(a.Nd, a.Nc);
    const size_t sbytes = tc_stage_bytes(a.Nd, a.Nc);
    const uint32_t b16 = (uint32_t)(bbytes / 16);
    auto stage_a = [&](uint32_t c) { return smem + (c % kStages) * sbytes; };
    auto stage_b = [&](uint32_t c) { return smem + (c % kStages) * sbytes + 2 * kAPart; };

    if (warp == 0) tc::tmem_alloc(&s_tmem, cols);
    if (tid < kStages) tc::mbar_init(&s_bar[tid], 1);
    if (tid < kTileProbes) {
        s_maxc[tid] = 0u;
        s_oor[tid] = 0u;
        int2 o = make_int2(-1, -1);
        if ((uint32_t)tid < np) {
            const uint32_t rx = (uint32_t)a.g.res[0], rxy = (uint32_t)(a.g.res[0] * a.g.res[1]);
            const uint32_t probe = a.probe_list ? a.probe_list[p0 + tid] : p0 + tid;
            if (probe < rxy * (uint32_t)a.g.res[2]) {
                const int ix = (int)(probe % rx), iy = (int)((probe % rxy) / rx), iz = (int)(probe / rxy);
                o = make_int2(iy * a.g.res[0] + ix, iz);
            } else {
                raise_error(a.err, DEV_BAD_INDEX);  // a probe list entry outside the grid
            }
        }
        s_org[tid] = o;
    }
    for (uint32_t i = tid; i < a.Nd + a.Nc; i += kThreads) {
        const float sum = a.rowsum[i];
        s_rinv[i] = sum > 1e-3f ? 1.0f / sum : 1.0f;
    }
    // A rows tile * 5 .. 127 stay zero in every stage
    const uint32_t zrows = 128u - a.tile * kRowsPerProbe;
    for (uint32_t i = tid; i < kStages * 2 * zrows * (kKChunk / 8); i += kThreads) {
        const uint32_t kg = i % (kKChunk / 8), r = a.tile * kRowsPerProbe + (i / (kKChunk / 8)) % zrows;
        const uint32_t part = (i / (zrows * (kKChunk / 8))) % 2, st = i / (2 * zrows * (kKChunk / 8));
        *reinterpret_cast<uint4*>(smem + st * sbytes + part * kAPart + canon_off(r, kg)) = make_uint4(0, 0, 0, 0);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = s_tmem;

    // thread -> (probe, 2 consecutive rays of the chunk); 200 of 256 threads
    const uint32_t pl = (uint32_t)tid >> 3, j = (uint32_t)tid & 7u;
    const bool builder = pl < a.tile;
    const bool live = builder && pl < np;
    const float4* prec = a.rays + (size_t)(p0 + (live ? pl : 0u)) * R;
    float4 va[2], vb[2];  // records of the even / odd chunks in flight
    auto load = [&](float4* v, uint32_t c) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const uint32_t r = c * kKChunk + j * 2 + e;
            v[e] = live && r < R ? __ldg(prec + r) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    };
    load(va, 0);
    load(vb, 1);
    uint32_t oor = 0;
    const uint32_t N = a.Nd + a.Nc;
    const uint32_t id_all = tc::idesc_bf16_f32(128, N), id_d = tc::idesc_bf16_f32(128, a.Nd),
                   id_c = tc::idesc_bf16_f32(128, a.Nc);
    bool ok = true;
    uint32_t waited = 0;  // chunk whose MMAs a completion wait was for (the drain's target on a timeout)
    int last = -1;        // the last chunk whose MMAs were issued
    for (uint32_t c = 0; c <= a.nchunks; ++c) {
        if (c < a.nchunks) {
            if (c >= (uint32_t)kStages) {  // the MMAs of chunk c - kStages read this stage
                const uint32_t old = c - kStages;
                const bool done = tc::mbar_wait(&s_bar[old % kStages], (old / kStages) & 1u, kWaitLimitNs);
                tc::fence_after_sync();
                if (!__syncthreads_and(done)) {
                    ok = false;
                    waited = old;
                    break;
                }
            }
            {   // weights of chunk c
                const uint4* src = a.wchunks + (size_t)c * b16;
                uint4* dst = reinterpret_cast<uint4*>(stage_b(c));
                for (uint32_t i = tid; i < b16; i += kThreads) tc::cp_async16(dst + i, src + i);
                tc::cp_async_commit();
            }
            if (builder) {  // A rows (r, g, b, d, d^2) of this thread's probe, 2 rays: a quarter core-matrix row
                float4 v[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) v[e] = (c & 1u) ? vb[e] : va[e];
                float dep[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const uint32_t r = c * kKChunk + j * 2 + e;
                    const float wv = v[e].w;
                    if (live && r < R && (wv < 0.0f || wv > cell)) ++oor;
                    float dd = fminf(cell, wv);
                    if (dd < 0.0f) dd = cell;
                    dep[e] = live && r < R ? dd : 0.0f;
                }
                uint32_t w[5][2];
                w[0][0] = pack2(v[0].x, v[1].x, &w[0][1]);
                w[1][0] = pack2(v[0].y, v[1].y, &w[1][1]);
                w[2][0] = pack2(v[0].z, v[1].z, &w[2][1]);
                w[3][0] = pack2(dep[0], dep[1], &w[3][1]);
                w[4][0] = pack2(dep[0] * dep[0], dep[1] * dep[1], &w[4][1]);
                uint8_t* sa = stage_a(c);
#pragma unroll
                for (int part = 0; part < 2; ++part)
#pragma unroll
                    for (int ch = 0; ch < kRowsPerProbe; ++ch)
                        *reinterpret_cast<uint32_t*>(sa + part * kAPart +
                                                     canon_off(pl * kRowsPerProbe + ch, j >> 2) + (j & 3u) * 4u) =
                            w[ch][part];
            }
            if (c + 2 < a.nchunks) {  // records two chunks ahead
                if (c & 1u) load(vb, c + 2);
                else load(va, c + 2);
            }
        }
        if (c >= 1) {  // the MMAs of chunk c - 1 (its weights were copied an iteration ago)
            if (c < a.nchunks) tc::cp_async_wait_group<1>();
            else tc::cp_async_wait_group<0>();
            tc::fence_proxy_async();
            __syncthreads();
            const uint32_t m = c - 1;
            if (tid == 0 && !a.stall) {
                tc::fence_after_sync();
                const uint32_t aH = tc::smem_u32(stage_a(m)), aL = aH + kAPart;
                const uint32_t bH = tc::smem_u32(stage_b(m)), bL = bH + N * (kKChunk * 2);
                // hi*hi + hi*lo + lo*hi, K = 16 per instruction
                const uint32_t a_[3] = {aH, aH, aL}, b_[3] = {bH, bL, bH};
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const uint32_t acc = (m > 0 || q > 0) ? 1u : 0u;
                    const uint64_t ad = tc::smem_desc(a_[q], kLBO, kSBO);
                    if (!split) {
                        tc::mma_bf16(tmem, ad, tc::smem_desc(b_[q], kLBO, kSBO), id_all, acc);
                    } else {
                        tc::mma_bf16(tmem, ad, tc::smem_desc(b_[q], kLBO, kSBO), id_d, acc);
                        tc::mma_bf16(tmem + 256u, ad, tc::smem_desc(b_[q] + a.Nd * (kKChunk * 2), kLBO, kSBO), id_c,
                                     acc);
                    }
                }
                tc::commit(&s_bar[m % kStages]);
            }
            last = (int)m;
            __syncwarp();
        }
    }
    if (ok && last >= 0) {  // the last chunk's MMAs (a commit tracks every earlier MMA too)
        const uint32_t m = (uint32_t)last;
        const bool done = tc::mbar_wait(&s_bar[m % kStages], (m / kStages) & 1u, kWaitLimitNs);
        tc::fence_after_sync();
        ok = __syncthreads_and(done);
        waited = m;
    }
    if (live && oor) atomicAdd(&s_oor[pl], oor);

    if (!ok) {
        // the MMAs did not complete in time: record it, give them one more,
        // longer bounded wait (a stall of the issuing thread means no MMA is
        // in flight; a preempted CTA's MMAs finish once it runs again), then
        // release the tensor memory: a CTA must not exit holding it
        if (tid == 0) raise_error(a.err, DEV_WAIT_TIMEOUT);
        if (!a.stall && last >= 0) {  // the stall hook issued none
            const uint32_t m = (uint32_t)last;
            tc::mbar_wait(&s_bar[m % kStages], (m / kStages) & 1u, kDrainLimitNs);
        }
        (void)waited;
    } else {
        // epilogue 1: accumulators -> normalised values in shared staging,
        // texel-major: S_c[probe][texel][r, g, b], S_d[probe][texel][d, d^2]
        const uint32_t ntc = a.nc * a.nc, ntd = a.nd * a.nd;
        float* S_c = reinterpret_cast<float*>(smem);
        float* S_d = S_c + kTileProbes * ntc * 3;
        const uint32_t quarter = (uint32_t)warp & 3u;
        const uint32_t row = quarter * 32u + (uint32_t)lane;
        const uint32_t rp = row / kRowsPerProbe, ch = row % kRowsPerProbe;
        const bool rvalid = rp < np;
        const uint32_t lane_base = tmem + ((quarter * 32u) << 16);
        const uint32_t steps_d = a.Nd / 16, steps = steps_d + a.Nc / 16;
        for (uint32_t s = (uint32_t)warp >> 2; s < steps; s += 2) {  // warps w and w + 4 share the lanes
            const bool depth = s < steps_d;
            const uint32_t col0 = depth ? s * 16 : cbase + (s - steps_d) * 16;
            float vv[16];
            tc::tmem_ld16(lane_base + col0, vv);
            if (!rvalid) continue;
            if (depth && ch >= 3) {
                float* dst = S_d + rp * ntd * 2 + (ch - 3);
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const uint32_t u = s * 16 + i;
                    if (u < ntd) dst[u * 2] = vv[i] * s_rinv[u];
                }
            } else if (!depth && ch < 3) {
                float* dst = S_c + rp * ntc * 3 + ch;
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const uint32_t t = (s - steps_d) * 16 + i;
                    if (t < ntc) dst[t * 3] = vv[i] * s_rinv[a.Nd + t];
                }
            }
        }
        __syncthreads();

        // epilogue 2: hysteresis in the FP32 accumulators, FP16 publish of
        // each interior texel and of the border texels copied from it
        // (probesCopyBorders.comp); loads of the previous values are issued
        // eight at a time per thread.  Where they fit, the FP16 tiles are
        // assembled in shared memory first and leave in whole rows
        // (sector-aligned 16-byte stores instead of scattered texels).
        const size_t stg_bytes = tc_staging_bytes(a.nc, a.nd);
        const bool assemble = stg_bytes + tc_tiles_bytes(a.nc, a.nd) <= a.smem_bytes;
        uint2* Tc = reinterpret_cast<uint2*>(smem + stg_bytes);  // [probe][ncr x ncr]
        uint32_t* Td = reinterpret_cast<uint32_t*>(smem + stg_bytes + tc_color_tiles_bytes(a.nc));
        const float hy = a.hyst_dev ? *a.hyst_dev : a.g.hyst;
        const int ncr = (int)a.g.color_res, ndr = (int)a.g.depth_res;
        // item i -> (probe, texel) and texel -> (x, y) without integer
        // division: floor((i + 0.5) / n) in float is exact here (i < 2^13,
        // n <= 256: the product's error is far below the 0.5 / n margin)
        const float inv_ntc = 1.0f / (float)ntc, inv_ntd = 1.0f / (float)ntd;
        const float inv_nc = 1.0f / (float)a.nc, inv_nd = 1.0f / (float)a.nd;
        auto split_index = [](uint32_t i, uint32_t n, float inv, uint32_t* q) {
            *q = (uint32_t)(((float)i + 0.5f) * inv);
            return i - *q * n;
        };
        constexpr int kBatch = 8;
        const uint32_t items_c = np * ntc;
        for (uint32_t base = 0; base < items_c; base += kBatch * kThreads) {
            float4 prev[kBatch];
            size_t ti[kBatch];
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                const uint32_t i = base + (uint32_t)k * kThreads + (uint32_t)tid;
                ti[k] = ~(size_t)0;
                if (i < items_c) {
                    uint32_t pl2, ty;
                    const uint32_t t = split_index(i, ntc, inv_ntc, &pl2);
                    const uint32_t tx = split_index(t, a.nc, inv_nc, &ty);
                    const int2 o = s_org[pl2];
                    if (o.x >= 0) {
                        ti[k] = (size_t)(ncr * o.y + 1 + (int)ty) * a.g.color_w + (size_t)(ncr * o.x + 1 + (int)tx);
                        prev[k] = a.acc_color[ti[k]];
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                if (ti[k] == ~(size_t)0) continue;
                const uint32_t i = base + (uint32_t)k * kThreads + (uint32_t)tid;
                uint32_t pl2, ty;
                const uint32_t t = split_index(i, ntc, inv_ntc, &pl2);
                const uint32_t tx = split_index(t, a.nc, inv_nc, &ty);
                const float* res = S_c + (pl2 * ntc + t) * 3;
                const float mc = fmaxf(fmaxf(fabsf(res[0] - prev[k].x), fabsf(res[1] - prev[k].y)),
                                       fabsf(res[2] - prev[k].z));
                atomicMax(&s_maxc[pl2], __float_as_uint(mc));
                const float4 nv = make_float4(res[0] * (1.0f - hy) + prev[k].x * hy,
                                              res[1] * (1.0f - hy) + prev[k].y * hy,
                                              res[2] * (1.0f - hy) + prev[k].z * hy, 1.0f);
                a.acc_color[ti[k]] = nv;
                const uint2 hv = float4_to_half4(nv.x, nv.y, nv.z, nv.w);
                if (assemble) {
                    uint2* T = Tc + (size_t)pl2 * ncr * ncr;
                    T[((int)ty + 1) * ncr + (int)tx + 1] = hv;
                    for_border_targets((int)tx + 1, (int)ty + 1, ncr, [&](int bx, int by) { T[by * ncr + bx] = hv; });
                } else {
                    a.color[ti[k]] = hv;
                    const int2 o = s_org[pl2];
                    const int ox = ncr * o.x, oy = ncr * o.y;
                    for_border_targets((int)tx + 1, (int)ty + 1, ncr, [&](int bx, int by) {
                        a.color[(size_t)(oy + by) * a.g.color_w + (size_t)(ox + bx)] = hv;
                    });
                }
            }
        }
        const uint32_t items_d = np * ntd;
        for (uint32_t base = 0; base < items_d; base += kBatch * kThreads) {
            float2 prev[kBatch];
            size_t ti[kBatch];
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                const uint32_t i = base + (uint32_t)k * kThreads + (uint32_t)tid;
                ti[k] = ~(size_t)0;
                if (i < items_d) {
                    uint32_t pl2, ty;
                    const uint32_t u = split_index(i, ntd, inv_ntd, &pl2);
                    const uint32_t tx = split_index(u, a.nd, inv_nd, &ty);
                    const int2 o = s_org[pl2];
                    if (o.x >= 0) {
                        ti[k] = (size_t)(ndr * o.y + 1 + (int)ty) * a.g.depth_w + (size_t)(ndr * o.x + 1 + (int)tx);
                        prev[k] = a.acc_depth[ti[k]];
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                if (ti[k] == ~(size_t)0) continue;
                const uint32_t i = base + (uint32_t)k * kThreads + (uint32_t)tid;
                uint32_t pl2, ty;
                const uint32_t u = split_index(i, ntd, inv_ntd, &pl2);
                const uint32_t tx = split_index(u, a.nd, inv_nd, &ty);
                const float* res = S_d + (pl2 * ntd + u) * 2;
                const float2 nv = make_float2(res[0] * (1.0f - hy) + prev[k].x * hy, res[1] * (1.0f - hy) + prev[k].y * hy);
                a.acc_depth[ti[k]] = nv;
                const __half2 h2 = __floats2half2_rn(nv.x, nv.y);
                const uint32_t hv = *reinterpret_cast<const uint32_t*>(&h2);
                if (assemble) {
                    uint32_t* T = Td + (size_t)pl2 * ndr * ndr;
                    T[((int)ty + 1) * ndr + (int)tx + 1] = hv;
                    for_border_targets((int)tx + 1, (int)ty + 1, ndr, [&](int bx, int by) { T[by * ndr + bx] = hv; });
                } else {
                    a.depth[ti[k]] = hv;
                    const int2 o = s_org[pl2];
                    const int ox = ndr * o.x, oy = ndr * o.y;
                    for_border_targets((int)tx + 1, (int)ty + 1, ndr, [&](int bx, int by) {
                        a.depth[(size_t)(oy + by) * a.g.depth_w + (size_t)(ox + bx)] = hv;
                    });
                }
            }
        }
        __syncthreads();
        if (assemble) {  // the tiles out, row by row, 16 bytes per store where the rows allow
            // texels per store: uint4 where rows and the atlas allow it, else one texel
            const uint32_t cq = (ncr * 8) % 16 == 0 && (reinterpret_cast<uintptr_t>(a.color) & 15u) == 0 ? 2u : 1u;
            const uint32_t c_per_row = ncr / cq, c_items = np * ncr * c_per_row;
            for (uint32_t i = tid; i < c_items; i += kThreads) {
                const uint32_t p = i / (ncr * c_per_row), r = i % (ncr * c_per_row), y = r / c_per_row,
                               x = (r % c_per_row) * cq;
                const int2 o = s_org[p];
                if (o.x < 0) continue;
                const uint2* src = Tc + (size_t)p * ncr * ncr + y * ncr + x;
                uint2* dst = a.color + (size_t)(ncr * o.y + (int)y) * a.g.color_w + (size_t)(ncr * o.x + (int)x);
                if (cq == 2) *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(src);
                else *dst = *src;
            }
            const uint32_t dq = (ndr * 4) % 16 == 0 && (reinterpret_cast<uintptr_t>(a.depth) & 15u) == 0 ? 4u : 1u;
            const uint32_t d_per_row = ndr / dq, d_items = np * ndr * d_per_row;
            for (uint32_t i = tid; i < d_items; i += kThreads) {
                const uint32_t p = i / (ndr * d_per_row), r = i % (ndr * d_per_row), y = r / d_per_row,
                               x = (r % d_per_row) * dq;
                const int2 o = s_org[p];
                if (o.x < 0) continue;
                const uint32_t* src = Td + (size_t)p * ndr * ndr + y * ndr + x;
                uint32_t* dst = a.depth + (size_t)(ndr * o.y + (int)y) * a.g.depth_w + (size_t)(ndr * o.x + (int)x);
                if (dq == 4) *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(src);
                else *dst = *src;
            }
        }

        const uint32_t rxy = (uint32_t)(a.g.res[0] * a.g.res[1]);
        const uint32_t nprobes_grid = rxy * (uint32_t)a.g.res[2];
        const uint32_t probe_t = (uint32_t)tid < np ? (a.probe_list ? a.probe_list[p0 + tid] : p0 + tid) : nprobes_grid;
        if (probe_t < nprobes_grid) {  // probesUpdate.glsl:110-119
            uint32_t s = a.states[probe_t];
            if (s_oor[tid] >= R) {
                s = 8;
            } else {
                const float mc = __uint_as_float(s_maxc[tid]);
                const float sf = (float)s;
                if (mc < 0.02f / sf) s = min(s + 1u, 8u);
                else if (mc > 0.04f / sf) s = max(s - 1u, 1u);
                else if (mc > 0.25f) s = 1;
            }
            a.states[probe_t] = s;
        }
    }

    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, cols);
    }
}

__global__ void __launch_bounds__(kThreads) k_blend_tc(TcArgs a) {
    const uint32_t n = a.dev_count ? *a.dev_count : a.nprobes;
    const uint32_t p0 = blockIdx.x * a.tile;
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
                                                             const float4* __restrict__ rays, uint32_t smem_bytes) {
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
        a.tile = kTileProbes;
        a.smem_bytes = smem_bytes;
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

// Probes per CTA for a launch over n probes with `per_sm` CTAs resident per
// SM: the grid runs in rounds of (SMs x per_sm) CTAs, and a CTA's time is
// a fixed part (the chunk pipeline, the accumulator read-back) plus a part
// per probe, measured on GB300 as about 70 probes' worth of fixed cost
// (tiles of 25 / 20 / 18 / 16 probes over 16,384 probes: 0.115 / 0.109 /
// 0.107 / 0.133 ms); the size with the fewest rounds x (70 + size) wins,
// the larger on ties.
uint32_t tc_tile_size(uint32_t n, uint32_t per_sm) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || sms <= 0) {
        cudaGetLastError();
        return kTileProbes;
    }
    const uint64_t slots = (uint64_t)sms * per_sm;
    uint32_t best = kTileProbes;
    uint64_t best_cost = ~0ull;
    for (uint32_t t = kTileProbes; t >= 16; --t) {
        const uint64_t tiles = (n + t - 1) / t, rounds = (tiles + slots - 1) / slots;
        const uint64_t cost = rounds * (70 + t);
        if (cost < best_cost) {
            best_cost = cost;
            best = t;
        }
    }
    return best;
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
    return (size_t)nchunks * tc_b_bytes(Nd, Nc);
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
    const size_t smem = tc_smem_bytes(nc, nd, Nc, Nd);
    cudaError_t e = set_tc_smem_limit();
    if (e != cudaSuccess) return e;
    a.tile = tc_tile_size(nprobes, Nd + Nc > 256 ? 1u : 2u);
    a.smem_bytes = (uint32_t)smem;
    uint32_t blocks = (nprobes + a.tile - 1) / a.tile;
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
    return tc_smem_bytes(nc, nd, Nc, Nd);
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
    k_batch_blend_tc<<<bl.ntiles, kThreads, smem, st>>>(bt, bl, rays, (uint32_t)smem);
    return cudaGetLastError();
}

}  // namespace ddgi

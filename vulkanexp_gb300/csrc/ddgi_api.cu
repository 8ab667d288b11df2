// ddgi_api.cu — the C ABI (include/ddgi.h): context, scene build, update.
//
// Mirrors the host orchestration of IrradianceProbes
// (src/IrradianceProbes.cpp:12-594): init allocates the atlases and per-ray
// buffers, update records trace -> blend (+border) on the caller's stream.
// Differences by design: the atlas is updated in place (the reference's
// work -> final image copy, :532-577, is not needed because nothing samples
// the atlas while a blend runs), the direction table is computed on the host
// once per update, and every call returns a status instead of throwing.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/ddgi.h"
#include "../../include/ddgi_exact.h"
#include "common.cuh"
#include "ctx.h"
#include "kernels.h"
#include "lbvh.h"
#include "nvtx.h"
#include "gbuild.h"
#include "sah.h"
#include "wide.h"

using namespace ddgi;

namespace {

ddgi_status fail(ddgi_ctx* c, ddgi_status s, const char* fmt, ...) {
    if (c) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(c->msg, sizeof(c->msg), fmt, ap);
        va_end(ap);
    }
    return s;
}

ddgi_status cuda_fail(ddgi_ctx* c, cudaError_t e, const char* what) {
    cudaGetLastError();  // clear a sticky-free error
    if (e == cudaErrorMemoryAllocation) return fail(c, DDGI_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(c, DDGI_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                                  \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

template <class T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}
void dfree_v(void*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

bool grid_valid(const ddgi_grid_desc* g, char* why, size_t n) {
    for (int k = 0; k < 3; ++k) {
        if (g->resolution[k] < 2) return snprintf(why, n, "resolution[%d] = %d < 2", k, g->resolution[k]), false;
        if (!std::isfinite(g->extent_min[k]) || !std::isfinite(g->extent_max[k]) || !(g->extent_max[k] > g->extent_min[k]))
            return snprintf(why, n, "extent axis %d is empty or not finite", k), false;
    }
    if (g->rays_per_probe < 1 || g->rays_per_probe > DDGI_MAX_RAYS_PER_PROBE)
        return snprintf(why, n, "rays_per_probe = %u outside [1, %u]", g->rays_per_probe, DDGI_MAX_RAYS_PER_PROBE), false;
    if (g->color_res < 3 || g->color_res > 64) return snprintf(why, n, "color_res = %u outside [3, 64]", g->color_res), false;
    if (g->depth_res < 3 || g->depth_res > 64) return snprintf(why, n, "depth_res = %u outside [3, 64]", g->depth_res), false;
    if (!std::isfinite(g->hysteresis) || !std::isfinite(g->depth_sharpness) || !std::isfinite(g->shadow_bias))
        return snprintf(why, n, "non-finite hysteresis/sharpness/bias"), false;
    if (g->precision != DDGI_PRECISION_FP32 && g->precision != DDGI_PRECISION_BF16 &&
        g->precision != DDGI_PRECISION_REFERENCE_FORMAT)
        return snprintf(why, n, "unknown precision %u", g->precision), false;
    uint64_t probes = (uint64_t)g->resolution[0] * g->resolution[1] * g->resolution[2];
    if (probes > (1u << 24)) return snprintf(why, n, "too many probes (%llu)", (unsigned long long)probes), false;
    if (probes * g->rays_per_probe > DDGI_MAX_RAYS_PER_UPDATE)
        return snprintf(why, n, "probes x rays_per_probe = %llu above %u", (unsigned long long)(probes * g->rays_per_probe),
                        DDGI_MAX_RAYS_PER_UPDATE),
               false;
    uint64_t w = (uint64_t)g->depth_res * g->resolution[0] * g->resolution[1];
    if (w > (1u << 30)) return snprintf(why, n, "atlas too wide"), false;
    // texel indices of the atlas lookups are 32-bit
    for (const uint32_t side : {g->color_res, g->depth_res}) {
        const uint64_t texels = (uint64_t)side * side * probes;
        if (texels > 0xFFFFFFFFull)
            return snprintf(why, n, "atlas of %llu texels (tile side %u) above 2^32 - 1", (unsigned long long)texels, side),
                   false;
    }
    return true;
}

DeviceGrid make_device_grid(const ddgi_grid_desc& g) {
    DeviceGrid d{};
    for (int k = 0; k < 3; ++k) {
        d.mn[k] = g.extent_min[k];
        d.mx[k] = g.extent_max[k];
        d.res[k] = g.resolution[k];
        volatile float diff = g.extent_max[k] - g.extent_min[k];
        d.cell[k] = diff / (float)(g.resolution[k] - 1);
    }
    {
        volatile float a = d.cell[0] * d.cell[0];
        volatile float b = d.cell[1] * d.cell[1];
        volatile float c = d.cell[2] * d.cell[2];
        volatile float s = a + b;
        s = s + c;
        d.cell_len = std::sqrt((float)s);
    }
    {
        volatile float dx = g.extent_max[0] - g.extent_min[0];
        volatile float dy = g.extent_max[1] - g.extent_min[1];
        volatile float dz = g.extent_max[2] - g.extent_min[2];
        volatile float a = dx * dx, b = dy * dy, c = dz * dz;
        volatile float s = a + b;
        s = s + c;
        d.tmax = std::sqrt((float)s);
    }
    d.rays = g.rays_per_probe;
    d.color_res = g.color_res;
    d.depth_res = g.depth_res;
    d.sharp = g.depth_sharpness;
    d.hyst = g.hysteresis;
    d.bias = g.shadow_bias;
    d.color_w = g.color_res * g.resolution[0] * g.resolution[1];
    d.color_h = g.color_res * g.resolution[2];
    d.depth_w = g.depth_res * g.resolution[0] * g.resolution[1];
    d.depth_h = g.depth_res * g.resolution[2];
    d.quant = g.precision == DDGI_PRECISION_REFERENCE_FORMAT ? 1u : 0u;
    return d;
}

uint32_t probe_count_of(const ddgi_grid_desc& g) {
    return (uint32_t)g.resolution[0] * (uint32_t)g.resolution[1] * (uint32_t)g.resolution[2];
}

size_t atlas_bytes(const DeviceGrid& d, ddgi_atlas_kind k, bool fp16) {
    size_t texels = k == DDGI_ATLAS_COLOR ? (size_t)d.color_w * d.color_h : (size_t)d.depth_w * d.depth_h;
    size_t per = k == DDGI_ATLAS_COLOR ? (fp16 ? 8 : 16) : (fp16 ? 4 : 8);
    return texels * per;
}

void free_scene(SceneBuffers& s) {
    dfree(s.wnodes);
    dfree(s.winst_leaf);
    dfree(s.leaf_lo);
    dfree(s.leaf_hi);
    dfree(s.leaf_parent);
    dfree(s.node_parent);
    dfree(s.refit_flags);
    dfree(s.sub_lo);
    dfree(s.sub_hi);
    dfree(s.nodes);
    dfree(s.tris);
    dfree(s.inst_leaf);
    dfree(s.inst_id);
    dfree(s.normals);
    dfree(s.indices);
    dfree(s.offsets);
    dfree(s.materials);
    s = SceneBuffers{};
}

ddgi_status ensure_ray_capacity(ddgi_ctx* ctx, size_t records) {
    if (records > ctx->rays_cap) {
        dfree(ctx->rays);
        dfree(ctx->wave_thit);
        dfree(ctx->wave_prim);
        dfree(ctx->wave_front);
        dfree(ctx->q_idx);
        dfree(ctx->q_pos);
        dfree(ctx->q_sun);
        ctx->rays_cap = 0;
        CK(cudaMalloc(&ctx->rays, records * sizeof(float4)), "cudaMalloc ray records");
        CK(cudaMalloc(&ctx->wave_thit, records * sizeof(float4)), "cudaMalloc hit buffer");
        CK(cudaMalloc(&ctx->wave_prim, records * sizeof(uint32_t)), "cudaMalloc hit buffer");
        CK(cudaMalloc(&ctx->wave_front, records * sizeof(uint32_t)), "cudaMalloc front-hit queue");
        CK(cudaMalloc(&ctx->q_idx, records * sizeof(uint32_t)), "cudaMalloc shadow queue");
        CK(cudaMalloc(&ctx->q_pos, records * sizeof(float4)), "cudaMalloc shadow queue");
        CK(cudaMalloc(&ctx->q_sun, records * sizeof(float4)), "cudaMalloc shadow queue");
        ctx->rays_cap = records;
    }
    if (ctx->record_hits && records > ctx->hits_cap) {
        dfree(ctx->hits);
        CK(cudaMalloc(&ctx->hits, records * sizeof(ddgi_hit)), "cudaMalloc hit records");
        ctx->hits_cap = records;
    }
    return DDGI_OK;
}

ddgi_status check_device_error(ddgi_ctx* ctx) {
    uint32_t e = 0;
    CK(cudaMemcpy(&e, ctx->err, sizeof(e), cudaMemcpyDeviceToHost), "read device error word");
    if (e != 0) {
        cudaMemset(ctx->err, 0, sizeof(uint32_t));
        const char* what = e == DEV_STACK_OVERFLOW ? "traversal stack overflow"
                           : e == DEV_BAD_INDEX    ? "index out of range in scene data"
                           : e == DEV_WAIT_TIMEOUT ? "device wait timed out"
                                                   : "unknown device error";
        return fail(ctx, DDGI_ERR_DEVICE, "device error %u: %s", e, what);
    }
    return DDGI_OK;
}

}  // namespace

extern "C" {

const char* ddgi_status_string(ddgi_status s) {
    switch (s) {
        case DDGI_OK: return "DDGI_OK";
        case DDGI_ERR_INVALID_ARGUMENT: return "DDGI_ERR_INVALID_ARGUMENT";
        case DDGI_ERR_CUDA: return "DDGI_ERR_CUDA";
        case DDGI_ERR_OUT_OF_MEMORY: return "DDGI_ERR_OUT_OF_MEMORY";
        case DDGI_ERR_NO_SCENE: return "DDGI_ERR_NO_SCENE";
        case DDGI_ERR_TIMEOUT: return "DDGI_ERR_TIMEOUT";
        case DDGI_ERR_DEVICE: return "DDGI_ERR_DEVICE";
        case DDGI_ERR_UNSUPPORTED: return "DDGI_ERR_UNSUPPORTED";
        case DDGI_ERR_IO: return "DDGI_ERR_IO";
    }
    return "DDGI_ERR_UNKNOWN";
}

const char* ddgi_last_error(const ddgi_ctx* ctx) { return ctx ? ctx->msg : "null context"; }

ddgi_status ddgi_create(const ddgi_grid_desc* grid, ddgi_ctx** out) {
    if (!out) return DDGI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!grid) return DDGI_ERR_INVALID_ARGUMENT;
    char why[256];
    if (!grid_valid(grid, why, sizeof(why))) return DDGI_ERR_INVALID_ARGUMENT;
    ddgi_ctx* ctx = new (std::nothrow) ddgi_ctx();
    if (!ctx) return DDGI_ERR_OUT_OF_MEMORY;
    ctx->grid = *grid;
    ctx->dg = make_device_grid(*grid);
    ctx->fp16 = grid->precision == DDGI_PRECISION_BF16;
    // default light: LightBuffer defaults (src/Light.hpp:6-9), black sky
    {
        float d[3] = {0.2f, 2.0f, 0.2f};
        float l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int k = 0; k < 3; ++k) {
            ctx->dl.dir[k] = d[k] / l;
            ctx->dl.color[k] = 10.0f;
            ctx->dl.sky[k] = 0.0f;
        }
        ctx->dl.sun_brightness = 10.0f;
        ctx->dl.sky_mode = DDGI_SKY_CONSTANT;
    }
    cudaError_t e = cudaGetDevice(&ctx->device);
    ddgi_status st = DDGI_OK;
    const uint32_t P = probe_count_of(*grid);
    auto bail = [&](ddgi_status s) {
        ddgi_destroy(ctx);
        return s;
    };
    if (e != cudaSuccess) return bail(DDGI_ERR_CUDA);
    if (cudaMalloc(&ctx->color, atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, ctx->fp16)) != cudaSuccess ||
        cudaMalloc(&ctx->depth, atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, ctx->fp16)) != cudaSuccess ||
        cudaMalloc(&ctx->states, sizeof(uint32_t) * P) != cudaSuccess ||
        cudaMalloc(&ctx->dirs, sizeof(float4) * DDGI_MAX_RAYS_PER_PROBE) != cudaSuccess ||
        cudaMalloc(&ctx->ray_order, sizeof(uint32_t) * DDGI_MAX_RAYS_PER_PROBE) != cudaSuccess ||
        cudaMalloc(&ctx->probe_list, sizeof(uint32_t) * P) != cudaSuccess ||
        cudaMalloc(&ctx->sched, 8 * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&ctx->probe_perm, sizeof(uint32_t) * P) != cudaSuccess ||
        cudaMalloc(&ctx->err, sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&ctx->counters, 4 * sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        return bail(DDGI_ERR_OUT_OF_MEMORY);
    }
    if (ctx->fp16) {
        if (!tc_blend_supported(grid->color_res, grid->depth_res)) return bail(DDGI_ERR_UNSUPPORTED);
        if (cudaMalloc(&ctx->tc_weights, tc_weight_bytes(DDGI_MAX_RAYS_PER_PROBE, grid->color_res, grid->depth_res)) !=
                cudaSuccess ||
            cudaMalloc(&ctx->tc_rowsum, 512 * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&ctx->acc_color, atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, false)) != cudaSuccess ||
            cudaMalloc(&ctx->acc_depth, atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, false)) != cudaSuccess) {
            cudaGetLastError();
            return bail(DDGI_ERR_OUT_OF_MEMORY);
        }
        cudaMemset(ctx->acc_color, 0, atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, false));
        cudaMemset(ctx->acc_depth, 0, atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, false));
    } else {
        // the FP32 wavefront blend's per-update weights (ray x texel) and sums
        const size_t ntex = (size_t)(grid->color_res - 2) * (grid->color_res - 2) +
                            (size_t)(grid->depth_res - 2) * (grid->depth_res - 2);
        if (cudaMalloc(&ctx->tc_weights, fp32_weight_bytes(DDGI_MAX_RAYS_PER_PROBE, grid->color_res,
                                                           grid->depth_res)) != cudaSuccess ||
            cudaMalloc(&ctx->tc_rowsum, ntex * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            return bail(DDGI_ERR_OUT_OF_MEMORY);
        }
    }
    st = ensure_ray_capacity(ctx, (size_t)P * grid->rays_per_probe);
    if (st != DDGI_OK) return bail(st);
    cudaMemset(ctx->color, 0, atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, ctx->fp16));
    cudaMemset(ctx->depth, 0, atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, ctx->fp16));
    cudaMemset(ctx->err, 0, sizeof(uint32_t));
    cudaMemset(ctx->sched, 0, 8 * sizeof(uint32_t));
    {
        std::vector<uint32_t> perm = probe_morton_order(grid->resolution);
        cudaMemcpy(ctx->probe_perm, perm.data(), sizeof(uint32_t) * P, cudaMemcpyHostToDevice);
    }
    std::vector<uint32_t> ones(P, 1u);
    cudaMemcpy(ctx->states, ones.data(), sizeof(uint32_t) * P, cudaMemcpyHostToDevice);
    for (int i = 0; i < 4; ++i)
        if (cudaEventCreate(&ctx->ev[i]) != cudaSuccess) return bail(DDGI_ERR_CUDA);
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(DDGI_ERR_CUDA);
    *out = ctx;
    return DDGI_OK;
}

ddgi_status ddgi_destroy(ddgi_ctx* ctx) {
    if (!ctx) return DDGI_OK;
    cudaDeviceSynchronize();
    free_scene(ctx->scene);
    dfree_v(ctx->color);
    dfree_v(ctx->depth);
    dfree(ctx->states);
    dfree(ctx->rays);
    dfree(ctx->wave_thit);
    dfree(ctx->wave_prim);
    dfree(ctx->wave_front);
    dfree(ctx->xfer);
    dfree(ctx->q_idx);
    dfree(ctx->q_pos);
    dfree(ctx->q_sun);
    dfree(ctx->counters);
    dfree(ctx->tc_weights);
    dfree(ctx->tc_rowsum);
    dfree(ctx->acc_color);
    dfree(ctx->acc_depth);
    dfree(ctx->rec_thit);
    dfree(ctx->rec_prim);
    dfree(ctx->ckpt_color);
    dfree(ctx->ckpt_depth);
    dfree(ctx->rec_states);
    dfree(ctx->work_states);
    dfree(ctx->work_color);
    dfree(ctx->work_depth);
    dfree(ctx->g_a);
    dfree(ctx->g_b);
    dfree(ctx->g_x);
    dfree(ctx->d_grad);
    dfree(ctx->hits);
    dfree(ctx->dirs);
    dfree(ctx->ray_order);
    dfree(ctx->probe_list);
    dfree(ctx->sched);
    dfree(ctx->probe_perm);
    dfree(ctx->init_dirs);
    dfree(ctx->init_back);
    dfree(ctx->init_near);
    dfree(ctx->err);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    delete ctx;
    return DDGI_OK;
}

uint32_t ddgi_probe_count(const ddgi_ctx* ctx) { return ctx ? probe_count_of(ctx->grid) : 0u; }

ddgi_status ddgi_get_grid(const ddgi_ctx* ctx, ddgi_grid_desc* out) {
    if (!ctx || !out) return DDGI_ERR_INVALID_ARGUMENT;
    *out = ctx->grid;
    return DDGI_OK;
}

ddgi_status ddgi_set_grid(ddgi_ctx* ctx, const ddgi_grid_desc* g) {
    if (!ctx || !g) return DDGI_ERR_INVALID_ARGUMENT;
    char why[256];
    if (!grid_valid(g, why, sizeof(why))) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "%s", why);
    for (int k = 0; k < 3; ++k)
        if (g->resolution[k] != ctx->grid.resolution[k])
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "resolution cannot change (recreate the context)");
    if (g->color_res != ctx->grid.color_res || g->depth_res != ctx->grid.depth_res)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "color_res/depth_res cannot change (recreate the context)");
    if (g->precision != ctx->grid.precision)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "precision cannot change (recreate the context)");
    ddgi_status st = ensure_ray_capacity(ctx, (size_t)probe_count_of(*g) * g->rays_per_probe);
    if (st != DDGI_OK) return st;
    ctx->grid = *g;
    ctx->dg = make_device_grid(*g);
    if (ctx->ramp_on) {  // updateUniforms() uploads GridParameters.hysteresis as given
        ctx->ramp_cmd.set |= kRampSetBlended | kRampSetParam;
        ctx->ramp_cmd.blended = ctx->ramp_cmd.param = g->hysteresis;
    }
    return DDGI_OK;
}

ddgi_status ddgi_set_target_hysteresis(ddgi_ctx* ctx, float target) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    if (!std::isfinite(target) || target > 1.0f)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "target hysteresis must be finite and at most 1");
    if (target < 0.0f) {  // off: the grid's hysteresis is blended as given
        ctx->ramp_on = false;
        ctx->ramp_cmd = RampCmd{};
        return DDGI_OK;
    }
    if (!ctx->ramp_on) {  // the ramp starts from the grid's hysteresis with no probes counted
        ctx->ramp_on = true;
        ctx->ramp_cmd.set = kRampSetBlended | kRampSetParam | kRampZeroCount;
        ctx->ramp_cmd.blended = ctx->ramp_cmd.param = ctx->grid.hysteresis;
    }
    ctx->ramp_cmd.set |= kRampSetTarget;
    ctx->ramp_cmd.target = target;
    return DDGI_OK;
}

ddgi_status ddgi_get_hysteresis(ddgi_ctx* ctx, float* blended, float* parameter, uint32_t* counted,
                                ddgi_stream stream) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    float b = ctx->grid.hysteresis, p = ctx->grid.hysteresis;
    uint32_t c = 0;
    if (ctx->ramp_on) {
        uint32_t h[4];
        cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
        CK(cudaMemcpyAsync(h, ctx->sched + 4, sizeof(h), cudaMemcpyDeviceToHost, st), "read ramp");
        CK(cudaStreamSynchronize(st), "read ramp");
        std::memcpy(&b, &h[0], 4);
        std::memcpy(&p, &h[1], 4);
        c = h[3];
        const RampCmd& m = ctx->ramp_cmd;  // host changes not applied yet
        if (m.set & kRampSetBlended) b = m.blended;
        if (m.set & kRampSetParam) p = m.param;
        if (m.set & kRampZeroCount) c = 0;
    }
    if (blended) *blended = b;
    if (parameter) *parameter = p;
    if (counted) *counted = c;
    return DDGI_OK;
}

ddgi_status ddgi_set_light(ddgi_ctx* ctx, const ddgi_light* l) {
    if (!ctx || !l) return DDGI_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < 3; ++k) {
        if (!std::isfinite(l->direction[k]) || !std::isfinite(l->color[k]) || !std::isfinite(l->sky[k]))
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "non-finite light");
        ctx->dl.dir[k] = l->direction[k];
        ctx->dl.color[k] = l->color[k];
        ctx->dl.sky[k] = l->sky[k];
    }
    if (!std::isfinite(l->color[3])) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "non-finite light");
    ctx->dl.sun_brightness = l->color[3];
    return DDGI_OK;
}

ddgi_status ddgi_set_sky_mode(ddgi_ctx* ctx, ddgi_sky_mode mode) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    if (mode != DDGI_SKY_CONSTANT && mode != DDGI_SKY_ATMOSPHERE)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "unknown sky mode %d", (int)mode);
    ctx->dl.sky_mode = (uint32_t)mode;
    return DDGI_OK;
}

ddgi_status ddgi_record_hits(ddgi_ctx* ctx, int enable) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    ctx->record_hits = enable != 0;
    if (ctx->record_hits) return ensure_ray_capacity(ctx, ctx->rays_cap);
    return DDGI_OK;
}

ddgi_status ddgi_set_pipeline(ddgi_ctx* ctx, ddgi_pipeline pipeline) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    if (pipeline != DDGI_PIPELINE_FUSED && pipeline != DDGI_PIPELINE_WAVEFRONT)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "unknown pipeline %d", (int)pipeline);
    ctx->pipeline = pipeline;
    return DDGI_OK;
}

ddgi_status ddgi_enable_timing(ddgi_ctx* ctx, int enable) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    ctx->timing = enable != 0;
    return DDGI_OK;
}

// ---------------------------------------------------------------------------
// Scene build (replaces the BLAS/TLAS build of src/Renderer.cpp:272-642)
// ---------------------------------------------------------------------------
namespace {

unsigned host_threads() {
    const unsigned n = std::thread::hardware_concurrency();
    return n ? std::min(n, 64u) : 1u;
}

uint64_t next_build_id() {
    static std::atomic<uint64_t> builds{0};
    return ++builds;
}

// World box of an instance: the 8 corners of its mesh's object-space bounds
// through the object-to-world transform (in double), rounded to float and
// enlarged like the tree builder's boxes; empty for an empty mesh.
void instance_world_box(const float* transform, const float* ml, const float* mh, bool valid, float4* olo,
                        float4* ohi) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (valid && ml[0] <= mh[0]) {
        for (int c = 0; c < 8; ++c) {
            double p[3] = {(c & 1) ? mh[0] : ml[0], (c & 2) ? mh[1] : ml[1], (c & 4) ? mh[2] : ml[2]};
            for (int k = 0; k < 3; ++k) {
                float q = (float)(transform[4 * k] * p[0] + transform[4 * k + 1] * p[1] + transform[4 * k + 2] * p[2] +
                                  transform[4 * k + 3]);
                lo[k] = std::min(lo[k], q);
                hi[k] = std::max(hi[k], q);
            }
        }
        for (int k = 0; k < 3; ++k) {
            float e = (hi[k] - lo[k]) * 1e-5f + (std::fabs(lo[k]) + std::fabs(hi[k])) * 1e-6f + 1e-7f;
            lo[k] -= e;
            hi[k] += e;
        }
    }
    *olo = make_float4(lo[0], lo[1], lo[2], 0.0f);
    *ohi = make_float4(hi[0], hi[1], hi[2], 0.0f);
}

// Top level over S.inst_lo/inst_hi (caller order) at nodes[node_base ...]:
// the LBVH, the instance records in leaf order, the leaf boxes and the
// parent links that a later refit needs.  Scratch for ni primitives; the
// top-level depth goes to depth_dev[0] (which must hold 1 on entry).
ddgi_status build_top_level(ddgi_ctx* ctx, uint64_t node_base, void* scratch, float4* box_lo, float4* box_hi,
                            uint32_t* sorted, uint32_t* depth_dev, cudaStream_t st) {
    SceneBuffers& S = ctx->scene;
    const uint32_t ni = (uint32_t)S.host_inst.size();
    if (ni == 0) {
        S.tlas_root = -1;
        return DDGI_OK;
    }
    const uint32_t inner = ni > 1 ? ni - 1 : 1;
    if (!S.leaf_lo) {
        CK(cudaMalloc(&S.leaf_lo, sizeof(float4) * ni), "alloc top level");
        CK(cudaMalloc(&S.leaf_hi, sizeof(float4) * ni), "alloc top level");
        CK(cudaMalloc(&S.leaf_parent, sizeof(uint32_t) * ni), "alloc top level");
        CK(cudaMalloc(&S.node_parent, sizeof(uint32_t) * inner), "alloc top level");
        CK(cudaMalloc(&S.refit_flags, sizeof(uint32_t) * inner), "alloc top level");
        CK(cudaMalloc(&S.sub_lo, sizeof(float4) * 2 * inner), "alloc top level");
        CK(cudaMalloc(&S.sub_hi, sizeof(float4) * 2 * inner), "alloc top level");
    }
    std::vector<uint32_t> order(ni);
    std::vector<BvhNode> top(inner);
    if (S.build_mode == DDGI_BUILD_FAST_TRACE) {
        CK(cudaMemcpyAsync(box_lo, S.inst_lo.data(), sizeof(float4) * ni, cudaMemcpyHostToDevice, st), "upload boxes");
        CK(cudaMemcpyAsync(box_hi, S.inst_hi.data(), sizeof(float4) * ni, cudaMemcpyHostToDevice, st), "upload boxes");
        GpuTreeBuilder gtb;
        CK(gtb.build_boxes(box_lo, box_hi, ni, kTlasLeafMax, ctx->err, st), "top-level build");
        CK(gtb.write(S.nodes, std::vector<int>{(int)node_base}, std::vector<int>{0}, sorted, std::vector<uint32_t>{0},
                     st),
           "top-level build");
        const uint32_t d = gtb.depths()[0];
        CK(cudaMemcpyAsync(depth_dev, &d, sizeof(d), cudaMemcpyHostToDevice, st), "upload depth");
        CK(cudaMemcpyAsync(order.data(), sorted, sizeof(uint32_t) * ni, cudaMemcpyDeviceToHost, st), "read order");
        CK(cudaMemcpyAsync(top.data(), S.nodes + node_base, sizeof(BvhNode) * inner, cudaMemcpyDeviceToHost, st),
           "read top level");
        CK(cudaStreamSynchronize(st), "top-level build");
    } else if (S.build_mode == DDGI_BUILD_FAST_TRACE_HOST) {
        uint32_t d = 1;
        sah_build(S.inst_lo.data(), S.inst_hi.data(), ni, kTlasLeafMax, (int)node_base, 0, top.data(), order.data(), &d,
                  host_threads());
        CK(cudaMemcpyAsync(S.nodes + node_base, top.data(), sizeof(BvhNode) * inner, cudaMemcpyHostToDevice, st),
           "upload top level");
        CK(cudaMemcpyAsync(depth_dev, &d, sizeof(d), cudaMemcpyHostToDevice, st), "upload depth");
        CK(cudaStreamSynchronize(st), "top-level build");
    } else {
        CK(cudaMemcpyAsync(box_lo, S.inst_lo.data(), sizeof(float4) * ni, cudaMemcpyHostToDevice, st), "upload boxes");
        CK(cudaMemcpyAsync(box_hi, S.inst_hi.data(), sizeof(float4) * ni, cudaMemcpyHostToDevice, st), "upload boxes");
        CK(lbvh_build(box_lo, box_hi, ni, kTlasLeafMax, S.nodes, (int)node_base, 0, sorted, scratch, ctx->err,
                      depth_dev, st),
           "top-level build");
        CK(cudaMemcpyAsync(order.data(), sorted, sizeof(uint32_t) * ni, cudaMemcpyDeviceToHost, st), "read order");
        CK(cudaMemcpyAsync(top.data(), S.nodes + node_base, sizeof(BvhNode) * inner, cudaMemcpyDeviceToHost, st),
           "read top level");
        CK(cudaStreamSynchronize(st), "top-level build");
    }
    std::vector<GpuInstance> leaf(ni);
    std::vector<float4> llo(ni), lhi(ni);
    S.leaf_of_id.assign(ni, 0);
    for (uint32_t s = 0; s < ni; ++s) {
        const uint32_t id = order[s] < ni ? order[s] : 0;
        leaf[s] = S.host_inst[id];
        llo[s] = S.inst_lo[id];
        lhi[s] = S.inst_hi[id];
        S.leaf_of_id[id] = s;
    }
    // parent links from the node references (a one-instance tree references
    // its leaf from both sides; the second side is the empty box)
    std::vector<uint32_t> lp(ni, 0xFFFFFFFFu), np(inner, 0xFFFFFFFFu);
    for (uint32_t k = 0; k < inner; ++k) {
        const int refs[2] = {top[k].d.x, top[k].d.y};
        for (uint32_t side = 0; side < 2; ++side) {
            const int r = refs[side];
            if (r >= 0) {
                const uint64_t c = (uint64_t)r - node_base;
                if (r < (int)node_base || c >= inner) return fail(ctx, DDGI_ERR_DEVICE, "top level: bad child link");
                np[c] = k << 1 | side;
            } else {
                const uint32_t slot = (uint32_t)((~r) >> 3);
                if (slot >= ni) return fail(ctx, DDGI_ERR_DEVICE, "top level: bad leaf link");
                if (lp[slot] == 0xFFFFFFFFu) lp[slot] = k << 1 | side;
            }
        }
    }
    CK(cudaMemcpyAsync(S.inst_leaf, leaf.data(), sizeof(GpuInstance) * ni, cudaMemcpyHostToDevice, st), "upload");
    CK(cudaMemcpyAsync(S.inst_id, S.host_inst.data(), sizeof(GpuInstance) * ni, cudaMemcpyHostToDevice, st), "upload");
    CK(cudaMemcpyAsync(S.leaf_lo, llo.data(), sizeof(float4) * ni, cudaMemcpyHostToDevice, st), "upload");
    CK(cudaMemcpyAsync(S.leaf_hi, lhi.data(), sizeof(float4) * ni, cudaMemcpyHostToDevice, st), "upload");
    CK(cudaMemcpyAsync(S.leaf_parent, lp.data(), sizeof(uint32_t) * ni, cudaMemcpyHostToDevice, st), "upload");
    CK(cudaMemcpyAsync(S.node_parent, np.data(), sizeof(uint32_t) * inner, cudaMemcpyHostToDevice, st), "upload");
    S.tlas_root = (int32_t)node_base;
    return DDGI_OK;
}

// Instances in leaf order with the mesh roots of the wide trees.
ddgi_status upload_wide_instances(ddgi_ctx* ctx, cudaStream_t st) {
    SceneBuffers& S = ctx->scene;
    const uint32_t ni = (uint32_t)S.host_inst.size();
    if (ni == 0) return DDGI_OK;
    std::vector<GpuInstance> leaf(ni);
    for (uint32_t id = 0; id < ni; ++id) {
        GpuInstance g = S.host_inst[id];
        g.blas_root = g.blas_root >= 0 ? S.wide_root_of_mesh[S.mesh_of_inst[id]] : -1;
        leaf[S.leaf_of_id[id]] = g;
    }
    CK(cudaMemcpyAsync(S.winst_leaf, leaf.data(), sizeof(GpuInstance) * ni, cudaMemcpyHostToDevice, st), "upload");
    return DDGI_OK;
}

// Top level of the wide trees again (after a refit or rebuild of the
// binary top level): collapsed from the binary top-level nodes, placed at
// wide_tlas_start.
ddgi_status refresh_wide_top(ddgi_ctx* ctx, cudaStream_t st) {
    SceneBuffers& S = ctx->scene;
    if (!S.wnodes) return DDGI_OK;
    const uint32_t ni = (uint32_t)S.host_inst.size();
    const uint32_t inner = ni > 1 ? ni - 1 : 1;
    std::vector<BvhNode> top(inner);
    CK(cudaMemcpyAsync(top.data(), S.nodes + S.tlas_root, sizeof(BvhNode) * inner, cudaMemcpyDeviceToHost, st),
       "read top level");
    CK(cudaStreamSynchronize(st), "read top level");
    for (auto& n : top) {  // references relative to the top level's first node
        if (n.d.x >= 0) n.d.x -= S.tlas_root;
        if (n.d.y >= 0) n.d.y -= S.tlas_root;
    }
    std::vector<WideNode> w;
    uint32_t lt = 0;
    bool ok = true;
    collapse_wide(top, 0, w, &lt, &ok);
    if (!ok || S.wide_tlas_start + w.size() > S.wide_cap) return fail(ctx, DDGI_ERR_DEVICE, "wide top level");
    for (auto& n : w) {
        for (int h = 0; h < 2; ++h) {
            int* r = &n.ref[h].x;
            for (int k = 0; k < 4; ++k)
                if (r[k] >= 0) r[k] += (int)S.wide_tlas_start;
        }
    }
    CK(cudaMemcpyAsync(S.wnodes + S.wide_tlas_start, w.data(), sizeof(WideNode) * w.size(), cudaMemcpyHostToDevice, st),
       "upload wide top level");
    S.wtlas_root = (int32_t)S.wide_tlas_start;
    S.wnode_count = S.wide_tlas_start + (uint32_t)w.size();
    // one node group per level, an exit marker between the levels; node
    // groups pack the node index into 23 bits
    const int cap = (int)(S.wlevels_blas + lt + 4);
    S.wstack_cap = cap <= kMaxStack && S.wnode_count < kMaxWideNodes ? cap : 0;
    return upload_wide_instances(ctx, st);
}

// Mesh tree in nodes[b, e) (root at b) laid out depth first: every node is
// followed by its first child's subtree, then its second child's, so that a
// walk down the tree mostly moves to the adjacent node (the same 128-byte
// cache line).  The root keeps index b, leaf references are unchanged, and
// the nodes a collapsed leaf made unreachable keep their slots after the
// reachable ones.  Returns false (nodes untouched) on a malformed tree.
bool depth_first_layout(std::vector<BvhNode>& nodes, uint32_t b, uint32_t e) {
    const uint32_t n = e - b;
    std::vector<int32_t> newidx(n, -1);
    std::vector<uint32_t> order;
    order.reserve(n);
    std::vector<uint32_t> stack{b};
    while (!stack.empty()) {
        const uint32_t k = stack.back();
        stack.pop_back();
        if (k < b || k >= e || newidx[k - b] >= 0) return false;
        newidx[k - b] = (int32_t)(b + order.size());
        order.push_back(k);
        const int4 d = nodes[k].d;
        if (d.y >= 0) stack.push_back((uint32_t)d.y);  // second child after the first one's subtree
        if (d.x >= 0 && d.x != d.y) stack.push_back((uint32_t)d.x);
    }
    std::vector<BvhNode> out(nodes.begin() + b, nodes.begin() + e);
    uint32_t pos = (uint32_t)order.size();
    for (uint32_t k = 0; k < n; ++k)
        if (newidx[k] < 0) out[pos++] = nodes[b + k];  // unreachable: kept, never referenced
    for (size_t i = 0; i < order.size(); ++i) {
        BvhNode nd = nodes[order[i]];
        if (nd.d.x >= 0) nd.d.x = newidx[nd.d.x - (int)b];
        if (nd.d.y >= 0) nd.d.y = newidx[nd.d.y - (int)b];
        out[i] = nd;
    }
    std::copy(out.begin(), out.end(), nodes.begin() + b);
    return true;
}

// A mesh tree built on the host, its references relative to its own first
// node and first triangle reference.
struct HostTree {
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> order;  // triangle of each leaf position
    uint32_t depth = 1;
};

// Fast-trace trees of every mesh (sbvh.cu): meshes of 64K or more triangles
// one after the other with every host thread, the others in parallel, the
// host threads shared among them.
void build_host_trees(const ddgi_scene_desc* d, const std::vector<float4>& pos, int leaf_max, float alpha,
                      std::vector<HostTree>& trees) {
    trees.assign(d->mesh_count, HostTree{});
    auto one = [&](uint32_t m, unsigned threads) {
        const ddgi_mesh& me = d->meshes[m];
        const uint32_t nt = me.index_count / 3;
        if (nt == 0) return;
        std::vector<float> tri((size_t)nt * 9);
        for (uint32_t t = 0; t < nt; ++t)
            for (int v = 0; v < 3; ++v) {
                const float4& p = pos[me.vertex_offset + d->indices[me.index_offset + 3 * t + v]];
                tri[9 * (size_t)t + 3 * v] = p.x;
                tri[9 * (size_t)t + 3 * v + 1] = p.y;
                tri[9 * (size_t)t + 3 * v + 2] = p.z;
            }
        sbvh_build(tri.data(), nt, leaf_max, alpha, 0, 0, trees[m].nodes, trees[m].order, &trees[m].depth, threads);
    };
    const unsigned hw = host_threads();
    std::vector<uint32_t> small;
    for (uint32_t m = 0; m < d->mesh_count; ++m) {
        if (d->meshes[m].index_count / 3 >= 65536u) one(m, hw);
        else small.push_back(m);
    }
    // largest first, so the long builds start early
    std::sort(small.begin(), small.end(),
              [&](uint32_t a, uint32_t b) { return d->meshes[a].index_count > d->meshes[b].index_count; });
    std::atomic<size_t> next{0};
    const unsigned nw = std::min<unsigned>(hw, (unsigned)small.size());
    const unsigned per = nw > 0 ? std::max(1u, hw / nw) : 1u;  // threads per mesh build
    auto worker = [&]() {
        for (size_t i = next.fetch_add(1); i < small.size(); i = next.fetch_add(1)) one(small[i], per);
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nw; ++t) {
        try {
            pool.emplace_back(worker);
        } catch (const std::system_error&) {
            break;
        }
    }
    worker();
    for (auto& th : pool) th.join();
}

// References of a host tree made absolute: inner + node_base, leaf first +
// prim_base.
void rebase_tree(std::vector<BvhNode>& nodes, int node_base, int prim_base) {
    for (BvhNode& n : nodes) {
        int* r[2] = {&n.d.x, &n.d.y};
        for (int s = 0; s < 2; ++s) {
            if (*r[s] >= 0) {
                *r[s] += node_base;
            } else {
                const int code = ~*r[s];
                *r[s] = ~((((code >> 3) + prim_base) << 3) | (code & 7));
            }
        }
    }
}

// Depth-first layout of every mesh tree of a linear BVH build (the
// fast-trace builders write theirs depth first already).
ddgi_status layout_depth_first(ddgi_ctx* ctx, const std::vector<int32_t>& mesh_root, cudaStream_t st) {
    SceneBuffers& S = ctx->scene;
    const uint32_t blas_end = S.tlas_root >= 0 ? (uint32_t)S.tlas_root : (uint32_t)S.node_count;
    if (blas_end == 0) return DDGI_OK;
    std::vector<BvhNode> bin(blas_end);
    CK(cudaMemcpyAsync(bin.data(), S.nodes, sizeof(BvhNode) * blas_end, cudaMemcpyDeviceToHost, st), "read trees");
    CK(cudaStreamSynchronize(st), "read trees");
    // mesh trees occupy consecutive ranges in mesh order, the top level follows
    std::vector<uint32_t> roots;
    for (int32_t r : mesh_root)
        if (r >= 0) roots.push_back((uint32_t)r);
    for (size_t i = 0; i < roots.size(); ++i) {
        const uint32_t e = i + 1 < roots.size() ? roots[i + 1] : blas_end;
        if (roots[i] < e && e <= blas_end) depth_first_layout(bin, roots[i], e);
    }
    CK(cudaMemcpyAsync(S.nodes, bin.data(), sizeof(BvhNode) * blas_end, cudaMemcpyHostToDevice, st),
       "upload mesh trees");
    CK(cudaStreamSynchronize(st), "upload mesh trees");  // `bin` is pageable and local
    return DDGI_OK;
}

// Eight-wide copies of every mesh tree and of the top level (node_width 8).
ddgi_status build_wide(ddgi_ctx* ctx, cudaStream_t st) {
    SceneBuffers& S = ctx->scene;
    const std::vector<int32_t>& mesh_root = S.mesh_root;
    S.wstack_cap = 0;
    if (S.node_count == 0) return DDGI_OK;
    std::vector<BvhNode> bin(S.node_count);
    CK(cudaMemcpyAsync(bin.data(), S.nodes, sizeof(BvhNode) * S.node_count, cudaMemcpyDeviceToHost, st),
       "read trees");
    CK(cudaStreamSynchronize(st), "read trees");
    std::vector<WideNode> w;
    bool ok = true;
    uint32_t lb = 0;
    S.wide_root_of_mesh.assign(mesh_root.size(), -1);
    for (size_t m = 0; m < mesh_root.size(); ++m) {
        if (mesh_root[m] < 0) continue;
        uint32_t lv = 0;
        S.wide_root_of_mesh[m] = collapse_wide(bin, mesh_root[m], w, &lv, &ok);
        lb = std::max(lb, lv);
    }
    if (!ok) return fail(ctx, DDGI_ERR_DEVICE, "malformed mesh tree");
    const uint32_t ni = (uint32_t)S.host_inst.size();
    S.wide_tlas_start = (uint32_t)w.size();
    S.wide_cap = S.wide_tlas_start + (ni > 1 ? ni - 1 : 1);
    S.wlevels_blas = lb;
    CK(cudaMalloc(&S.wnodes, sizeof(WideNode) * std::max<uint32_t>(S.wide_cap, 1)), "alloc wide nodes");
    CK(cudaMalloc(&S.winst_leaf, sizeof(GpuInstance) * std::max<uint32_t>(ni, 1)), "alloc wide instances");
    if (!w.empty())
        CK(cudaMemcpyAsync(S.wnodes, w.data(), sizeof(WideNode) * w.size(), cudaMemcpyHostToDevice, st), "upload");
    S.wnode_count = (uint32_t)w.size();
    S.wtlas_root = -1;
    if (S.tlas_root < 0) {
        S.wstack_cap = S.wnode_count < kMaxWideNodes ? (int)(lb + 4) : 0;
        return DDGI_OK;
    }
    return refresh_wide_top(ctx, st);
}

}  // namespace

}  // extern "C"

namespace ddgi {
// The eight-wide trees of the built scene, made on first use (they are
// collapsed from the binary trees on the host).
ddgi_status ensure_wide(ddgi_ctx* ctx) {
    SceneBuffers& S = ctx->scene;
    if (!S.built || S.wide_ready) return DDGI_OK;
    // every stream's work on the trees (an instance refit) is done
    CK(cudaDeviceSynchronize(), "synchronise before the wide trees");
    ddgi_status s = build_wide(ctx, nullptr);
    if (s == DDGI_OK) {
        cudaError_t e = cudaStreamSynchronize(nullptr);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "wide trees");
        S.wide_ready = true;
    }
    return s;
}
}  // namespace ddgi

extern "C" {

ddgi_status ddgi_scene_build(ddgi_ctx* ctx, const ddgi_scene_desc* d, ddgi_stream stream) {
    ddgi::NvtxRange nvtx_range("ddgi_scene_build");
    if (!ctx || !d) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // ---- validation (the reference would fault on any of these) ----
    if ((d->vertex_count && !d->vertices) || (d->index_count && !d->indices) || (d->mesh_count && !d->meshes) ||
        (d->instance_count && !d->instances) || (d->offset_count && !d->offsets) ||
        (d->material_count && !d->materials))
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "null array with a non-zero count");
    for (uint32_t m = 0; m < d->mesh_count; ++m) {
        const ddgi_mesh& me = d->meshes[m];
        if (me.index_count % 3) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "mesh %u: index_count not a multiple of 3", m);
        if ((uint64_t)me.index_offset + me.index_count > d->index_count ||
            (uint64_t)me.vertex_offset + me.vertex_count > d->vertex_count)
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "mesh %u: range outside the vertex/index arrays", m);
        for (uint32_t i = 0; i < me.index_count; ++i) {
            const uint32_t v = d->indices[me.index_offset + i];
            if (v >= me.vertex_count)
                return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "mesh %u: index %u out of range", m, i);
            const float* p = d->vertices[me.vertex_offset + v].pos;
            if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[2]))
                return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "mesh %u: vertex %u of a triangle is not finite", m, v);
        }
        if ((uint64_t)me.index_count / 3 >= (1ull << 28))
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "mesh %u: too many triangles", m);
    }
    for (uint32_t o = 0; o < d->offset_count; ++o) {
        const ddgi_offset_entry& oe = d->offsets[o];
        if (oe.material_index >= d->material_count)
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "offset entry %u: material out of range", o);
        if (oe.index_offset > d->index_count || oe.vertex_offset > d->vertex_count)
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "offset entry %u: offsets out of range", o);
    }
    std::vector<float> w2o((size_t)d->instance_count * 12);
    // (vertex_offset, index_offset, index_count) ranges already checked
    std::vector<std::array<uint32_t, 3>> checked;
    for (uint32_t i = 0; i < d->instance_count; ++i) {
        const ddgi_instance& in = d->instances[i];
        if (in.mesh_index >= d->mesh_count)
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u: mesh_index out of range", i);
        if ((in.custom_index & 0xFFFFFFu) >= d->offset_count)
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u: custom_index out of range", i);
        for (int k = 0; k < 12; ++k)
            if (!std::isfinite(in.transform[k]))
                return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u: non-finite transform", i);
        if (!ddgi_affine_inverse(in.transform, &w2o[(size_t)i * 12]))
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u: singular transform", i);
        // an instance's shading reads must stay inside the arrays
        const ddgi_offset_entry& oe = d->offsets[in.custom_index & 0xFFFFFFu];
        const ddgi_mesh& me = d->meshes[in.mesh_index];
        if ((uint64_t)oe.index_offset + me.index_count > d->index_count)
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u: offset entry index range too short", i);
        std::array<uint32_t, 3> key = {oe.vertex_offset, oe.index_offset, me.index_count};
        if (std::find(checked.begin(), checked.end(), key) == checked.end()) {
            for (uint32_t q = 0; q < me.index_count; ++q)
                if ((uint64_t)oe.vertex_offset + d->indices[oe.index_offset + q] >= d->vertex_count)
                    return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u: shading vertex out of range", i);
            checked.push_back(key);
        }
    }

    CK(cudaStreamSynchronize(st), "sync before scene build");
    free_scene(ctx->scene);
    SceneBuffers& S = ctx->scene;

    // ---- upload shading data ----
    std::vector<float4> pos(d->vertex_count), nrm(d->vertex_count);
    for (uint32_t v = 0; v < d->vertex_count; ++v) {
        const ddgi_vertex& vx = d->vertices[v];
        pos[v] = make_float4(vx.pos[0], vx.pos[1], vx.pos[2], 1.0f);
        nrm[v] = make_float4(vx.normal[0], vx.normal[1], vx.normal[2], 0.0f);
    }
    float4* dpos = nullptr;
    float* dsoup = nullptr;      // triangles as 9 floats (GPU fast-trace builder input)
    uint32_t* gorder = nullptr;  // leaf order of the GPU-built mesh trees
    void* scratch = nullptr;
    float4* box_lo = nullptr;
    float4* box_hi = nullptr;
    uint32_t* sorted = nullptr;
    uint32_t* depth = nullptr;  // [0] deepest mesh tree, [1] top-level tree
    auto cleanup = [&]() {
        if (dpos) cudaFree(dpos);
        if (dsoup) cudaFree(dsoup);
        if (gorder) cudaFree(gorder);
        if (scratch) cudaFree(scratch);
        if (box_lo) cudaFree(box_lo);
        if (box_hi) cudaFree(box_hi);
        if (sorted) cudaFree(sorted);
        if (depth) cudaFree(depth);
    };
#define CKB(call, what)                               \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) {                      \
            cleanup();                                \
            free_scene(ctx->scene);                   \
            return cuda_fail(ctx, e_, what);          \
        }                                             \
    } while (0)
    size_t vbytes = sizeof(float4) * std::max<uint32_t>(d->vertex_count, 1);
    CKB(cudaMalloc(&dpos, vbytes), "alloc positions");
    CKB(cudaMalloc(&S.normals, vbytes), "alloc normals");
    CKB(cudaMalloc(&S.indices, sizeof(uint32_t) * std::max<uint32_t>(d->index_count, 1)), "alloc indices");
    CKB(cudaMalloc(&S.offsets, sizeof(ddgi_offset_entry) * std::max<uint32_t>(d->offset_count, 1)), "alloc offsets");
    CKB(cudaMalloc(&S.materials, sizeof(ddgi_material) * std::max<uint32_t>(d->material_count, 1)), "alloc materials");
    if (d->vertex_count) {
        CKB(cudaMemcpyAsync(dpos, pos.data(), sizeof(float4) * d->vertex_count, cudaMemcpyHostToDevice, st), "upload");
        CKB(cudaMemcpyAsync(S.normals, nrm.data(), sizeof(float4) * d->vertex_count, cudaMemcpyHostToDevice, st), "upload");
    }
    if (d->index_count)
        CKB(cudaMemcpyAsync(S.indices, d->indices, sizeof(uint32_t) * d->index_count, cudaMemcpyHostToDevice, st), "upload");
    if (d->offset_count)
        CKB(cudaMemcpyAsync(S.offsets, d->offsets, sizeof(ddgi_offset_entry) * d->offset_count, cudaMemcpyHostToDevice, st),
            "upload");
    if (d->material_count)
        CKB(cudaMemcpyAsync(S.materials, d->materials, sizeof(ddgi_material) * d->material_count, cudaMemcpyHostToDevice,
                            st),
            "upload");

    // fast-trace mesh trees are built first: their node and triangle-reference
    // counts (spatial splits reference some triangles more than once) size
    // the device arrays
    const bool host_trees = ctx->build_mode == DDGI_BUILD_FAST_TRACE_HOST;
    const bool gpu_trees = ctx->build_mode == DDGI_BUILD_FAST_TRACE;
    std::vector<HostTree> trees;
    if (host_trees) build_host_trees(d, pos, ctx->blas_leaf_max, ctx->split_alpha, trees);
    GpuTreeBuilder gtb;
    if (gpu_trees) {
        std::vector<uint32_t> counts(d->mesh_count);
        uint64_t soup = 0;
        for (uint32_t m = 0; m < d->mesh_count; ++m) soup += counts[m] = d->meshes[m].index_count / 3;
        CKB(cudaMalloc(&dsoup, sizeof(float) * 9 * std::max<uint64_t>(soup, 1)), "alloc build triangles");
        uint64_t o = 0;
        for (uint32_t m = 0; m < d->mesh_count; ++m) {
            const ddgi_mesh& me = d->meshes[m];
            CKB(gather_triangle_soup(dpos, S.indices, me.vertex_offset, me.index_offset, counts[m], dsoup + 9 * o, st),
                "gather build triangles");
            o += counts[m];
        }
        CKB(gtb.build_triangles(dsoup, counts, ctx->blas_leaf_max, ctx->split_alpha, ctx->err, st), "mesh tree build");
        S.gpu_build_ms = gtb.build_ms();
    }
    uint64_t total_tris = 0, total_nodes = 0;
    uint32_t max_tris = 0;
    for (uint32_t m = 0; m < d->mesh_count; ++m) {
        uint32_t nt = d->meshes[m].index_count / 3;
        if (host_trees) {
            total_tris += trees[m].order.size();
            total_nodes += trees[m].nodes.size();
            max_tris = std::max(max_tris, (uint32_t)std::min<size_t>(trees[m].order.size(), 0xFFFFFFFFu));
            continue;
        }
        if (gpu_trees) {
            total_tris += gtb.ref_counts()[m];
            total_nodes += gtb.node_counts()[m];
            max_tris = std::max(max_tris, gtb.ref_counts()[m]);
            continue;
        }
        total_tris += nt;
        total_nodes += nt > 1 ? nt - 1 : (nt == 1 ? 1 : 0);
        max_tris = std::max(max_tris, nt);
    }
    uint32_t ni = d->instance_count;
    uint64_t tlas_nodes = ni > 1 ? ni - 1 : (ni == 1 ? 1 : 0);
    uint32_t max_prims = std::max(max_tris, ni);
    if (total_tris >= (1ull << 28) - 8 || total_nodes + tlas_nodes >= (1ull << 31)) {
        cleanup();
        free_scene(ctx->scene);
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "scene too large (%llu triangles)", (unsigned long long)total_tris);
    }
    CKB(cudaMalloc(&S.nodes, sizeof(BvhNode) * std::max<uint64_t>(total_nodes + tlas_nodes, 1)), "alloc nodes");
    CKB(cudaMalloc(&S.tris, sizeof(BvhTri) * std::max<uint64_t>(total_tris, 1)), "alloc triangles");
    CKB(cudaMalloc(&S.inst_leaf, sizeof(GpuInstance) * std::max<uint32_t>(ni, 1)), "alloc instances");
    CKB(cudaMalloc(&S.inst_id, sizeof(GpuInstance) * std::max<uint32_t>(ni, 1)), "alloc instances");
    CKB(cudaMalloc(&scratch, lbvh_scratch_bytes(std::max<uint32_t>(max_prims, 1))), "alloc build scratch");
    CKB(cudaMalloc(&box_lo, sizeof(float4) * std::max<uint32_t>(max_prims, 1)), "alloc build boxes");
    CKB(cudaMalloc(&box_hi, sizeof(float4) * std::max<uint32_t>(max_prims, 1)), "alloc build boxes");
    CKB(cudaMalloc(&sorted, sizeof(uint32_t) * std::max<uint32_t>(max_prims, 1)), "alloc build order");
    CKB(cudaMalloc(&depth, 2 * sizeof(uint32_t)), "alloc depth");
    if (gpu_trees) CKB(cudaMalloc(&gorder, sizeof(uint32_t) * std::max<uint64_t>(total_tris, 1)), "alloc leaf order");
    {
        const uint32_t one[2] = {1u, 1u};
        CKB(cudaMemcpyAsync(depth, one, sizeof(one), cudaMemcpyHostToDevice, st), "init depth");
    }

    // ---- bottom level: one tree per mesh ----
    S.build_mode = ctx->build_mode;
    uint32_t host_blas_depth = 1;
    std::vector<int32_t> mesh_root(d->mesh_count, -1);
    std::vector<float> mesh_lo((size_t)d->mesh_count * 3, INFINITY), mesh_hi((size_t)d->mesh_count * 3, -INFINITY);
    std::vector<int> gnode_base(d->mesh_count, 0), gprim_base(d->mesh_count, 0);
    std::vector<uint32_t> gorder_base(d->mesh_count, 0);
    uint64_t node_base = 0, tri_base = 0;
    for (uint32_t m = 0; m < d->mesh_count; ++m) {
        const ddgi_mesh& me = d->meshes[m];
        uint32_t nt = me.index_count / 3;
        if (nt == 0) continue;
        for (uint32_t q = 0; q < me.index_count; ++q) {
            const float4& p = pos[me.vertex_offset + d->indices[me.index_offset + q]];
            float pp[3] = {p.x, p.y, p.z};
            for (int k = 0; k < 3; ++k) {
                if (pp[k] == pp[k]) {
                    mesh_lo[m * 3 + k] = std::min(mesh_lo[m * 3 + k], pp[k]);
                    mesh_hi[m * 3 + k] = std::max(mesh_hi[m * 3 + k], pp[k]);
                }
            }
        }
        if (gpu_trees) {
            gnode_base[m] = (int)node_base;
            gprim_base[m] = (int)tri_base;
            gorder_base[m] = (uint32_t)tri_base;
            host_blas_depth = std::max(host_blas_depth, gtb.depths()[m]);
            mesh_root[m] = (int32_t)node_base;
            node_base += gtb.node_counts()[m];
            tri_base += gtb.ref_counts()[m];
            continue;
        }
        if (host_trees) {
            HostTree& tr = trees[m];
            rebase_tree(tr.nodes, (int)node_base, (int)tri_base);
            host_blas_depth = std::max(host_blas_depth, tr.depth);
            const uint32_t nref = (uint32_t)tr.order.size();
            // pageable sources: both copies have read them when they return
            CKB(cudaMemcpyAsync(S.nodes + node_base, tr.nodes.data(), sizeof(BvhNode) * tr.nodes.size(),
                                cudaMemcpyHostToDevice, st),
                "upload mesh tree");
            CKB(cudaMemcpyAsync(sorted, tr.order.data(), sizeof(uint32_t) * nref, cudaMemcpyHostToDevice, st),
                "upload leaf order");
            CKB(gather_mesh_tris(dpos, S.indices, me.vertex_offset, me.vertex_count, me.index_offset, nt, nref, sorted,
                                 S.tris + tri_base, st),
                "gather triangles");
            mesh_root[m] = (int32_t)node_base;
            node_base += tr.nodes.size();
            tri_base += nref;
            tr = HostTree{};
            continue;
        } else {
            CKB(build_mesh_blas(dpos, S.indices, me.vertex_offset, me.vertex_count, me.index_offset, nt,
                                ctx->blas_leaf_max, S.nodes, (int)node_base, S.tris, (int)tri_base, box_lo, box_hi,
                                sorted, scratch, ctx->err, depth, st),
                "bottom-level build");
        }
        mesh_root[m] = (int32_t)node_base;
        node_base += nt > 1 ? nt - 1 : 1;
        tri_base += nt;
    }
    if (gpu_trees) {
        CKB(gtb.write(S.nodes, gnode_base, gprim_base, gorder, gorder_base, st), "write mesh trees");
        for (uint32_t m = 0; m < d->mesh_count; ++m) {
            const ddgi_mesh& me = d->meshes[m];
            const uint32_t nt = me.index_count / 3;
            if (nt == 0) continue;
            CKB(gather_mesh_tris(dpos, S.indices, me.vertex_offset, me.vertex_count, me.index_offset, nt,
                                 gtb.ref_counts()[m], gorder + gorder_base[m], S.tris + gprim_base[m], st),
                "gather triangles");
        }
    }

    // ---- top level over instance world boxes ----
    S.host_inst.assign(ni, GpuInstance{});
    S.inst_lo.assign(ni, make_float4(0, 0, 0, 0));
    S.inst_hi.assign(ni, make_float4(0, 0, 0, 0));
    S.mesh_of_inst.assign(ni, 0);
    S.mesh_lo = mesh_lo;
    S.mesh_hi = mesh_hi;
    for (uint32_t i = 0; i < ni; ++i) {
        const ddgi_instance& in = d->instances[i];
        GpuInstance& r = S.host_inst[i];
        const float* w = &w2o[(size_t)i * 12];
        for (int k = 0; k < 3; ++k) r.w2o[k] = make_float4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
        r.blas_root = mesh_root[in.mesh_index];
        r.custom = in.custom_index & 0xFFFFFFu;
        r.mask = in.mask & 0xFFu;
        r.id = i;
        S.mesh_of_inst[i] = in.mesh_index;
        instance_world_box(in.transform, &mesh_lo[(size_t)in.mesh_index * 3], &mesh_hi[(size_t)in.mesh_index * 3],
                           r.blas_root >= 0, &S.inst_lo[i], &S.inst_hi[i]);
    }
    {
        ddgi_status ts = build_top_level(ctx, node_base, scratch, box_lo, box_hi, sorted, depth + 1, st);
        if (ts != DDGI_OK) {
            cleanup();
            free_scene(ctx->scene);
            return ts;
        }
    }
    uint32_t depths[2] = {1u, 1u};
    CKB(cudaMemcpyAsync(depths, depth, sizeof(depths), cudaMemcpyDeviceToHost, st), "read depth");
    CKB(cudaStreamSynchronize(st), "scene build");
    cleanup();
#undef CKB
    depths[0] = std::max(depths[0], host_blas_depth);
    // traversal stack: one entry per inner node on a root-to-leaf path in each
    // level, plus the resume node and the EXIT marker of an instance entry
    S.stack_cap = (int)(depths[0] + depths[1] + 4);
    S.depth_blas = depths[0];
    S.depth_tlas = depths[1];
    if (S.stack_cap > kMaxStack) {
        free_scene(ctx->scene);
        return fail(ctx, DDGI_ERR_UNSUPPORTED, "trees too deep for the traversal stack (%u + %u levels)", depths[0],
                    depths[1]);
    }
    S.vertex_count = d->vertex_count;
    S.index_count = d->index_count;
    S.offset_count = d->offset_count;
    S.material_count = d->material_count;
    S.instance_count = ni;
    S.node_count = total_nodes + tlas_nodes;
    S.tri_count = total_tris;
    S.mesh_root = mesh_root;
    if (S.build_mode == DDGI_BUILD_FAST_BUILD) {
        ddgi_status ls = layout_depth_first(ctx, mesh_root, st);
        if (ls != DDGI_OK) {
            free_scene(ctx->scene);
            return ls;
        }
    }
    S.build_id = next_build_id();
    S.built = true;
    if (ctx->tune.node_width == 8) {  // the wide copies are made when first asked for
        ddgi_status ws = ensure_wide(ctx);
        if (ws != DDGI_OK) {
            free_scene(ctx->scene);
            return ws;
        }
    }
    return check_device_error(ctx);
}



// ---------------------------------------------------------------------------
// Moving instances (Renderer::updateAccelerationStructureInstances +
// updateTLAS, src/Renderer.cpp:671-742)
// ---------------------------------------------------------------------------
ddgi_status ddgi_update_instances(ddgi_ctx* ctx, const uint32_t* ids, const float* transforms, uint32_t count,
                                  int rebuild, ddgi_stream stream) {
    ddgi::NvtxRange nvtx_range("ddgi_update_instances");
    if (!ctx || (count && !transforms)) return DDGI_ERR_INVALID_ARGUMENT;
    SceneBuffers& S = ctx->scene;
    if (!S.built) return fail(ctx, DDGI_ERR_NO_SCENE, "ddgi_update_instances before ddgi_scene_build");
    const uint32_t ni = (uint32_t)S.host_inst.size();
    if (count > ni) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "%u transforms for %u instances", count, ni);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // validate everything before changing anything
    std::vector<float> w2o((size_t)count * 12);
    std::vector<uint8_t> seen(ni, 0);
    for (uint32_t q = 0; q < count; ++q) {
        const uint32_t id = ids ? ids[q] : q;
        if (id >= ni) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u out of range", id);
        if (seen[id]++) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u listed twice", id);
        for (int k = 0; k < 12; ++k)
            if (!std::isfinite(transforms[12 * (size_t)q + k]))
                return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u: non-finite transform", id);
        if (!ddgi_affine_inverse(&transforms[12 * (size_t)q], &w2o[12 * (size_t)q]))
            return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "instance %u: singular transform", id);
    }
    for (uint32_t q = 0; q < count; ++q) {
        const uint32_t id = ids ? ids[q] : q;
        GpuInstance& r = S.host_inst[id];
        const float* w = &w2o[12 * (size_t)q];
        for (int k = 0; k < 3; ++k) r.w2o[k] = make_float4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
        const uint32_t m = S.mesh_of_inst[id];
        instance_world_box(&transforms[12 * (size_t)q], &S.mesh_lo[(size_t)m * 3], &S.mesh_hi[(size_t)m * 3],
                           r.blas_root >= 0, &S.inst_lo[id], &S.inst_hi[id]);
    }
    if (ni == 0) return DDGI_OK;
    if (rebuild) {
        // a new top-level tree over the new boxes (same node range)
        void* scratch = nullptr;
        float4 *blo = nullptr, *bhi = nullptr;
        uint32_t *sorted = nullptr, *depth = nullptr;
        auto release = [&]() {
            if (scratch) cudaFree(scratch);
            if (blo) cudaFree(blo);
            if (bhi) cudaFree(bhi);
            if (sorted) cudaFree(sorted);
            if (depth) cudaFree(depth);
        };
        if (cudaMalloc(&scratch, lbvh_scratch_bytes(ni)) != cudaSuccess ||
            cudaMalloc(&blo, sizeof(float4) * ni) != cudaSuccess || cudaMalloc(&bhi, sizeof(float4) * ni) != cudaSuccess ||
            cudaMalloc(&sorted, sizeof(uint32_t) * ni) != cudaSuccess ||
            cudaMalloc(&depth, sizeof(uint32_t)) != cudaSuccess) {
            release();
            cudaGetLastError();
            return fail(ctx, DDGI_ERR_OUT_OF_MEMORY, "instance rebuild scratch");
        }
        const uint32_t one = 1;
        uint32_t dtop = 1;
        ddgi_status s = DDGI_OK;
        if (cudaMemcpyAsync(depth, &one, sizeof(one), cudaMemcpyHostToDevice, st) != cudaSuccess)
            s = fail(ctx, DDGI_ERR_CUDA, "instance rebuild");
        if (s == DDGI_OK) s = build_top_level(ctx, (uint64_t)S.tlas_root, scratch, blo, bhi, sorted, depth, st);
        if (s == DDGI_OK && (cudaMemcpyAsync(&dtop, depth, sizeof(dtop), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                             cudaStreamSynchronize(st) != cudaSuccess))
            s = fail(ctx, DDGI_ERR_CUDA, "instance rebuild");
        release();
        if (s != DDGI_OK) return s;
        const int cap = (int)(S.depth_blas + dtop + 4);
        if (cap > kMaxStack)
            return fail(ctx, DDGI_ERR_UNSUPPORTED, "rebuilt top level too deep (%u levels)", dtop);
        S.depth_tlas = dtop;
        S.stack_cap = cap;
    } else {
        // refit: same topology, new leaf boxes, boxes recomputed bottom-up
        std::vector<GpuInstance> leaf(ni);
        std::vector<float4> llo(ni), lhi(ni);
        for (uint32_t id = 0; id < ni; ++id) {
            const uint32_t slot = S.leaf_of_id[id];
            leaf[slot] = S.host_inst[id];
            llo[slot] = S.inst_lo[id];
            lhi[slot] = S.inst_hi[id];
        }
        CK(cudaMemcpyAsync(S.inst_leaf, leaf.data(), sizeof(GpuInstance) * ni, cudaMemcpyHostToDevice, st), "upload");
        CK(cudaMemcpyAsync(S.inst_id, S.host_inst.data(), sizeof(GpuInstance) * ni, cudaMemcpyHostToDevice, st),
           "upload");
        CK(cudaMemcpyAsync(S.leaf_lo, llo.data(), sizeof(float4) * ni, cudaMemcpyHostToDevice, st), "upload");
        CK(cudaMemcpyAsync(S.leaf_hi, lhi.data(), sizeof(float4) * ni, cudaMemcpyHostToDevice, st), "upload");
        CK(lbvh_refit_top(S.nodes, S.tlas_root, S.leaf_lo, S.leaf_hi, ni, S.leaf_parent, S.node_parent, S.refit_flags,
                          S.sub_lo, S.sub_hi, ctx->err, st),
           "top-level refit");
        // the host vectors above are staged by the copies before they return
    }
    {
        ddgi_status ws = refresh_wide_top(ctx, st);
        if (ws != DDGI_OK) return ws;
    }
    S.build_id = next_build_id();  // batches made from the old top level are stale
    return DDGI_OK;
}

// ---------------------------------------------------------------------------
// Update (IrradianceProbes::update, src/IrradianceProbes.cpp:426-594)
// ---------------------------------------------------------------------------
namespace {

// Validates the request, uploads the direction table, the octant-binned ray
// order and the probe list; returns the device probe list (NULL = all).
ddgi_status prepare_update(ddgi_ctx* ctx, const float orientation[9], const uint32_t* probe_list,
                           uint32_t probe_count, cudaStream_t st, const uint32_t** dlist, uint32_t* n_out) {
    if (!ctx->scene.built) return fail(ctx, DDGI_ERR_NO_SCENE, "ddgi_update before ddgi_scene_build");
    for (int k = 0; k < 9; ++k)
        if (!std::isfinite(orientation[k])) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "non-finite orientation");
    const uint32_t P = probe_count_of(ctx->grid);
    const uint32_t R = ctx->grid.rays_per_probe;
    uint32_t n = probe_list ? probe_count : P;
    if (probe_list) {
        if (probe_count > P) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "probe list longer than the grid");
        std::vector<uint8_t> seen(P, 0);
        for (uint32_t i = 0; i < probe_count; ++i) {
            if (probe_list[i] >= P) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "probe %u out of range", probe_list[i]);
            if (seen[probe_list[i]]++) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "probe %u listed twice", probe_list[i]);
        }
    }
    // direction table (exact host definition) and octant-binned ray order
    ctx->host_dirs.resize(4 * (size_t)R);
    ddgi_ray_direction_table(orientation, R, ctx->host_dirs.data());
    ctx->host_order.resize(R);
    {
        const uint32_t rpw = ctx->tune.rays_per_warp;
        ray_order_of(ctx->host_dirs.data(), R, ctx->host_order.data(), rpw > 0 && rpw < 32);
    }
    CK(cudaMemcpyAsync(ctx->dirs, ctx->host_dirs.data(), sizeof(float4) * R, cudaMemcpyHostToDevice, st), "upload dirs");
    CK(cudaMemcpyAsync(ctx->ray_order, ctx->host_order.data(), sizeof(uint32_t) * R, cudaMemcpyHostToDevice, st),
       "upload order");
    *dlist = nullptr;
    if (probe_list && n > 0) {
        CK(cudaMemcpyAsync(ctx->probe_list, probe_list, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st), "upload list");
        *dlist = ctx->probe_list;
    }
    ddgi_status s = ensure_ray_capacity(ctx, (size_t)n * R);
    if (s != DDGI_OK) return s;
    *n_out = n;
    return DDGI_OK;
}

TraceTuning trace_tuning(const ddgi_ctx* ctx) {
    TraceTuning t;
    t.ctas_per_sm = ctx->tune.ctas_per_sm;
    t.refill = ctx->tune.refill_lanes;
    t.split = ctx->tune.smem_stack;
    t.rays_per_warp = ctx->tune.rays_per_warp;
    t.wide = ctx->tune.node_width == 8 ? 1u : 0u;
    t.wait = ctx->tune.straggler_lanes;
    return t;
}

// One-shot test hook: true once after ddgi_inject_fault(DDGI_FAULT_STALL_TENSOR_WAIT).
bool take_stall(ddgi_ctx* ctx) {
    const bool s = (ctx->inject & DDGI_FAULT_STALL_TENSOR_WAIT) != 0;
    ctx->inject &= ~(uint32_t)DDGI_FAULT_STALL_TENSOR_WAIT;
    return s;
}

// Blend + border copy of the ray records in ctx->rays, by the context's
// precision and pipeline: the BF16 tensor-core kernel; the FP32 kernel with
// the weights computed once per update (wavefront); the per-probe FP32
// kernel that computes them per texel like the reference's shader (fused).
// hyst: the ramp's hysteresis in device memory (NULL: the grid's); dcount:
// the selected probe count on the device (NULL: n).
cudaError_t launch_blend(ddgi_ctx* ctx, const uint32_t* dlist, uint32_t n, cudaStream_t st,
                         const float* hyst = nullptr, const uint32_t* dcount = nullptr) {
    if (ctx->fp16)
        return launch_blend_tc(ctx->dg, dlist, n, ctx->rays, ctx->dirs, ctx->tc_weights, ctx->tc_rowsum, ctx->states,
                               ctx->color, ctx->depth, ctx->acc_color, ctx->acc_depth, ctx->err, st, dcount,
                               take_stall(ctx), hyst);
    if (ctx->pipeline == DDGI_PIPELINE_WAVEFRONT)
        return launch_blend_fp32_shared(ctx->dg, dlist, n, ctx->rays, ctx->dirs,
                                        reinterpret_cast<float*>(ctx->tc_weights), ctx->tc_rowsum, ctx->states,
                                        static_cast<float4*>(ctx->color), static_cast<float2*>(ctx->depth), st,
                                        dcount, hyst);
    return launch_blend_fp32(ctx->dg, dlist, n, ctx->rays, ctx->dirs, ctx->states, static_cast<float4*>(ctx->color),
                             static_cast<float2*>(ctx->depth), st, dcount, hyst);
}

// The hysteresis ramp step of an update when the ramp is on (count: the
// update's probes, or *dcount on the device); returns the blended value's
// device address, or NULL when the grid's hysteresis applies.
const float* ramp_step(ddgi_ctx* ctx, const uint32_t* dcount, uint32_t count, cudaStream_t st, cudaError_t* e) {
    *e = cudaSuccess;
    if (!ctx->ramp_on) return nullptr;
    *e = launch_hysteresis_ramp(ctx->sched, ctx->ramp_cmd, dcount, count, probe_count_of(ctx->grid), st);
    ctx->ramp_cmd.set = 0;
    return reinterpret_cast<const float*>(ctx->sched + 4);
}

}  // namespace

ddgi_status ddgi_blend_records(ddgi_ctx* ctx, const float orientation[9], const uint32_t* probe_list,
                               uint32_t probe_count, const float* records, size_t count, ddgi_stream stream) {
    if (!ctx || !orientation || !records) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t n = probe_list ? probe_count : probe_count_of(ctx->grid);
    if (count != (size_t)n * ctx->grid.rays_per_probe)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "expected %zu ray records", (size_t)n * ctx->grid.rays_per_probe);
    // the blend needs no scene: mark one as present only for the preparation step
    const bool built = ctx->scene.built;
    ctx->scene.built = true;
    const uint32_t* dlist = nullptr;
    uint32_t n2 = 0;
    ddgi_status s = prepare_update(ctx, orientation, probe_list, probe_count, st, &dlist, &n2);
    ctx->scene.built = built;
    if (s != DDGI_OK) return s;
    CK(cudaMemcpyAsync(ctx->rays, records, count * sizeof(float4), cudaMemcpyHostToDevice, st), "upload records");
    CK(launch_blend(ctx, dlist, n, st), "blend launch");
    CK(cudaStreamSynchronize(st), "blend");
    ctx->last_count = n;
    ctx->last_rays = ctx->grid.rays_per_probe;
    return check_device_error(ctx);
}

ddgi_status ddgi_update(ddgi_ctx* ctx, const float orientation[9], const uint32_t* probe_list, uint32_t probe_count,
                        ddgi_stream stream) {
    ddgi::NvtxRange nvtx_range("ddgi_update");
    if (!ctx || !orientation) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t* dlist = nullptr;
    uint32_t n = 0;
    ddgi_status s = prepare_update(ctx, orientation, probe_list, probe_count, st, &dlist, &n);
    if (s != DDGI_OK) return s;
    DeviceScene sc = device_scene(ctx);
    if (ctx->timing) CK(cudaEventRecord(ctx->ev[0], st), "event");
    ddgi_hit* hits_out = ctx->record_hits ? ctx->hits : nullptr;
    if (ctx->pipeline == DDGI_PIPELINE_FUSED) {
        CK(launch_trace_shade(sc, ctx->dg, ctx->dl, dlist, n, ctx->dirs, ctx->ray_order, ctx->states, ctx->color,
                              ctx->depth, ctx->fp16, ctx->rays, hits_out, ctx->err, st),
           "trace launch");
        if (ctx->timing) CK(cudaEventRecord(ctx->ev[3], st), "event");
    } else {
        WaveHits wh{ctx->wave_thit, ctx->wave_prim, ctx->wave_front};
        ShadowQueue q{ctx->q_idx, ctx->q_pos, ctx->q_sun, nullptr};
        CK(launch_wavefront(sc, ctx->dg, ctx->dl, dlist, n, ctx->dirs, ctx->ray_order, ctx->states, ctx->color,
                            ctx->depth, ctx->fp16, wh, q, ctx->counters, ctx->rays, hits_out, ctx->scene.stack_cap,
                            ctx->scene.wstack_cap, ctx->err, st, ctx->timing ? ctx->ev[3] : nullptr, nullptr,
                            trace_tuning(ctx), ctx->probe_perm),
           "wavefront trace launch");
    }
    if (ctx->dl.sky_mode == DDGI_SKY_ATMOSPHERE)
        CK(launch_shade_sky(ctx->dg, ctx->dl, n, nullptr, dlist, ctx->dirs, ctx->rays, st), "sky launch");
    if (ctx->timing) CK(cudaEventRecord(ctx->ev[1], st), "event");
    cudaError_t re;
    const float* hyst = ramp_step(ctx, nullptr, n, st, &re);
    CK(re, "hysteresis ramp launch");
    CK(launch_blend(ctx, dlist, n, st, hyst), "blend launch");
    if (ctx->timing) {
        CK(cudaEventRecord(ctx->ev[2], st), "event");
        ctx->timing_pending = true;
    }
    ctx->last_count = n;
    ctx->last_rays = ctx->grid.rays_per_probe;
    return DDGI_OK;
}

// ---------------------------------------------------------------------------
// Probe classification and adaptive schedule (IrradianceProbes::initProbes,
// src/IrradianceProbes.cpp:357-394, and selectProbesToUpdate, :396-424)
// ---------------------------------------------------------------------------
ddgi_status ddgi_init_probes(ddgi_ctx* ctx, const float orientation[9], ddgi_stream stream) {
    ddgi::NvtxRange nvtx_range("ddgi_init_probes");
    if (!ctx || !orientation) return DDGI_ERR_INVALID_ARGUMENT;
    if (!ctx->scene.built) return fail(ctx, DDGI_ERR_NO_SCENE, "ddgi_init_probes before ddgi_scene_build");
    for (int k = 0; k < 9; ++k)
        if (!std::isfinite(orientation[k])) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "non-finite orientation");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t P = probe_count_of(ctx->grid);
    if (!ctx->init_dirs) {
        CK(cudaMalloc(&ctx->init_dirs, sizeof(float4) * kInitRays), "alloc init directions");
        CK(cudaMalloc(&ctx->init_back, sizeof(uint32_t) * P), "alloc init counters");
        CK(cudaMalloc(&ctx->init_near, sizeof(uint32_t) * P), "alloc init counters");
    }
    // probesInit.rgen:41-42: direction i of 512 from the raysPerProbe-point
    // spherical Fibonacci set (i >= raysPerProbe: the degenerate directions
    // the shader's formula gives there)
    std::vector<float> d(4 * (size_t)kInitRays);
    for (uint32_t i = 0; i < kInitRays; ++i) ddgi_ray_direction(orientation, i, ctx->grid.rays_per_probe, &d[4 * i]);
    CK(cudaMemcpyAsync(ctx->init_dirs, d.data(), sizeof(float4) * kInitRays, cudaMemcpyHostToDevice, st), "upload");
    CK(launch_init_probes(device_scene(ctx), ctx->dg, ctx->init_dirs, P, ctx->init_back, ctx->init_near, ctx->states,
                          ctx->counters, ctx->scene.stack_cap, ctx->err, st),
       "init launch");
    CK(cudaStreamSynchronize(st), "init probes");  // also keeps `d` alive for the copy
    if (ctx->ramp_on) {  // initProbes restarts the ramp's host value (IrradianceProbes.cpp:357-358)
        ctx->ramp_cmd.set |= kRampSetParam;
        ctx->ramp_cmd.param = 0.0f;
    }
    return check_device_error(ctx);
}

ddgi_status ddgi_update_scheduled(ddgi_ctx* ctx, const float orientation[9], uint32_t max_probes, ddgi_stream stream) {
    ddgi::NvtxRange nvtx_range("ddgi_update_scheduled");
    if (!ctx || !orientation) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t* unused = nullptr;
    uint32_t P = 0;
    ddgi_status s = prepare_update(ctx, orientation, nullptr, 0, st, &unused, &P);
    if (s != DDGI_OK) return s;
    uint32_t* dcount = ctx->sched + 2;
    if (ctx->timing) CK(cudaEventRecord(ctx->ev[0], st), "event");
    CK(launch_select_probes(ctx->states, P, max_probes, ctx->sched, ctx->probe_list, st), "schedule launch");
    WaveHits wh{ctx->wave_thit, ctx->wave_prim, ctx->wave_front};
    ShadowQueue q{ctx->q_idx, ctx->q_pos, ctx->q_sun, nullptr};
    ddgi_hit* hits_out = ctx->record_hits ? ctx->hits : nullptr;
    CK(launch_wavefront(device_scene(ctx), ctx->dg, ctx->dl, ctx->probe_list, P, ctx->dirs, ctx->ray_order,
                        ctx->states, ctx->color, ctx->depth, ctx->fp16, wh, q, ctx->counters, ctx->rays, hits_out,
                        ctx->scene.stack_cap, ctx->scene.wstack_cap, ctx->err, st,
                        ctx->timing ? ctx->ev[3] : nullptr, dcount, trace_tuning(ctx), nullptr),
       "wavefront trace launch");
    if (ctx->dl.sky_mode == DDGI_SKY_ATMOSPHERE)
        CK(launch_shade_sky(ctx->dg, ctx->dl, P, dcount, ctx->probe_list, ctx->dirs, ctx->rays, st), "sky launch");
    if (ctx->timing) CK(cudaEventRecord(ctx->ev[1], st), "event");
    cudaError_t re;
    const float* hyst = ramp_step(ctx, dcount, 0, st, &re);
    CK(re, "hysteresis ramp launch");
    CK(launch_blend(ctx, ctx->probe_list, P, st, hyst, dcount), "blend launch");
    if (ctx->timing) {
        CK(cudaEventRecord(ctx->ev[2], st), "event");
        ctx->timing_pending = true;
    }
    ctx->last_count = P;  // records of the selected probes come first
    ctx->last_rays = ctx->grid.rays_per_probe;
    return DDGI_OK;
}

ddgi_status ddgi_get_schedule(ddgi_ctx* ctx, uint32_t* count, uint32_t* offset, uint32_t* loop, uint32_t* list,
                              size_t list_capacity, ddgi_stream stream) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    uint32_t h[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(h, ctx->sched, sizeof(h), cudaMemcpyDeviceToHost, st), "read schedule");
    CK(cudaStreamSynchronize(st), "read schedule");
    if (offset) *offset = h[0];
    if (loop) *loop = h[1];
    if (count) *count = h[2];
    if (list) {
        if (list_capacity < h[2]) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "list holds %zu of %u", list_capacity, h[2]);
        if (h[2])
            CK(cudaMemcpy(list, ctx->probe_list, sizeof(uint32_t) * h[2], cudaMemcpyDeviceToHost), "read schedule");
    }
    return DDGI_OK;
}

ddgi_status ddgi_set_schedule(ddgi_ctx* ctx, uint32_t offset, uint32_t loop, ddgi_stream stream) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    if (offset >= probe_count_of(ctx->grid))
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "offset %u outside the grid", offset);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t h[4] = {offset, loop, 0, 0};
    CK(cudaMemcpyAsync(ctx->sched, h, sizeof(h), cudaMemcpyHostToDevice, st), "write schedule");
    CK(cudaStreamSynchronize(st), "write schedule");
    return DDGI_OK;
}

// ---------------------------------------------------------------------------
// Final gather (src/shaders/FinalGather.frag:39-80)
// ---------------------------------------------------------------------------
ddgi_status ddgi_final_gather(ddgi_ctx* ctx, const ddgi_gbuffer* gb, const float camera_origin[3], float* color_out,
                              ddgi_stream stream) {
    ddgi::NvtxRange nvtx_range("ddgi_final_gather");
    if (!ctx || !gb || !camera_origin || !color_out) return DDGI_ERR_INVALID_ARGUMENT;
    const uint64_t px = (uint64_t)gb->width * gb->height;
    if (px == 0) return DDGI_OK;
    if (px >= (1ull << 31)) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "G-buffer too large");
    if (!gb->position_depth || !gb->normal_metalness || !gb->albedo_roughness || !gb->emissive || !gb->direct_light)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "a required G-buffer array is NULL");
    const uintptr_t al = (uintptr_t)gb->position_depth | (uintptr_t)gb->normal_metalness |
                         (uintptr_t)gb->albedo_roughness | (uintptr_t)gb->emissive | (uintptr_t)gb->reflection |
                         (uintptr_t)color_out;
    if (al & 15u) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "float4 G-buffer arrays must be 16-byte aligned");
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(camera_origin[k])) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "non-finite camera origin");
    GatherArgs a;
    a.position_depth = reinterpret_cast<const float4*>(gb->position_depth);
    a.normal_metalness = reinterpret_cast<const float4*>(gb->normal_metalness);
    a.albedo_roughness = reinterpret_cast<const float4*>(gb->albedo_roughness);
    a.emissive = reinterpret_cast<const float4*>(gb->emissive);
    a.direct_light = gb->direct_light;
    a.reflection = reinterpret_cast<const float4*>(gb->reflection);
    a.out = reinterpret_cast<float4*>(color_out);
    a.pixels = (uint32_t)px;
    a.origin = make_float3(camera_origin[0], camera_origin[1], camera_origin[2]);
    a.g = ctx->dg;
    a.L = ctx->dl;
    a.states = ctx->states;
    CK(launch_final_gather(a, ctx->color, ctx->depth, ctx->fp16, reinterpret_cast<cudaStream_t>(stream)),
       "final gather launch");
    return DDGI_OK;
}

// ---------------------------------------------------------------------------
// Traversal launch tuning
// ---------------------------------------------------------------------------
ddgi_status ddgi_set_trace_tuning(ddgi_ctx* ctx, const ddgi_trace_tuning* t) {
    if (!ctx || !t) return DDGI_ERR_INVALID_ARGUMENT;
    const uint32_t r = t->rays_per_warp;
    if (!(r == 0 || r == 1 || r == 2 || r == 4 || r == 8 || r == 16 || r == 32))
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "rays_per_warp = %u: want 0, 1, 2, 4, 8, 16 or 32", r);
    if (t->refill_lanes < 1 || t->refill_lanes > 32)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "refill_lanes = %u outside [1, 32]", t->refill_lanes);
    if (t->smem_stack > (uint32_t)kMaxStack || t->ctas_per_sm > 32)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "smem_stack or ctas_per_sm out of range");
    if (t->node_width != 2 && t->node_width != 8)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "node_width = %u: want 2 or 8", t->node_width);
    if (t->straggler_lanes > 31)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "straggler_lanes = %u outside [0, 31]", t->straggler_lanes);
    ctx->tune = *t;
    return t->node_width == 8 ? ensure_wide(ctx) : DDGI_OK;
}

ddgi_status ddgi_set_leaf_size(ddgi_ctx* ctx, uint32_t max_triangles) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    if (max_triangles < 1 || max_triangles > 8)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "leaf size %u outside [1, 8]", max_triangles);
    ctx->blas_leaf_max = (int)max_triangles;
    return DDGI_OK;
}

ddgi_status ddgi_inject_fault(ddgi_ctx* ctx, uint32_t faults) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    if (faults & ~(uint32_t)DDGI_FAULT_STALL_TENSOR_WAIT)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "unknown fault bits 0x%x", faults);
    ctx->inject |= faults;
    return DDGI_OK;
}

ddgi_status ddgi_set_spatial_splits(ddgi_ctx* ctx, float overlap) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    if (!(overlap >= 0.0f && overlap <= 1.0f))
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "spatial-split overlap %g outside [0, 1]", (double)overlap);
    ctx->split_alpha = overlap;
    return DDGI_OK;
}

ddgi_status ddgi_set_build_mode(ddgi_ctx* ctx, ddgi_build_mode mode) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    if (mode != DDGI_BUILD_FAST_TRACE && mode != DDGI_BUILD_FAST_BUILD && mode != DDGI_BUILD_FAST_TRACE_HOST)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "unknown build mode %d", (int)mode);
    ctx->build_mode = mode;
    return DDGI_OK;
}

ddgi_status ddgi_get_scene_info(const ddgi_ctx* ctx, ddgi_scene_info* out) {
    if (!ctx || !out) return DDGI_ERR_INVALID_ARGUMENT;
    const SceneBuffers& S = ctx->scene;
    if (!S.built) return DDGI_ERR_NO_SCENE;
    out->node_count = S.node_count;
    out->tri_refs = S.tri_count;
    out->depth_blas = S.depth_blas;
    out->depth_tlas = S.depth_tlas;
    out->build_mode = (uint32_t)S.build_mode;
    out->tree_build_ms = S.build_mode == DDGI_BUILD_FAST_TRACE ? S.gpu_build_ms : 0.0f;
    return DDGI_OK;
}

ddgi_status ddgi_read_trees(ddgi_ctx* ctx, void* nodes, uint64_t node_capacity, void* tris, uint64_t tri_capacity,
                            ddgi_stream stream) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    const SceneBuffers& S = ctx->scene;
    if (!S.built) return fail(ctx, DDGI_ERR_NO_SCENE, "ddgi_read_trees before ddgi_scene_build");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t nn = std::min<uint64_t>(node_capacity, S.node_count), nt = std::min<uint64_t>(tri_capacity, S.tri_count);
    if (nodes && nn) CK(cudaMemcpyAsync(nodes, S.nodes, sizeof(BvhNode) * nn, cudaMemcpyDeviceToHost, st), "read nodes");
    if (tris && nt) CK(cudaMemcpyAsync(tris, S.tris, sizeof(BvhTri) * nt, cudaMemcpyDeviceToHost, st), "read triangles");
    CK(cudaStreamSynchronize(st), "read trees");
    return DDGI_OK;
}

ddgi_status ddgi_get_trace_tuning(const ddgi_ctx* ctx, ddgi_trace_tuning* out) {
    if (!ctx || !out) return DDGI_ERR_INVALID_ARGUMENT;
    *out = ctx->tune;
    return DDGI_OK;
}

ddgi_status ddgi_autotune(ddgi_ctx* ctx, const float orientation[9], uint32_t reps, ddgi_stream stream,
                          ddgi_trace_tuning* chosen) {
    if (!ctx || !orientation) return DDGI_ERR_INVALID_ARGUMENT;
    if (!ctx->scene.built) return fail(ctx, DDGI_ERR_NO_SCENE, "ddgi_autotune before ddgi_scene_build");
    {
        ddgi_status ws = ensure_wide(ctx);  // node_width 8 is one of the candidates
        if (ws != DDGI_OK) return ws;
    }
    if (reps == 0) reps = 3;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // save what the trial updates overwrite
    struct Saved {
        void* dst;
        void* copy;
        size_t bytes;
    };
    std::vector<Saved> saved;
    const size_t cb = atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, ctx->fp16), db = atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, ctx->fp16);
    // the schedule and hysteresis-ramp words too: the trial updates step the
    // ramp when it is on (its pending host-side commands are kept below)
    std::vector<std::pair<void*, size_t>> parts = {{ctx->color, cb},
                                                   {ctx->depth, db},
                                                   {ctx->states, sizeof(uint32_t) * probe_count_of(ctx->grid)},
                                                   {ctx->sched, 8 * sizeof(uint32_t)}};
    if (ctx->fp16) {
        parts.push_back({ctx->acc_color, atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, false)});
        parts.push_back({ctx->acc_depth, atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, false)});
    }
    auto release = [&]() {
        for (auto& x : saved) cudaFree(x.copy);
        saved.clear();
    };
    for (auto& pt : parts) {
        void* c = nullptr;
        if (cudaMalloc(&c, pt.second) != cudaSuccess) {
            cudaGetLastError();
            release();
            return fail(ctx, DDGI_ERR_OUT_OF_MEMORY, "autotune: no room to save the atlases");
        }
        saved.push_back({pt.first, c, pt.second});
        CK(cudaMemcpyAsync(c, pt.first, pt.second, cudaMemcpyDeviceToDevice, st), "autotune save");
    }
    const ddgi_trace_tuning start = ctx->tune;
    const RampCmd ramp_cmd = ctx->ramp_cmd;
    const bool timing = ctx->timing;
    ctx->timing = true;
    auto measure = [&](const ddgi_trace_tuning& t, float* out) -> ddgi_status {
        ctx->tune = t;
        std::vector<float> v;
        for (uint32_t r = 0; r <= reps; ++r) {  // the first run is not timed
            ddgi_status q = ddgi_update(ctx, orientation, nullptr, 0, stream);
            if (q != DDGI_OK) return q;
            CK(cudaEventSynchronize(ctx->ev[2]), "autotune");
            ctx->timing_pending = false;
            float a = 0.0f;
            cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);  // trace: primary + shading + shadow rays
            if (r > 0) v.push_back(a);
        }
        std::sort(v.begin(), v.end());
        *out = v[v.size() / 2];
        return check_device_error(ctx);
    };
    ddgi_trace_tuning best = start;
    float best_t = 0.0f;
    ddgi_status err = measure(best, &best_t);
    const uint32_t R = ctx->grid.rays_per_probe;
    const uint32_t width_c[] = {8u, 2u};
    const uint32_t rpw_c[] = {0u, 32u, 16u, 8u, 4u, 2u, 1u};
    const uint32_t refill_c[] = {4u, 8u, 16u, 24u};
    const uint32_t split_c[] = {0u, 32u, 24u, 16u};
    const uint32_t ctas_c[] = {0u, 6u, 4u};
    const uint32_t wait_c[] = {6u, 8u, 10u, 12u, 14u};
    for (int p = 0; p < 6 && err == DDGI_OK; ++p) {
        const uint32_t* cand = p == 0   ? width_c
                               : p == 1 ? wait_c
                               : p == 2 ? rpw_c
                               : p == 3 ? refill_c
                               : p == 4 ? split_c
                                        : ctas_c;
        const int nc = p == 0 ? 2 : p == 1 ? 5 : p == 2 ? 7 : p == 5 ? 3 : 4;
        for (int i = 0; i < nc && err == DDGI_OK; ++i) {
            ddgi_trace_tuning t = best;
            uint32_t* field = p == 0   ? &t.node_width
                              : p == 1 ? &t.straggler_lanes
                              : p == 2 ? &t.rays_per_warp
                              : p == 3 ? &t.refill_lanes
                              : p == 4 ? &t.smem_stack
                                       : &t.ctas_per_sm;
            if (*field == cand[i]) continue;
            if (p == 2 && grouped_rays_per_warp(cand[i], R) != cand[i]) continue;
            const int cap = t.node_width == 8 && ctx->scene.wstack_cap > 0 ? ctx->scene.wstack_cap : ctx->scene.stack_cap;
            if (p == 4 && cand[i] != 0 && (int)cand[i] >= cap) continue;
            *field = cand[i];
            float tt = 0.0f;
            err = measure(t, &tt);
            if (err == DDGI_OK && tt < best_t) {
                best_t = tt;
                best = t;
            }
        }
    }
    for (auto& x : saved) cudaMemcpyAsync(x.dst, x.copy, x.bytes, cudaMemcpyDeviceToDevice, st);
    cudaError_t e = cudaStreamSynchronize(st);
    release();
    ctx->ramp_cmd = ramp_cmd;
    ctx->timing = timing;
    ctx->tune = err == DDGI_OK ? best : start;
    if (err != DDGI_OK) return err;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "autotune restore");
    if (chosen) *chosen = best;
    return DDGI_OK;
}

ddgi_status ddgi_count_fetches(ddgi_ctx* ctx, const float orientation[9], const uint32_t* probe_list,
                               uint32_t probe_count, uint64_t out[11], ddgi_stream stream) {
    if (!ctx || !orientation || !out) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t* dlist = nullptr;
    uint32_t n = 0;
    ddgi_status s = prepare_update(ctx, orientation, probe_list, probe_count, st, &dlist, &n);
    if (s != DDGI_OK) return s;
    unsigned long long* dc = nullptr;
    CK(cudaMalloc(&dc, 11 * sizeof(unsigned long long)), "alloc counters");
    cudaError_t e = cudaMemsetAsync(dc, 0, 11 * sizeof(unsigned long long), st);
    if (e == cudaSuccess)
        e = launch_trace_shade(device_scene(ctx), ctx->dg, ctx->dl, dlist, n, ctx->dirs, ctx->ray_order, ctx->states,
                               ctx->color, ctx->depth, ctx->fp16, ctx->rays, nullptr, ctx->err, st, dc);
    unsigned long long h[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, dc, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dc);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "count fetches");
    for (int k = 0; k < 11; ++k) out[k] = h[k];
    ctx->last_count = n;
    ctx->last_rays = ctx->grid.rays_per_probe;
    return check_device_error(ctx);
}

ddgi_status ddgi_get_timings(const ddgi_ctx* cctx, ddgi_timings* out) {
    ddgi_ctx* ctx = const_cast<ddgi_ctx*>(cctx);
    if (!ctx || !out) return DDGI_ERR_INVALID_ARGUMENT;
    if (ctx->timing_pending) {
        CK(cudaEventSynchronize(ctx->ev[2]), "timing");
        float a = 0, b = 0, p = 0;
        cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
        cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&p, ctx->ev[0], ctx->ev[3]);
        ctx->timings.primary_ms = p;
        ctx->timings.trace_ms = a;
        ctx->timings.blend_ms = b;
        ctx->timings.border_ms = 0.0f;  // fused into the blend
        ctx->timings.copy_ms = 0.0f;    // atlas updated in place
        ctx->timings.total_ms = a + b;
        ctx->timing_pending = false;
    }
    *out = ctx->timings;
    return DDGI_OK;
}

ddgi_status ddgi_synchronize(ddgi_ctx* ctx, ddgi_stream stream, int timeout_ms) {
    if (!ctx) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return cuda_fail(ctx, e, "stream");
        if (timeout_ms >= 0) {
            auto el = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            if (el >= timeout_ms) return fail(ctx, DDGI_ERR_TIMEOUT, "stream not idle after %d ms", timeout_ms);
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return check_device_error(ctx);
}

ddgi_status ddgi_atlas_dims(const ddgi_ctx* ctx, ddgi_atlas_kind kind, uint32_t* w, uint32_t* h, uint32_t* ch) {
    if (!ctx || (kind != DDGI_ATLAS_COLOR && kind != DDGI_ATLAS_DEPTH)) return DDGI_ERR_INVALID_ARGUMENT;
    if (w) *w = kind == DDGI_ATLAS_COLOR ? ctx->dg.color_w : ctx->dg.depth_w;
    if (h) *h = kind == DDGI_ATLAS_COLOR ? ctx->dg.color_h : ctx->dg.depth_h;
    if (ch) *ch = kind == DDGI_ATLAS_COLOR ? 4u : 2u;
    return DDGI_OK;
}

namespace {

__global__ void k_half_to_float(const __half* __restrict__ in, float* __restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __half2float(in[i]);
}

}  // namespace

ddgi_status ddgi_get_atlas(ddgi_ctx* ctx, ddgi_atlas_kind kind, float* dst, size_t bytes, ddgi_stream stream) {
    if (!ctx || !dst || (kind != DDGI_ATLAS_COLOR && kind != DDGI_ATLAS_DEPTH)) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    uint32_t w, h, ch;
    ddgi_atlas_dims(ctx, kind, &w, &h, &ch);
    size_t count = (size_t)w * h * ch;
    if (bytes != count * sizeof(float)) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "atlas needs %zu bytes", count * 4);
    void* src = kind == DDGI_ATLAS_COLOR ? ctx->color : ctx->depth;
    if (!ctx->fp16) {
        CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st), "atlas download");
        CK(cudaStreamSynchronize(st), "atlas download");
    } else {
        // widen on the device, then one copy into the caller's buffer
        if (ctx->xfer_cap < count) {
            dfree(ctx->xfer);
            ctx->xfer_cap = 0;
            CK(cudaMalloc(&ctx->xfer, count * sizeof(float)), "alloc atlas staging");
            ctx->xfer_cap = count;
        }
        k_half_to_float<<<1216, 256, 0, st>>>(static_cast<const __half*>(src), ctx->xfer, count);
        CK(cudaGetLastError(), "atlas widen");
        CK(cudaMemcpyAsync(dst, ctx->xfer, bytes, cudaMemcpyDeviceToHost, st), "atlas download");
        CK(cudaStreamSynchronize(st), "atlas download");
    }
    return check_device_error(ctx);
}

ddgi_status ddgi_get_atlas_raw(ddgi_ctx* ctx, ddgi_atlas_kind kind, void* dst, size_t bytes, ddgi_stream stream) {
    if (!ctx || !dst || (kind != DDGI_ATLAS_COLOR && kind != DDGI_ATLAS_DEPTH)) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t need = atlas_bytes(ctx->dg, kind, ctx->fp16);
    if (bytes != need) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "atlas needs %zu bytes", need);
    CK(cudaMemcpyAsync(dst, kind == DDGI_ATLAS_COLOR ? ctx->color : ctx->depth, bytes, cudaMemcpyDeviceToHost, st),
       "atlas download");
    CK(cudaStreamSynchronize(st), "atlas download");
    return check_device_error(ctx);
}

ddgi_status ddgi_set_atlas(ddgi_ctx* ctx, ddgi_atlas_kind kind, const float* src, size_t bytes, ddgi_stream stream) {
    if (!ctx || !src || (kind != DDGI_ATLAS_COLOR && kind != DDGI_ATLAS_DEPTH)) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    uint32_t w, h, ch;
    ddgi_atlas_dims(ctx, kind, &w, &h, &ch);
    size_t count = (size_t)w * h * ch;
    if (bytes != count * sizeof(float)) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "atlas needs %zu bytes", count * 4);
    void* dstp = kind == DDGI_ATLAS_COLOR ? ctx->color : ctx->depth;
    if (!ctx->fp16) {
        CK(cudaMemcpyAsync(dstp, src, bytes, cudaMemcpyHostToDevice, st), "atlas upload");
        CK(cudaStreamSynchronize(st), "atlas upload");
    } else {
        std::vector<__half> tmp(count);
        for (size_t i = 0; i < count; ++i) tmp[i] = __float2half(src[i]);
        CK(cudaMemcpyAsync(dstp, tmp.data(), count * sizeof(__half), cudaMemcpyHostToDevice, st), "atlas upload");
        // the FP32 hysteresis accumulator takes the values as given
        void* acc = kind == DDGI_ATLAS_COLOR ? (void*)ctx->acc_color : (void*)ctx->acc_depth;
        CK(cudaMemcpyAsync(acc, src, bytes, cudaMemcpyHostToDevice, st), "atlas upload");
        CK(cudaStreamSynchronize(st), "atlas upload");
    }
    return DDGI_OK;
}

namespace {

struct AtlasFileHeader {
    char magic[8];
    uint32_t version, fp16;
    ddgi_grid_desc grid;
    uint32_t color_w, color_h, depth_w, depth_h, probes;
    uint32_t reserved[3];
};
static_assert(sizeof(AtlasFileHeader) == 112, "checkpoint header is 112 bytes");
constexpr char kAtlasMagic[8] = {'D', 'D', 'G', 'I', 'A', 'T', 'L', '1'};

struct FileCloser {
    FILE* f;
    ~FileCloser() {
        if (f) fclose(f);
    }
};

// The device buffers of a checkpoint in file order, with their sizes.
std::vector<std::pair<void*, size_t>> checkpoint_parts(ddgi_ctx* ctx) {
    std::vector<std::pair<void*, size_t>> parts = {
        {ctx->color, atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, ctx->fp16)},
        {ctx->depth, atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, ctx->fp16)}};
    if (ctx->fp16) {
        parts.push_back({ctx->acc_color, atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, false)});
        parts.push_back({ctx->acc_depth, atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, false)});
    }
    parts.push_back({ctx->states, sizeof(uint32_t) * (size_t)probe_count_of(ctx->grid)});
    return parts;
}

AtlasFileHeader checkpoint_header(const ddgi_ctx* ctx) {
    AtlasFileHeader h{};
    std::memcpy(h.magic, kAtlasMagic, 8);
    h.version = 1;
    h.fp16 = ctx->fp16 ? 1u : 0u;
    h.grid = ctx->grid;
    uint32_t ch;
    ddgi_atlas_dims(ctx, DDGI_ATLAS_COLOR, &h.color_w, &h.color_h, &ch);
    ddgi_atlas_dims(ctx, DDGI_ATLAS_DEPTH, &h.depth_w, &h.depth_h, &ch);
    h.probes = probe_count_of(ctx->grid);
    return h;
}

}  // namespace

ddgi_status ddgi_atlas_save(ddgi_ctx* ctx, const char* path, ddgi_stream stream) {
    if (!ctx || !path) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaStreamSynchronize(st), "checkpoint");
    ddgi_status s = check_device_error(ctx);
    if (s != DDGI_OK) return s;
    const AtlasFileHeader h = checkpoint_header(ctx);
    FileCloser fc{fopen(path, "wb")};
    if (!fc.f) return fail(ctx, DDGI_ERR_IO, "cannot open %s for writing", path);
    if (fwrite(&h, sizeof(h), 1, fc.f) != 1) return fail(ctx, DDGI_ERR_IO, "write failed: %s", path);
    std::vector<uint8_t> buf;
    for (const auto& part : checkpoint_parts(ctx)) {
        buf.resize(part.second);
        CK(cudaMemcpy(buf.data(), part.first, part.second, cudaMemcpyDeviceToHost), "checkpoint read");
        if (fwrite(buf.data(), 1, part.second, fc.f) != part.second)
            return fail(ctx, DDGI_ERR_IO, "write failed: %s", path);
    }
    if (fflush(fc.f) != 0) return fail(ctx, DDGI_ERR_IO, "write failed: %s", path);
    return DDGI_OK;
}

ddgi_status ddgi_atlas_load(ddgi_ctx* ctx, const char* path, ddgi_stream stream) {
    if (!ctx || !path) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    FileCloser fc{fopen(path, "rb")};
    if (!fc.f) return fail(ctx, DDGI_ERR_IO, "cannot open %s", path);
    AtlasFileHeader h{};
    if (fread(&h, sizeof(h), 1, fc.f) != 1 || std::memcmp(h.magic, kAtlasMagic, 8) != 0 || h.version != 1)
        return fail(ctx, DDGI_ERR_IO, "%s is not an atlas checkpoint", path);
    const AtlasFileHeader mine = checkpoint_header(ctx);
    if (h.fp16 != mine.fp16 || h.color_w != mine.color_w || h.color_h != mine.color_h ||
        h.depth_w != mine.depth_w || h.depth_h != mine.depth_h || h.probes != mine.probes ||
        h.grid.color_res != mine.grid.color_res || h.grid.depth_res != mine.grid.depth_res ||
        std::memcmp(h.grid.resolution, mine.grid.resolution, sizeof(h.grid.resolution)) != 0)
        return fail(ctx, DDGI_ERR_IO, "%s: grid or precision differs from the context's", path);
    // read everything before changing anything
    const auto parts = checkpoint_parts(ctx);
    std::vector<std::vector<uint8_t>> data(parts.size());
    for (size_t i = 0; i < parts.size(); ++i) {
        data[i].resize(parts[i].second);
        if (fread(data[i].data(), 1, parts[i].second, fc.f) != parts[i].second)
            return fail(ctx, DDGI_ERR_IO, "%s is truncated", path);
    }
    if (fgetc(fc.f) != EOF) return fail(ctx, DDGI_ERR_IO, "%s has trailing data", path);
    CK(cudaStreamSynchronize(st), "checkpoint");
    for (size_t i = 0; i < parts.size(); ++i)
        CK(cudaMemcpy(parts[i].first, data[i].data(), parts[i].second, cudaMemcpyHostToDevice), "checkpoint write");
    return DDGI_OK;
}

ddgi_status ddgi_atlas_device_ptr(const ddgi_ctx* ctx, ddgi_atlas_kind kind, void** ptr) {
    if (!ctx || !ptr || (kind != DDGI_ATLAS_COLOR && kind != DDGI_ATLAS_DEPTH)) return DDGI_ERR_INVALID_ARGUMENT;
    *ptr = kind == DDGI_ATLAS_COLOR ? ctx->color : ctx->depth;
    return DDGI_OK;
}

ddgi_status ddgi_get_ray_records(ddgi_ctx* ctx, float* dst, size_t count, ddgi_stream stream) {
    if (!ctx || !dst) return DDGI_ERR_INVALID_ARGUMENT;
    size_t n = (size_t)ctx->last_count * ctx->last_rays;
    if (count != n) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "expected %zu ray records", n);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaMemcpyAsync(dst, ctx->rays, n * sizeof(float4), cudaMemcpyDeviceToHost, st), "ray download");
    CK(cudaStreamSynchronize(st), "ray download");
    return check_device_error(ctx);
}

ddgi_status ddgi_get_hits(ddgi_ctx* ctx, ddgi_hit* dst, size_t count, ddgi_stream stream) {
    if (!ctx || !dst) return DDGI_ERR_INVALID_ARGUMENT;
    if (!ctx->record_hits || !ctx->hits) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "hit recording is off");
    size_t n = (size_t)ctx->last_count * ctx->last_rays;
    if (count != n) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "expected %zu hit records", n);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaMemcpyAsync(dst, ctx->hits, n * sizeof(ddgi_hit), cudaMemcpyDeviceToHost, st), "hit download");
    CK(cudaStreamSynchronize(st), "hit download");
    return check_device_error(ctx);
}

ddgi_status ddgi_get_ray_directions(ddgi_ctx* ctx, float* dst, size_t count) {
    if (!ctx || !dst) return DDGI_ERR_INVALID_ARGUMENT;
    if (count != ctx->host_dirs.size() / 4)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "expected %zu directions", ctx->host_dirs.size() / 4);
    std::memcpy(dst, ctx->host_dirs.data(), ctx->host_dirs.size() * sizeof(float));
    return DDGI_OK;
}

ddgi_status ddgi_get_probe_states(ddgi_ctx* ctx, uint32_t* dst, size_t count, ddgi_stream stream) {
    if (!ctx || !dst || count != probe_count_of(ctx->grid)) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaMemcpyAsync(dst, ctx->states, count * sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "state download");
    CK(cudaStreamSynchronize(st), "state download");
    return DDGI_OK;
}

ddgi_status ddgi_set_probe_states(ddgi_ctx* ctx, const uint32_t* src, size_t count, ddgi_stream stream) {
    if (!ctx || !src || count != probe_count_of(ctx->grid)) return DDGI_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < count; ++i)
        if (src[i] > 8) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "probe state %u > 8", src[i]);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    CK(cudaMemcpyAsync(ctx->states, src, count * sizeof(uint32_t), cudaMemcpyHostToDevice, st), "state upload");
    CK(cudaStreamSynchronize(st), "state upload");
    return DDGI_OK;
}

ddgi_status ddgi_trace_rays(ddgi_ctx* ctx, const float* origins, const float* dirs, uint32_t n, float tmin, float tmax,
                            uint32_t mask, int any_hit, ddgi_hit* hits, float* barycentrics, ddgi_stream stream) {
    if (!ctx || (n && (!origins || !dirs || !hits))) return DDGI_ERR_INVALID_ARGUMENT;
    if (!ctx->scene.built) return fail(ctx, DDGI_ERR_NO_SCENE, "no scene");
    if (n == 0) return DDGI_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    float *dor = nullptr, *ddir = nullptr, *dbar = nullptr;
    ddgi_hit* dh = nullptr;
    auto cleanup = [&]() {
        if (dor) cudaFree(dor);
        if (ddir) cudaFree(ddir);
        if (dbar) cudaFree(dbar);
        if (dh) cudaFree(dh);
    };
    cudaError_t e = cudaMalloc(&dor, sizeof(float) * 3 * n);
    if (e == cudaSuccess) e = cudaMalloc(&ddir, sizeof(float) * 3 * n);
    if (e == cudaSuccess) e = cudaMalloc(&dh, sizeof(ddgi_hit) * n);
    if (e == cudaSuccess && barycentrics) e = cudaMalloc(&dbar, sizeof(float) * 2 * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dor, origins, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ddir, dirs, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = launch_trace_rays(device_scene(ctx), dor, ddir, n, tmin, tmax, mask, any_hit, dh, dbar, ctx->err, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hits, dh, sizeof(ddgi_hit) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && barycentrics)
        e = cudaMemcpyAsync(barycentrics, dbar, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "trace rays");
    return check_device_error(ctx);
}

ddgi_status ddgi_set_materials(ddgi_ctx* ctx, const ddgi_material* materials, uint32_t count) {
    if (!ctx || (count && !materials)) return DDGI_ERR_INVALID_ARGUMENT;
    if (!ctx->scene.built) return fail(ctx, DDGI_ERR_NO_SCENE, "no scene");
    if (count != ctx->scene.material_count)
        return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "expected %u materials", ctx->scene.material_count);
    for (uint32_t m = 0; m < count; ++m)
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(materials[m].base_color[k]) || !std::isfinite(materials[m].emissive[k]))
                return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "material %u not finite", m);
    CK(cudaMemcpy(ctx->scene.materials, materials, sizeof(ddgi_material) * count, cudaMemcpyHostToDevice),
       "upload materials");
    return DDGI_OK;
}

namespace {

ddgi_status ensure_rec_buffers(ddgi_ctx* ctx, uint32_t K, uint32_t ncheck) {
    const size_t rays = (size_t)probe_count_of(ctx->grid) * ctx->grid.rays_per_probe;
    if (rays != ctx->rec_cap || K > ctx->rec_updates_cap) {
        dfree(ctx->rec_thit);
        dfree(ctx->rec_prim);
        dfree(ctx->g_x);
        ctx->rec_cap = 0;
        ctx->rec_updates_cap = 0;
        CK(cudaMalloc(&ctx->rec_thit, rays * K * sizeof(float4)), "alloc hit record");
        CK(cudaMalloc(&ctx->rec_prim, rays * K * sizeof(uint32_t)), "alloc hit record");
        CK(cudaMalloc(&ctx->g_x, rays * sizeof(float4)), "alloc ray gradients");
        ctx->rec_cap = rays;
        ctx->rec_updates_cap = K;
    }
    const size_t cb = atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, false), db = atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, false);
    if (ncheck > ctx->ckpt_cap) {
        dfree(ctx->ckpt_color);
        dfree(ctx->ckpt_depth);
        ctx->ckpt_cap = 0;
        CK(cudaMalloc(&ctx->ckpt_color, cb * ncheck), "alloc checkpoints");
        CK(cudaMalloc(&ctx->ckpt_depth, db * ncheck), "alloc checkpoints");
        ctx->ckpt_cap = ncheck;
    }
    const uint32_t P = probe_count_of(ctx->grid);
    if (!ctx->rec_states) {
        CK(cudaMalloc(&ctx->rec_states, sizeof(uint32_t) * P), "alloc states");
        CK(cudaMalloc(&ctx->work_states, sizeof(uint32_t) * P), "alloc states");
        CK(cudaMalloc(&ctx->work_color, cb), "alloc work atlas");
        CK(cudaMalloc(&ctx->work_depth, db), "alloc work atlas");
        CK(cudaMalloc(&ctx->g_a, cb), "alloc atlas gradients");
        CK(cudaMalloc(&ctx->g_b, cb), "alloc atlas gradients");
    }
    const uint32_t ng = ctx->scene.material_count * 3 + 6;
    if (ng > ctx->grad_cap) {
        dfree(ctx->d_grad);
        ctx->grad_cap = 0;
        CK(cudaMalloc(&ctx->d_grad, sizeof(double) * ng), "alloc gradients");
        ctx->grad_cap = ng;
    }
    return DDGI_OK;
}

ddgi_status upload_dirs(ddgi_ctx* ctx, const float* orientation, cudaStream_t st) {
    const uint32_t R = ctx->grid.rays_per_probe;
    ctx->host_dirs.resize(4 * (size_t)R);
    ddgi_ray_direction_table(orientation, R, ctx->host_dirs.data());
    CK(cudaMemcpyAsync(ctx->dirs, ctx->host_dirs.data(), sizeof(float4) * R, cudaMemcpyHostToDevice, st),
       "upload dirs");
    return DDGI_OK;
}

}  // namespace

ddgi_status ddgi_forward_record(ddgi_ctx* ctx, uint32_t K, const float* orientations, uint32_t checkpoint_every,
                                ddgi_stream stream) {
    ddgi::NvtxRange nvtx_range("ddgi_forward_record");
    if (!ctx || !orientations || K == 0 || checkpoint_every == 0) return DDGI_ERR_INVALID_ARGUMENT;
    if (ctx->fp16 || ctx->dg.quant)
        return fail(ctx, DDGI_ERR_UNSUPPORTED, "gradients need the FP32 form (unrounded atlas)");
    if (ctx->dl.sky_mode != DDGI_SKY_CONSTANT)
        return fail(ctx, DDGI_ERR_UNSUPPORTED, "gradients need the constant sky (a parameter)");
    // the adjoint differentiates the blend with the grid's hysteresis
    if (ctx->ramp_on)
        return fail(ctx, DDGI_ERR_UNSUPPORTED, "gradients need a fixed hysteresis (no ddgi_set_target_hysteresis ramp)");
    if (!ctx->scene.built) return fail(ctx, DDGI_ERR_NO_SCENE, "no scene");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t C = checkpoint_every, ncheck = (K + C - 1) / C;
    ddgi_status s = ensure_rec_buffers(ctx, K, ncheck);
    if (s != DDGI_OK) return s;
    const uint32_t P = probe_count_of(ctx->grid);
    const size_t rays = (size_t)P * ctx->grid.rays_per_probe;
    const size_t cb = atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, false), db = atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, false);
    CK(cudaMemcpyAsync(ctx->rec_states, ctx->states, sizeof(uint32_t) * P, cudaMemcpyDeviceToDevice, st), "states");
    const ddgi_pipeline saved = ctx->pipeline;
    ctx->pipeline = DDGI_PIPELINE_WAVEFRONT;  // the wavefront form keeps the hit buffer and shadow flags
    for (uint32_t k = 0; k < K; ++k) {
        if (k % C == 0) {
            CK(cudaMemcpyAsync((char*)ctx->ckpt_color + cb * (k / C), ctx->color, cb, cudaMemcpyDeviceToDevice, st),
               "checkpoint");
            CK(cudaMemcpyAsync((char*)ctx->ckpt_depth + db * (k / C), ctx->depth, db, cudaMemcpyDeviceToDevice, st),
               "checkpoint");
        }
        s = ddgi_update(ctx, orientations + 9 * (size_t)k, nullptr, 0, stream);
        if (s != DDGI_OK) {
            ctx->pipeline = saved;
            return s;
        }
        CK(cudaMemcpyAsync(ctx->rec_thit + rays * k, ctx->wave_thit, rays * sizeof(float4), cudaMemcpyDeviceToDevice,
                           st),
           "record hits");
        CK(cudaMemcpyAsync(ctx->rec_prim + rays * k, ctx->wave_prim, rays * sizeof(uint32_t),
                           cudaMemcpyDeviceToDevice, st),
           "record hits");
    }
    ctx->pipeline = saved;
    ctx->rec_K = K;
    ctx->rec_C = C;
    ctx->rec_orient.assign(orientations, orientations + 9 * (size_t)K);
    return DDGI_OK;
}

ddgi_status ddgi_backward(ddgi_ctx* ctx, const float* dL_dcolor, size_t bytes, float* grad_albedo, float grad_sun[3],
                          float grad_sky[3], ddgi_stream stream) {
    ddgi::NvtxRange nvtx_range("ddgi_backward");
    if (!ctx || !dL_dcolor || !grad_albedo || !grad_sun || !grad_sky) return DDGI_ERR_INVALID_ARGUMENT;
    if (ctx->rec_K == 0) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "ddgi_backward without ddgi_forward_record");
    const size_t cb = atlas_bytes(ctx->dg, DDGI_ATLAS_COLOR, false), db = atlas_bytes(ctx->dg, DDGI_ATLAS_DEPTH, false);
    if (bytes != cb) return fail(ctx, DDGI_ERR_INVALID_ARGUMENT, "gradient needs %zu bytes", cb);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t P = probe_count_of(ctx->grid), M = ctx->scene.material_count;
    const size_t rays = (size_t)P * ctx->grid.rays_per_probe;
    const uint32_t K = ctx->rec_K, C = ctx->rec_C;
    DeviceScene sc = device_scene(ctx);
    CK(cudaMemcpyAsync(ctx->g_a, dL_dcolor, cb, cudaMemcpyHostToDevice, st), "upload gradient");
    CK(cudaMemsetAsync(ctx->d_grad, 0, sizeof(double) * (M * 3 + 6), st), "zero gradients");
    for (uint32_t u = K; u-- > 0;) {
        // atlas before update u: checkpoint, then replay the updates after it
        const uint32_t c0 = (u / C) * C;
        CK(cudaMemcpyAsync(ctx->work_color, (char*)ctx->ckpt_color + cb * (u / C), cb, cudaMemcpyDeviceToDevice, st),
           "restore");
        CK(cudaMemcpyAsync(ctx->work_depth, (char*)ctx->ckpt_depth + db * (u / C), db, cudaMemcpyDeviceToDevice, st),
           "restore");
        CK(cudaMemcpyAsync(ctx->work_states, ctx->rec_states, sizeof(uint32_t) * P, cudaMemcpyDeviceToDevice, st),
           "restore");
        for (uint32_t v = c0; v < u; ++v) {
            ddgi_status s = upload_dirs(ctx, &ctx->rec_orient[9 * (size_t)v], st);
            if (s != DDGI_OK) return s;
            CK(launch_replay_update(sc, ctx->dg, ctx->dl, ctx->dirs, ctx->work_states, ctx->work_color, ctx->work_depth,
                                    ctx->rec_thit + rays * v, ctx->rec_prim + rays * v, ctx->rays, ctx->err, st),
               "replay");
        }
        CK(cudaMemcpyAsync(ctx->work_states, ctx->rec_states, sizeof(uint32_t) * P, cudaMemcpyDeviceToDevice, st),
           "restore");
        ddgi_status s = upload_dirs(ctx, &ctx->rec_orient[9 * (size_t)u], st);
        if (s != DDGI_OK) return s;
        CK(launch_adjoint_step(sc, ctx->dg, ctx->dl, ctx->dirs, ctx->work_states, ctx->work_color, ctx->work_depth,
                               ctx->rec_thit + rays * u, ctx->rec_prim + rays * u, ctx->g_a, ctx->g_b, ctx->g_x,
                               ctx->d_grad, ctx->err, st),
           "adjoint");
        std::swap(ctx->g_a, ctx->g_b);
    }
    std::vector<double> h(M * 3 + 6);
    CK(cudaMemcpyAsync(h.data(), ctx->d_grad, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st), "gradients");
    CK(cudaStreamSynchronize(st), "backward");
    for (uint32_t i = 0; i < M * 3; ++i) grad_albedo[i] = (float)h[i];
    for (int k = 0; k < 3; ++k) {
        grad_sun[k] = (float)h[M * 3 + k];
        grad_sky[k] = (float)h[M * 3 + 3 + k];
    }
    return check_device_error(ctx);
}

}  // extern "C"

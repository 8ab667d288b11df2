// ctx.h — the context behind the opaque ddgi_ctx handle (internal; shared
// by the translation units that implement the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/ddgi.h"
#include "common.cuh"
#include "kernels.h"

namespace ddgi {

constexpr int kBlasLeafMax = 2;  // default; measured best of 1, 2, 4, 8 on the 1M-triangle scene
constexpr int kTlasLeafMax = 1;
// Overlap (of the root's surface area) above which a fast-trace mesh-tree
// node tries a spatial split.  On the 1M-triangle terrain + box-cluster
// scene (update / scene build on 16 Arm cores): 0 -> 13.8 ms / 0.18 s,
// 0.01 -> 10.7 ms / 1.1 s, 0.003 -> 9.74 ms / 1.3 s, 0.001 -> 9.36 ms /
// 2.3 s, 0.0003 -> 9.30 ms / 3.8 s.
constexpr float kDefaultSplitAlpha = 1e-3f;
// deepest traversal stack of the wavefront kernels (entries per thread in
// shared memory: 96 x 128 threads x 4 bytes = 48 KB per block)
constexpr int kMaxStack = 96;

struct SceneBuffers {
    BvhNode* nodes = nullptr;
    BvhTri* tris = nullptr;
    GpuInstance* inst_leaf = nullptr;
    GpuInstance* inst_id = nullptr;
    float4* normals = nullptr;
    uint32_t* indices = nullptr;
    ddgi_offset_entry* offsets = nullptr;
    ddgi_material* materials = nullptr;
    int32_t tlas_root = -1;
    int stack_cap = 0;
    uint32_t depth_blas = 0, depth_tlas = 0;
    uint32_t vertex_count = 0, index_count = 0, offset_count = 0, material_count = 0, instance_count = 0;
    uint64_t node_count = 0, tri_count = 0;
    uint64_t build_id = 0;  // distinct for every successful build or instance update in the process
    ddgi_build_mode build_mode = DDGI_BUILD_FAST_BUILD;  // builder of these trees
    float gpu_build_ms = 0.0f;  // device time of the GPU fast-trace mesh-tree build
    bool built = false;
    // top level, kept for instance updates (refit / rebuild)
    std::vector<GpuInstance> host_inst;      // caller order
    std::vector<float> mesh_lo, mesh_hi;     // object-space bounds, 3 per mesh
    std::vector<uint32_t> mesh_of_inst;
    std::vector<float4> inst_lo, inst_hi;    // world boxes, caller order
    std::vector<uint32_t> leaf_of_id;        // leaf slot of each instance
    float4* leaf_lo = nullptr;               // world boxes in leaf order (device)
    float4* leaf_hi = nullptr;
    uint32_t* leaf_parent = nullptr;         // parent links of the top level (node << 1 | side)
    uint32_t* node_parent = nullptr;
    uint32_t* refit_flags = nullptr;
    float4* sub_lo = nullptr;
    float4* sub_hi = nullptr;
    // eight-wide copy of the trees: [mesh trees | top level, with room for
    // a rebuilt top level]; instances in leaf order with wide mesh roots
    WideNode* wnodes = nullptr;
    GpuInstance* winst_leaf = nullptr;
    uint32_t wnode_count = 0, wide_tlas_start = 0, wide_cap = 0, wlevels_blas = 0;
    int32_t wtlas_root = -1;
    int wstack_cap = 0;  // 0: no wide trees (too deep for the stack)
    std::vector<int32_t> wide_root_of_mesh;
    std::vector<int32_t> mesh_root;  // root node of each mesh tree (-1: empty mesh)
    bool wide_ready = false;         // the wide copies exist (made on first use)
};

}  // namespace ddgi

struct ddgi_ctx {
    ddgi_grid_desc grid{};
    ddgi::DeviceGrid dg{};
    ddgi::DeviceLight dl{};
    int device = 0;
    bool fp16 = false;
    void* color = nullptr;
    void* depth = nullptr;
    uint32_t* states = nullptr;
    float4* rays = nullptr;
    size_t rays_cap = 0;  // in records
    // wavefront pipeline: hit buffer, shadow-ray queue, work counters
    float4* wave_thit = nullptr;
    uint32_t* wave_prim = nullptr;
    uint32_t* wave_front = nullptr;  // compacted front-face hits
    float* xfer = nullptr;           // FP32 staging of an FP16 atlas being read back
    size_t xfer_cap = 0;             // in floats
    uint32_t* q_idx = nullptr;
    float4* q_pos = nullptr;
    float4* q_sun = nullptr;
    uint32_t* counters = nullptr;
    ddgi_pipeline pipeline = DDGI_PIPELINE_WAVEFRONT;
    // BF16 tensor-core blend: per-update weight matrices and their row sums
    uint8_t* tc_weights = nullptr;
    float* tc_rowsum = nullptr;
    // BF16 form: FP32 hysteresis accumulators behind the FP16 atlas
    float4* acc_color = nullptr;
    float2* acc_depth = nullptr;
    // differentiation: recorded hits of K updates, atlas checkpoints, and the
    // reverse-pass buffers
    uint32_t rec_K = 0, rec_C = 0;
    size_t rec_cap = 0;  // rays per update the record buffers hold
    uint32_t rec_updates_cap = 0;
    std::vector<float> rec_orient;
    float4* rec_thit = nullptr;
    uint32_t* rec_prim = nullptr;
    float4* ckpt_color = nullptr;
    float2* ckpt_depth = nullptr;
    uint32_t ckpt_cap = 0;
    uint32_t* rec_states = nullptr;
    uint32_t* work_states = nullptr;
    float4* work_color = nullptr;
    float2* work_depth = nullptr;
    float4* g_a = nullptr;
    float4* g_b = nullptr;
    float4* g_x = nullptr;
    double* d_grad = nullptr;
    uint32_t grad_cap = 0;
    ddgi_hit* hits = nullptr;
    size_t hits_cap = 0;
    bool record_hits = false;
    float4* dirs = nullptr;
    uint32_t* ray_order = nullptr;
    uint32_t* probe_list = nullptr;
    // adaptive schedule (selectProbesToUpdate on the device): {offset, loop
    // index, selected count, -}, then the hysteresis ramp {blended value,
    // host-side value, target (float bits), probes counted}
    uint32_t* sched = nullptr;
    bool ramp_on = false;
    ddgi::RampCmd ramp_cmd{};  // host changes the next update's ramp step applies first
    // traversal launch tuning; probes in Morton order of the grid (grouped warps)
    ddgi_trace_tuning tune{0, 8, 0, 0, 2, ddgi::kDefaultWait};
    int blas_leaf_max = ddgi::kBlasLeafMax;  // triangles per mesh-tree leaf (scene build option)
    ddgi_build_mode build_mode = DDGI_BUILD_FAST_TRACE;  // tree builder (scene build option)
    float split_alpha = ddgi::kDefaultSplitAlpha;          // spatial splits of fast-trace mesh trees (0: none)
    uint32_t inject = 0;  // one-shot test hooks (DDGI_FAULT_*), cleared by the launch that uses them
    uint32_t* probe_perm = nullptr;
    float4* init_dirs = nullptr;
    uint32_t* init_back = nullptr;
    uint32_t* init_near = nullptr;
    uint32_t* err = nullptr;
    uint32_t last_count = 0;
    uint32_t last_rays = 0;
    std::vector<float> host_dirs;
    std::vector<uint32_t> host_order;
    ddgi::SceneBuffers scene;
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool timing_pending = false;
    ddgi_timings timings{};
    char msg[512] = "";
};


namespace ddgi {

// Ray order of one update: octant-binned (sign bits of x, y, z); within an
// octant by ray index (`fine` = false: the spherical-Fibonacci index, i.e.
// by elevation) or along a Morton curve over the octahedral map (`fine`:
// |x|, |y| of the direction scaled to |x| + |y| + |z| = 1, so that short
// runs are close directions, for warps that take a few rays per probe).
// Only the order in which rays are traced depends on it.
inline void ray_order_of(const float* dirs4, uint32_t R, uint32_t* order, bool fine) {
    std::vector<uint64_t> key(R);
    for (uint32_t r = 0; r < R; ++r) {
        const float* d = dirs4 + 4 * (size_t)r;
        uint32_t oct = (d[0] < 0.0f ? 1u : 0u) | (d[1] < 0.0f ? 2u : 0u) | (d[2] < 0.0f ? 4u : 0u);
        float s = std::fabs(d[0]) + std::fabs(d[1]) + std::fabs(d[2]);
        float u = s > 0.0f ? std::fabs(d[0]) / s : 0.0f, v = s > 0.0f ? std::fabs(d[1]) / s : 0.0f;
        uint32_t qu = (uint32_t)std::min(1023.0f, u * 1024.0f), qv = (uint32_t)std::min(1023.0f, v * 1024.0f);
        uint32_t m = 0;
        for (int b = 0; b < 10; ++b) m |= ((qu >> b) & 1u) << (2 * b) | ((qv >> b) & 1u) << (2 * b + 1);
        key[r] = ((uint64_t)oct << 40) | ((uint64_t)(fine ? m : 0u) << 12) | r;
    }
    std::sort(key.begin(), key.end());
    for (uint32_t r = 0; r < R; ++r) order[r] = (uint32_t)(key[r] & 0xFFFu);
}

// Probes of a grid sorted by the Morton code of (x, y, z).
inline std::vector<uint32_t> probe_morton_order(const int32_t res[3]) {
    const uint32_t P = (uint32_t)res[0] * (uint32_t)res[1] * (uint32_t)res[2];
    auto spread = [](uint64_t x) {
        uint64_t r = 0;
        for (int b = 0; b < 21; ++b) r |= ((x >> b) & 1ull) << (3 * b);
        return r;
    };
    std::vector<uint64_t> key(P);
    for (uint32_t p = 0; p < P; ++p) {
        uint32_t x = p % (uint32_t)res[0], y = (p / (uint32_t)res[0]) % (uint32_t)res[1];
        uint32_t z = p / ((uint32_t)res[0] * (uint32_t)res[1]);
        key[p] = spread(x) | spread(y) << 1 | spread(z) << 2;
    }
    std::vector<uint32_t> order(P);
    for (uint32_t p = 0; p < P; ++p) order[p] = p;
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
    return order;
}

// Traversal view of a context's scene buffers.
inline DeviceScene device_scene(const ddgi_ctx* c) {
    DeviceScene s{};
    s.nodes = c->scene.nodes;
    s.tris = c->scene.tris;
    s.instances = c->scene.inst_leaf;
    s.instances_by_id = c->scene.inst_id;
    s.normals = c->scene.normals;
    s.indices = c->scene.indices;
    s.offsets = c->scene.offsets;
    s.materials = c->scene.materials;
    s.tlas_root = c->scene.tlas_root;
    s.vertex_count = c->scene.vertex_count;
    s.index_count = c->scene.index_count;
    s.offset_count = c->scene.offset_count;
    s.material_count = c->scene.material_count;
    s.node_count = (uint32_t)c->scene.node_count;
    s.tri_count = (uint32_t)c->scene.tri_count;
    s.instance_count = c->scene.instance_count;
    s.wnodes = c->scene.wstack_cap > 0 ? c->scene.wnodes : nullptr;
    s.winstances = c->scene.wstack_cap > 0 ? c->scene.winst_leaf : nullptr;
    s.wtlas_root = c->scene.wtlas_root;
    s.wnode_count = c->scene.wnode_count;
    set_step_limits(s);
    return s;
}

// The eight-wide copies of the built scene's trees (ddgi_api.cu), made on
// first use: by a node_width 8 tuning, an autotune or a batch.
ddgi_status ensure_wide(ddgi_ctx* ctx);

}  // namespace ddgi

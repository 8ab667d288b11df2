// kernels.h — host-side launchers of the DDGI kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace ddgi {

// Raises a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device.  The limit belongs to the device's context, so it is read
// back on every call (a microsecond, no stream work) rather than remembered
// per process: a second GPU, or a context made again after a reset, starts
// from the default limit.
template <class K>
inline cudaError_t ensure_dynamic_smem(K* kernel, int bytes) {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    if (fa.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

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
    float4* thit;     // (t, b1, b2, instance bits) per ray
    uint32_t* prim;   // primitive | backface << 31
    uint32_t* front;  // compacted queue of front-face hits (record indices)
};
struct ShadowQueue {
    uint32_t* idx;   // ray record index
    float4* pos;     // shadow-ray origin (hit position)
    float4* sun;     // unshadowed sun term (xyz) and night fade (w)
    uint32_t* count;
};
// Launch shape of the persistent traversals.
struct TraceTuning {
    uint32_t ctas_per_sm;    // 0: occupancy limit
    uint32_t refill;         // idle lanes that trigger a warp's work request
    uint32_t split;          // stack entries in shared memory (0 or >= cap: all)
    uint32_t rays_per_warp;  // 0: a warp per probe in slot order; 1..32: grouped order (see below)
    uint32_t wide;           // 1: eight-wide quantised nodes (made on first use), 0: binary nodes
    uint32_t wait = kDefaultWait;  // straggler lanes that end a warp's search loop (0: wait for all)
};
// Per-launch constants of the persistent traversal loop.
struct WalkKnobs {
    int refill;     // idle lanes that trigger a warp's work request (1..32)
    uint32_t wait;  // lanes still searching for a first leaf that no longer hold the search loop (0..31)
};
inline WalkKnobs walk_knobs(const TraceTuning& t) {
    return WalkKnobs{(int)(t.refill < 1 ? 1 : (t.refill > 32 ? 32 : t.refill)), t.wait > 31 ? 31u : t.wait};
}
// Grouped order: lane groups of rays_per_warp consecutive directions (of the
// octant-binned ray order) from 32 / rays_per_warp probes taken in `perm`
// order (Morton order of the grid).  Usable values divide 32 and R (32
// always); anything else falls back to 0.
inline uint32_t grouped_rays_per_warp(uint32_t rpw, uint32_t R) {
    if (rpw == 32u) return 32u;
    return (rpw == 1 || rpw == 2 || rpw == 4 || rpw == 8 || rpw == 16) && R % rpw == 0 ? rpw : 0u;
}
// perm: probes in the order lane groups take them (all probes, no list), or
// NULL for a warp per probe in slot order.
cudaError_t launch_wavefront(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L,
                             const uint32_t* probe_list, uint32_t nprobes, const float4* dirs,
                             const uint32_t* ray_order, const uint32_t* states, const void* color, const void* depth,
                             bool fp16_atlas, WaveHits hits, ShadowQueue q, uint32_t* counters, float4* rays_out,
                             ddgi_hit* hits_out, int stack_cap, int wstack_cap, uint32_t* err, cudaStream_t st,
                             cudaEvent_t after_primary, const uint32_t* dev_count, const TraceTuning& tune,
                             const uint32_t* perm);
// Probe classification (probesInit): kInitRays rays per probe.
constexpr uint32_t kInitRays = 512;
cudaError_t launch_init_probes(const DeviceScene& sc, const DeviceGrid& g, const float4* dirs, uint32_t P,
                               uint32_t* back, uint32_t* near, uint32_t* states, uint32_t* counters, int stack_cap,
                               uint32_t* err, cudaStream_t st);
// schedule.cu: selectProbesToUpdate on the device.  sched = {offset, loop
// index, selected count} (kept on the device between updates); the selected
// probes go to list[0 .. count).
cudaError_t launch_select_probes(const uint32_t* states, uint32_t P, uint32_t max_probes, uint32_t* sched,
                                 uint32_t* list, cudaStream_t st);
// Hysteresis ramp of one update (sched[4..7]: blended value, host-side value,
// target, probes counted); `cmd` carries the host's changes since the last
// update; the update's probe count is *dev_count when given, else `count`.
constexpr uint32_t kRampSetBlended = 1, kRampSetParam = 2, kRampSetTarget = 4, kRampZeroCount = 8;
struct RampCmd {
    uint32_t set;
    float blended, param, target;
};
cudaError_t launch_hysteresis_ramp(uint32_t* sched, const RampCmd& cmd, const uint32_t* dev_count, uint32_t count,
                                   uint32_t P, cudaStream_t st);

// ---------------------------------------------------------------------------
// Batched update of many probe volumes (batch.cu drives these launchers)
// ---------------------------------------------------------------------------
constexpr uint32_t kMaxBatchVolumes = 1024;

// One volume of a batch.  `sc` points at the volume's own shading data;
// traversal runs over the batch arena, where the volume's trees start at
// `root`.  Ray records of the volume are [ray_base, ray_base + P * R) of the
// batch buffers; its direction table and ray order start at dir_base.
struct BatchVolume {
    DeviceScene sc;
    DeviceGrid g;
    DeviceLight L;
    int32_t root;
    uint32_t fp16;  // BF16 form: FP16 atlas + FP32 accumulators, tensor-core blend
    uint32_t ray_base, dir_base;
    uint32_t* states;
    void* color;
    void* depth;
    float4* acc_color;
    float2* acc_depth;
    uint8_t* wbuf;  // tensor-core weight chunks of this update (BF16 form)
    float* rowsum;
    const uint32_t* perm;  // probe order of grouped warps (NULL: a warp per probe)
    uint32_t rays_per_warp;
    int32_t wroot;  // top-level root among the arena's wide nodes (-1: empty)
};

struct BatchTables {
    const BatchVolume* vols;
    uint32_t nvol;
    const uint32_t* ray_base;  // nvol + 1 record offsets
    const float4* dirs;
    const uint32_t* ray_order;
    unsigned long long* clock;  // [0] batch start, [1 + v] blend completion of volume v (ns, globaltimer)
    uint32_t* done;             // blend work items finished, per volume
    uint32_t* err;
    uint32_t first;             // record of a launch's first work item (a group of volumes; 0: all)
};

// Volumes one blend kernel covers: list[i] is a volume index, its work items
// are [tile_base[i], tile_base[i + 1]).
struct BatchBlendList {
    const uint32_t* list;
    const uint32_t* tile_base;
    uint32_t n, ntiles;
};

// wavefront.cu: primary trace, shading and shadow rays of all volumes
cudaError_t launch_batch_trace(const DeviceScene& arena, const BatchTables& bt, uint32_t total, WaveHits hits,
                               ShadowQueue q, uint32_t* counters, float4* rays_out, int stack_cap, int wstack_cap,
                               const TraceTuning& tune, cudaStream_t st, cudaEvent_t after_primary,
                               cudaEvent_t after_shade);
// blend.cu
cudaError_t launch_batch_blend_fp32(const BatchTables& bt, const BatchBlendList& bl, uint32_t max_rays,
                                    const float4* rays, uint32_t threads, cudaStream_t st);
// blend_tc.cu
cudaError_t launch_batch_tc_weights(const BatchTables& bt, const BatchBlendList& bl, uint32_t max_rows,
                                    cudaStream_t st);
size_t batch_tc_smem(uint32_t color_res, uint32_t depth_res);
uint32_t tc_tiles(uint32_t nprobes);  // tensor-core blend work items of a volume
cudaError_t prepare_batch_kernels();  // kernel attributes, set once before any graph capture
cudaError_t launch_batch_blend_tc(const BatchTables& bt, const BatchBlendList& bl, const float4* rays, size_t smem,
                                  cudaStream_t st);

// gather.cu: the final-gather consumer over a device G-buffer
struct GatherArgs {
    const float4* position_depth;
    const float4* normal_metalness;
    const float4* albedo_roughness;
    const float4* emissive;
    const float* direct_light;
    const float4* reflection;  // may be NULL
    float4* out;
    uint32_t pixels;
    float3 origin;  // camera
    DeviceGrid g;
    DeviceLight L;
    const uint32_t* states;
};
cudaError_t launch_final_gather(const GatherArgs& a, const void* color, const void* depth, bool fp16_atlas,
                                cudaStream_t st);

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
                            void* depth, float4* acc_color, float2* acc_depth, uint32_t* err, cudaStream_t st,
                            const uint32_t* dev_count = nullptr, bool stall = false,
                            const float* hyst_dev = nullptr);

// blend_shared.cu: FP32 blend with the weights computed once per update
size_t fp32_weight_bytes(uint32_t rays, uint32_t color_res, uint32_t depth_res);
uint32_t fp32_shared_tiles(uint32_t nprobes);
cudaError_t set_shared_smem_limit();  // both shared-weight FP32 blend kernels, current device
cudaError_t launch_blend_fp32_shared(const DeviceGrid& g, const uint32_t* probe_list, uint32_t nprobes,
                                     const float4* rays, const float4* dirs, float* W, float* wsum, uint32_t* states,
                                     float4* color, float2* depth, cudaStream_t st, const uint32_t* dev_count = nullptr,
                                     const float* hyst_dev = nullptr);
cudaError_t launch_batch_blend_fp32_shared(const BatchTables& bt, const BatchBlendList& bl, uint32_t max_ntex,
                                           uint32_t max_rays, const float4* rays, cudaStream_t st);

// sky.cu: miss records of an update shaded with the atmospheric sky
cudaError_t launch_shade_sky(const DeviceGrid& g, const DeviceLight& L, uint32_t nprobes, const uint32_t* dev_count,
                             const uint32_t* probe_list, const float4* dirs, float4* rays, cudaStream_t st);

// blend.cu
cudaError_t launch_blend_fp32(const DeviceGrid& g, const uint32_t* probe_list, uint32_t nprobes, const float4* rays,
                              const float4* dirs, uint32_t* states, float4* color, float2* depth, cudaStream_t st,
                              const uint32_t* dev_count = nullptr, const float* hyst_dev = nullptr);

}  // namespace ddgi

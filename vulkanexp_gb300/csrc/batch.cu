// batch.cu — batched update of many probe volumes (ddgi_batch_* in ddgi.h).
//
// The reference updates one IrradianceProbes volume per call
// (src/IrradianceProbes.cpp:426-594).  Here a batch of contexts is updated
// together, so that small volumes share the GPU instead of each leaving it
// mostly idle:
//
//   * acceleration structures: every volume's node, triangle and instance
//     arrays are copied into one arena with their references rebased, so one
//     persistent traversal kernel serves every volume (only the top-level
//     root differs per ray).  The hit of a ray is the same as in the
//     volume's own arrays: same trees, same order, same arithmetic.
//   * ray records: one index space, volume after volume; the volume of a
//     record is found by binary search of the record offsets.
//   * per-update inputs (direction tables, octant-binned ray orders and the
//     volume table with the current lights) are written into one pinned host
//     buffer and copied by one memcpy at the head of the update.
//   * volumes are kept in increasing order of their ray counts and split
//     into up to kGroups groups of equal volume count; the groups' pipelines
//     (primary traversal, shading, shadow traversal, FP32 and BF16 blends)
//     run one after another, smallest first, so a group's volumes are done
//     when its own pipeline ends instead of every volume waiting for the
//     whole batch's traversal.  (Groups on concurrent graph branches do not
//     give that: each group's persistent traversal holds the SMs it gets,
//     and the first group's shading and blends queue behind the others'
//     traversals.)  The captured sequence (clear + clock, tensor-core
//     weights of every volume, the groups) is replayed from a CUDA graph.
//     Results do not depend on the grouping.
//   * an autotuner times candidate launch parameters on real updates.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "../../include/ddgi.h"
#include "../../include/ddgi_exact.h"
#include "common.cuh"
#include "ctx.h"
#include "kernels.h"
#include "nvtx.h"
#include "traverse.cuh"
#include "wide.h"

using namespace ddgi;

struct ddgi_batch {
    std::vector<ddgi_ctx*> vols;
    // what the batch was built from, to detect a volume changed afterwards
    std::vector<uint64_t> scene_builds;
    std::vector<ddgi_grid_desc> grids;
    // arena
    BvhNode* nodes = nullptr;
    BvhTri* tris = nullptr;
    GpuInstance* insts = nullptr;
    uint64_t node_count = 0, tri_count = 0, inst_count = 0;
    std::vector<int32_t> roots;
    int stack_cap = 1;
    // the eight-wide trees of every volume (wstack_cap 0: some volume has none)
    WideNode* wnodes = nullptr;
    GpuInstance* winsts = nullptr;
    uint64_t wnode_count = 0;
    std::vector<int32_t> wroots;
    int wstack_cap = 0;
    // per-ray buffers (all volumes)
    uint32_t total = 0;
    float4* thit = nullptr;
    uint32_t* prim = nullptr;
    uint32_t* front = nullptr;
    float4* rays = nullptr;
    uint32_t* q_idx = nullptr;
    float4* q_pos = nullptr;
    float4* q_sun = nullptr;
    uint32_t* counters = nullptr;
    // tables
    uint32_t* d_ray_base = nullptr;
    std::vector<uint32_t> ray_base;
    std::vector<uint32_t> dir_base;
    uint32_t dir_total = 0;
    unsigned long long* d_clock = nullptr;
    uint32_t* d_done = nullptr;
    uint32_t* d_err = nullptr;
    uint32_t* d_lists = nullptr;  // fp32 list, fp32 tile base, tc list, tc tile base, fp32 shared-weight tile base
    BatchBlendList fp32_bl{}, tc_bl{}, fp32s_bl{};  // fp32s: tiles of several probes, shared weights
    // internal volume i is the caller's volume order[i] (increasing ray count)
    std::vector<uint32_t> order;
    // groups of consecutive internal volumes, each with its own work
    // counters, queue regions (at its first record) and blend lists
    struct Group {
        uint32_t v0, v1, first, total;
        BatchBlendList fp32_bl, tc_bl, fp32s_bl;
    };
    std::vector<Group> groups;
    uint32_t* d_glists = nullptr;
    uint32_t max_rays_fp32 = 0, max_rows_tc = 0, max_ntex_fp32 = 0;
    size_t tc_smem = 0;
    // per-update staging: [dirs | ray orders | volume table], host pinned + device
    uint8_t* h_stage = nullptr;
    uint8_t* d_stage = nullptr;
    size_t stage_bytes = 0, off_order = 0, off_vols = 0;
    // launch state
    ddgi_batch_tuning tuning{0, 8, 0, 0, 0, 2, kDefaultWait};
    bool use_graph = true;
    cudaStream_t cap = nullptr, side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr, done_ev = nullptr;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool pending = false;
    char msg[512] = "";
};

namespace {

ddgi_status bfail(ddgi_batch* b, ddgi_status s, const char* fmt, ...) {
    if (b) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(b->msg, sizeof(b->msg), fmt, ap);
        va_end(ap);
    }
    return s;
}

ddgi_status bcuda(ddgi_batch* b, cudaError_t e, const char* what) {
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) return bfail(b, DDGI_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return bfail(b, DDGI_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define BCK(call, what)                                  \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return bcuda(b, e_, what); \
    } while (0)

template <class T>
void bfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

constexpr uint32_t kGroups = 4;  // volume groups of the graph's branches

// Node references of a volume's trees moved into the arena: inner nodes by
// node_off; leaves of the mesh trees (node index < tlas_start) by tri_off,
// leaves of the top-level tree by inst_off.
__global__ void k_rebase_nodes(const BvhNode* __restrict__ src, uint32_t n, uint32_t tlas_start, int node_off,
                               int tri_off, int inst_off, BvhNode* __restrict__ dst) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BvhNode nd = src[i];
    const int prim_off = i >= tlas_start ? inst_off : tri_off;
    int r[2] = {nd.d.x, nd.d.y};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (r[k] >= 0) {
            r[k] += node_off;
        } else {
            int first = (~r[k]) >> 3, cnt = (~r[k]) & 7;
            r[k] = ~(((first + prim_off) << 3) | cnt);
        }
    }
    nd.d.x = r[0];
    nd.d.y = r[1];
    dst[i] = nd;
}

__global__ void k_rebase_instances(const GpuInstance* __restrict__ src, uint32_t n, int node_off,
                                   GpuInstance* __restrict__ dst) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    GpuInstance g = src[i];
    if (g.blas_root >= 0) g.blas_root += node_off;
    dst[i] = g;
}

// Head of every update: clear the work counters and completion counts,
// stamp the start time.
__global__ void k_batch_begin(uint32_t* counters, uint32_t ncounters, uint32_t* done, unsigned long long* clock,
                              uint32_t nvol) {
    for (uint32_t i = threadIdx.x; i < nvol; i += blockDim.x) {
        done[i] = 0u;
        clock[1 + i] = 0ull;
    }
    for (uint32_t i = threadIdx.x; i < ncounters; i += blockDim.x) counters[i] = 0u;
    if (threadIdx.x == 0) clock[0] = globaltimer_ns();
}

ddgi_status wait_event(ddgi_batch* b, cudaEvent_t ev, int timeout_ms) {
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess) return DDGI_OK;
        if (e != cudaErrorNotReady) return bcuda(b, e, "event");
        if (timeout_ms >= 0) {
            auto el = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            if (el >= timeout_ms) return bfail(b, DDGI_ERR_TIMEOUT, "batch work not finished after %d ms", timeout_ms);
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

ddgi_status check_batch_error(ddgi_batch* b) {
    uint32_t e = 0;
    BCK(cudaMemcpy(&e, b->d_err, sizeof(e), cudaMemcpyDeviceToHost), "read device error word");
    if (e != 0) {
        cudaMemset(b->d_err, 0, sizeof(uint32_t));
        const char* what = e == DEV_STACK_OVERFLOW ? "traversal stack overflow"
                           : e == DEV_BAD_INDEX    ? "index out of range in scene data"
                           : e == DEV_WAIT_TIMEOUT ? "device wait timed out"
                                                   : "unknown device error";
        return bfail(b, DDGI_ERR_DEVICE, "device error %u: %s", e, what);
    }
    return DDGI_OK;
}

BatchTables tables(const ddgi_batch* b) {
    BatchTables t;
    t.vols = reinterpret_cast<const BatchVolume*>(b->d_stage + b->off_vols);
    t.nvol = (uint32_t)b->vols.size();
    t.ray_base = b->d_ray_base;
    t.dirs = reinterpret_cast<const float4*>(b->d_stage);
    t.ray_order = reinterpret_cast<const uint32_t*>(b->d_stage + b->off_order);
    t.clock = b->d_clock;
    t.done = b->d_done;
    t.err = b->d_err;
    t.first = 0;
    return t;
}

DeviceScene arena_scene(const ddgi_batch* b) {
    DeviceScene s{};
    s.nodes = b->nodes;
    s.tris = b->tris;
    s.instances = b->insts;
    s.tlas_root = -1;
    s.node_count = (uint32_t)b->node_count;
    s.tri_count = (uint32_t)b->tri_count;
    s.instance_count = (uint32_t)b->inst_count;
    s.wnodes = b->wstack_cap > 0 ? b->wnodes : nullptr;
    s.winstances = b->wstack_cap > 0 ? b->winsts : nullptr;
    s.wtlas_root = -1;
    s.wnode_count = (uint32_t)b->wnode_count;
    set_step_limits(s);
    return s;
}

// Volumes unchanged since the batch was made?
ddgi_status check_volumes(ddgi_batch* b) {
    for (size_t v = 0; v < b->vols.size(); ++v) {
        const ddgi_ctx* c = b->vols[v];
        if (!c->scene.built || c->scene.build_id != b->scene_builds[v])
            return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "volume %u: scene rebuilt or released since the batch was made",
                         b->order[v]);
        // extent, hysteresis, sharpness and bias are read per update; the
        // sizes fix the batch's buffers and tables
        const ddgi_grid_desc& g0 = b->grids[v];
        if (memcmp(c->grid.resolution, g0.resolution, sizeof(g0.resolution)) != 0 ||
            c->grid.rays_per_probe != g0.rays_per_probe || c->grid.color_res != g0.color_res ||
            c->grid.depth_res != g0.depth_res || c->grid.precision != g0.precision)
            return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "volume %u: grid sizes changed since the batch was made",
                         b->order[v]);
        if (c->dl.sky_mode != DDGI_SKY_CONSTANT)
            return bfail(b, DDGI_ERR_UNSUPPORTED, "volume %u: the atmospheric sky is not batched", b->order[v]);
        // the batch blends with each grid's hysteresis; a volume whose
        // hysteresis ramps (ddgi_set_target_hysteresis) would drift from
        // its own ddgi_update, so it is refused rather than blended otherwise
        if (c->ramp_on)
            return bfail(b, DDGI_ERR_UNSUPPORTED, "volume %u: the hysteresis ramp is not batched", b->order[v]);
    }
    return DDGI_OK;
}

// Direction tables, ray orders and the volume table of one update into the
// pinned staging buffer.
ddgi_status stage_inputs(ddgi_batch* b, const float* orientations) {
    const uint32_t V = (uint32_t)b->vols.size();
    for (uint32_t v = 0; v < V; ++v)
        for (int k = 0; k < 9; ++k)
            if (!std::isfinite(orientations[9 * v + k]))
                return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "volume %u: non-finite orientation", v);
    float* dirs = reinterpret_cast<float*>(b->h_stage);
    uint32_t* order = reinterpret_cast<uint32_t*>(b->h_stage + b->off_order);
    BatchVolume* bv = reinterpret_cast<BatchVolume*>(b->h_stage + b->off_vols);
    for (uint32_t v = 0; v < V; ++v) {
        ddgi_ctx* c = b->vols[v];
        const uint32_t R = c->grid.rays_per_probe;
        float* d = dirs + 4 * (size_t)b->dir_base[v];
        ddgi_ray_direction_table(&orientations[9 * (size_t)b->order[v]], R, d);  // internal v: caller's order[v]
        // the volume's own record of its current direction table
        c->host_dirs.assign(d, d + 4 * (size_t)R);
        const uint32_t rpw = grouped_rays_per_warp(b->tuning.rays_per_warp, R);
        ray_order_of(d, R, order + b->dir_base[v], rpw > 0 && rpw < 32);

        BatchVolume& x = bv[v];
        memset(&x, 0, sizeof(x));
        x.sc = device_scene(c);
        x.g = c->dg;
        x.L = c->dl;
        x.root = b->roots[v];
        x.fp16 = c->fp16 ? 1u : 0u;
        x.ray_base = b->ray_base[v];
        x.dir_base = b->dir_base[v];
        x.states = c->states;
        x.color = c->color;
        x.depth = c->depth;
        x.acc_color = c->acc_color;
        x.acc_depth = c->acc_depth;
        x.wbuf = c->tc_weights;
        x.rowsum = c->tc_rowsum;
        x.wroot = b->wroots[v];
        x.rays_per_warp = grouped_rays_per_warp(b->tuning.rays_per_warp, R);
        x.perm = x.rays_per_warp ? c->probe_perm : nullptr;
    }
    return DDGI_OK;
}

// The launch sequence of one update.  `timed`: plain launches with events
// between the phases (ev[0] start, ev[1] after the primary traversal, ev[2]
// after shading, ev[3] after the shadow rays, ev[4] after the FP32 blend,
// ev[5] after the BF16 blend); otherwise the two blends run on two branches.
cudaError_t enqueue(ddgi_batch* b, cudaStream_t st, bool timed) {
    const BatchTables bt = tables(b);
    const uint32_t V = (uint32_t)b->vols.size();
    if (timed) cudaEventRecord(b->ev[0], st);
    cudaError_t e = cudaMemcpyAsync(b->d_stage, b->h_stage, b->stage_bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    k_batch_begin<<<1, 256, 0, st>>>(b->counters, 4 * (1 + (uint32_t)b->groups.size()), b->d_done, b->d_clock, V);
    e = launch_batch_tc_weights(bt, b->tc_bl, b->max_rows_tc, st);
    if (e != cudaSuccess) return e;
    TraceTuning tt;
    tt.ctas_per_sm = b->tuning.trace_ctas_per_sm;
    tt.refill = b->tuning.refill_lanes;
    tt.split = b->tuning.smem_stack;
    tt.rays_per_warp = b->tuning.rays_per_warp;  // applied per volume through the volume table
    tt.wide = b->tuning.node_width == 8 ? 1u : 0u;
    tt.wait = b->tuning.straggler_lanes;
    if (!timed && b->groups.size() > 1) {  // the volume groups one after another, smallest first
        for (size_t gi = 0; gi < b->groups.size() && e == cudaSuccess; ++gi) {
            const ddgi_batch::Group& G = b->groups[gi];
            cudaStream_t gs = st;
            BatchTables gbt = bt;
            gbt.first = G.first;
            WaveHits gwh{b->thit, b->prim, b->front + G.first};
            ShadowQueue gq{b->q_idx + G.first, b->q_pos + G.first, b->q_sun + G.first, nullptr};
            if (e == cudaSuccess)
                e = launch_batch_trace(arena_scene(b), gbt, G.total, gwh, gq, b->counters + 4 * (1 + gi), b->rays,
                                       b->stack_cap, b->wstack_cap, tt, gs, nullptr, nullptr);
            if (e == cudaSuccess && G.fp32_bl.ntiles > 0)
                e = b->tuning.blend_threads == 0
                        ? launch_batch_blend_fp32_shared(gbt, G.fp32s_bl, b->max_ntex_fp32, b->max_rays_fp32, b->rays,
                                                         gs)
                        : launch_batch_blend_fp32(gbt, G.fp32_bl, b->max_rays_fp32, b->rays, b->tuning.blend_threads,
                                                  gs);
            if (e == cudaSuccess && G.tc_bl.ntiles > 0) e = launch_batch_blend_tc(gbt, G.tc_bl, b->rays, b->tc_smem, gs);
        }
        return e;
    }
    WaveHits wh{b->thit, b->prim, b->front};
    ShadowQueue q{b->q_idx, b->q_pos, b->q_sun, nullptr};
    e = launch_batch_trace(arena_scene(b), bt, b->total, wh, q, b->counters, b->rays, b->stack_cap, b->wstack_cap,
                           tt, st, timed ? b->ev[1] : nullptr, timed ? b->ev[2] : nullptr);
    if (e != cudaSuccess) return e;
    if (timed) cudaEventRecord(b->ev[3], st);
    const bool both = b->fp32_bl.ntiles > 0 && b->tc_bl.ntiles > 0;
    auto blend_fp32 = [&](cudaStream_t s) {
        return b->tuning.blend_threads == 0
                   ? launch_batch_blend_fp32_shared(bt, b->fp32s_bl, b->max_ntex_fp32, b->max_rays_fp32, b->rays, s)
                   : launch_batch_blend_fp32(bt, b->fp32_bl, b->max_rays_fp32, b->rays, b->tuning.blend_threads, s);
    };
    if (timed || !both) {
        e = blend_fp32(st);
        if (e != cudaSuccess) return e;
        if (timed) cudaEventRecord(b->ev[4], st);
        e = launch_batch_blend_tc(bt, b->tc_bl, b->rays, b->tc_smem, st);
        if (e != cudaSuccess) return e;
        if (timed) cudaEventRecord(b->ev[5], st);
        return cudaGetLastError();
    }
    // two branches: FP32 blend on the side stream, tensor-core blend here
    e = cudaEventRecord(b->fork_ev, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->side, b->fork_ev, 0);
    if (e == cudaSuccess)
        e = blend_fp32(b->side);
    if (e == cudaSuccess) e = launch_batch_blend_tc(bt, b->tc_bl, b->rays, b->tc_smem, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->join_ev, b->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, b->join_ev, 0);
    return e;
}

void drop_graph(ddgi_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

ddgi_status capture_graph(ddgi_batch* b) {
    drop_graph(b);
    BCK(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t e = enqueue(b, b->cap, false);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->cap, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bcuda(b, e != cudaSuccess ? e : e2, "capture batch update");
    }
    b->graph = g;
    e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) {
        drop_graph(b);
        return bcuda(b, e, "instantiate batch graph");
    }
    return DDGI_OK;
}

// Previous update's inputs consumed (the staging buffer may be rewritten)?
ddgi_status wait_previous(ddgi_batch* b) {
    if (!b->pending) return DDGI_OK;
    ddgi_status s = wait_event(b, b->done_ev, 60000);
    if (s == DDGI_OK) b->pending = false;
    return s;
}

ddgi_status run_update(ddgi_batch* b, const float* orientations, cudaStream_t st, bool timed) {
    ddgi_status s = check_volumes(b);
    if (s != DDGI_OK) return s;
    s = wait_previous(b);
    if (s != DDGI_OK) return s;
    s = stage_inputs(b, orientations);
    if (s != DDGI_OK) return s;
    if (b->use_graph && !timed) {
        if (!b->exec) {
            s = capture_graph(b);
            if (s != DDGI_OK) return s;
        }
        BCK(cudaGraphLaunch(b->exec, st), "graph launch");
    } else {
        BCK(enqueue(b, st, timed), "batch launch");
    }
    BCK(cudaEventRecord(b->done_ev, st), "event");
    b->pending = true;
    return DDGI_OK;
}

}  // namespace

extern "C" {

ddgi_status ddgi_batch_create(ddgi_ctx* const* volumes, uint32_t count, ddgi_stream stream, ddgi_batch** out) {
    if (!volumes || !out || count == 0) return DDGI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (count > kMaxBatchVolumes) return DDGI_ERR_UNSUPPORTED;
    ddgi_batch* b = new (std::nothrow) ddgi_batch();
    if (!b) return DDGI_ERR_OUT_OF_MEMORY;
    auto bail = [&](ddgi_status s) {
        // keep the message for the caller only through the status; free everything
        ddgi_batch_destroy(b);
        return s;
    };
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    for (uint32_t v = 0; v < count; ++v) {
        const ddgi_ctx* c = volumes[v];
        if (!c) return bail(DDGI_ERR_INVALID_ARGUMENT);
        for (uint32_t u = 0; u < v; ++u)
            if (volumes[u] == c) return bail(DDGI_ERR_INVALID_ARGUMENT);  // listed twice
        if (!c->scene.built) return bail(DDGI_ERR_NO_SCENE);
        // the arena carries the wide trees for node_width 8 tunings
        const ddgi_status ws = ensure_wide(volumes[v]);
        if (ws != DDGI_OK) return bail(ws);
    }
    // internal order: increasing ray count (stable)
    b->order.resize(count);
    for (uint32_t v = 0; v < count; ++v) b->order[v] = v;
    auto rays_of = [&](uint32_t v) {
        const ddgi_grid_desc& g = volumes[v]->grid;
        return (uint64_t)g.resolution[0] * g.resolution[1] * g.resolution[2] * g.rays_per_probe;
    };
    std::stable_sort(b->order.begin(), b->order.end(), [&](uint32_t x, uint32_t y) { return rays_of(x) < rays_of(y); });
    for (uint32_t v = 0; v < count; ++v) {
        ddgi_ctx* c = volumes[b->order[v]];
        b->vols.push_back(c);
        b->scene_builds.push_back(c->scene.build_id);
        b->grids.push_back(c->grid);
    }
    // ---- sizes ----
    uint64_t nodes = 0, tris = 0, insts = 0, rays = 0, dirs = 0;
    std::vector<uint32_t> fp32_list, fp32_base{0}, tc_list, tc_base{0}, fp32s_base{0};
    for (uint32_t v = 0; v < count; ++v) {
        const ddgi_ctx* c = b->vols[v];
        const uint32_t P = (uint32_t)c->grid.resolution[0] * c->grid.resolution[1] * c->grid.resolution[2];
        const uint32_t R = c->grid.rays_per_probe;
        b->ray_base.push_back((uint32_t)rays);
        b->dir_base.push_back((uint32_t)dirs);
        rays += (uint64_t)P * R;
        dirs += R;
        nodes += c->scene.node_count;
        tris += c->scene.tri_count;
        insts += c->scene.instance_count;
        b->stack_cap = std::max(b->stack_cap, c->scene.stack_cap);
        b->wnode_count += c->scene.wnode_count;
        if (v == 0) b->wstack_cap = c->scene.wstack_cap;
        b->wstack_cap = c->scene.wstack_cap > 0 && b->wstack_cap > 0 ? std::max(b->wstack_cap, c->scene.wstack_cap) : 0;
        if (b->wnode_count >= kMaxWideNodes) b->wstack_cap = 0;  // beyond the stack entries' node field
        if (c->fp16) {
            tc_list.push_back(v);
            tc_base.push_back(tc_base.back() + tc_tiles(P));
            const uint32_t nc = c->grid.color_res - 2, nd = c->grid.depth_res - 2;
            const uint32_t rows = (nc * nc + 15) / 16 * 16 + (nd * nd + 15) / 16 * 16;
            b->max_rows_tc = std::max(b->max_rows_tc, rows);
            b->tc_smem = std::max(b->tc_smem, batch_tc_smem(c->grid.color_res, c->grid.depth_res));
        } else {
            fp32_list.push_back(v);
            fp32_base.push_back(fp32_base.back() + P);
            fp32s_base.push_back(fp32s_base.back() + fp32_shared_tiles(P));
            b->max_rays_fp32 = std::max(b->max_rays_fp32, R);
            const uint32_t nc = c->grid.color_res - 2, nd = c->grid.depth_res - 2;
            b->max_ntex_fp32 = std::max(b->max_ntex_fp32, nc * nc + nd * nd);
        }
    }
    b->ray_base.push_back((uint32_t)rays);
    if (rays > DDGI_MAX_RAYS_PER_UPDATE || tris >= (1ull << 28) - 8 || insts >= (1ull << 28) - 8 || nodes >= (1ull << 31))
        return bail(DDGI_ERR_UNSUPPORTED);
    b->total = (uint32_t)rays;
    b->dir_total = (uint32_t)dirs;
    b->node_count = nodes;
    b->tri_count = tris;
    b->inst_count = insts;

    // ---- allocations ----
    const size_t N = std::max<uint64_t>(rays, 1);
    if (cudaMalloc(&b->nodes, sizeof(BvhNode) * std::max<uint64_t>(nodes, 1)) != cudaSuccess ||
        cudaMalloc(&b->tris, sizeof(BvhTri) * std::max<uint64_t>(tris, 1)) != cudaSuccess ||
        cudaMalloc(&b->insts, sizeof(GpuInstance) * std::max<uint64_t>(insts, 1)) != cudaSuccess ||
        cudaMalloc(&b->wnodes, sizeof(WideNode) * std::max<uint64_t>(b->wnode_count, 1)) != cudaSuccess ||
        cudaMalloc(&b->winsts, sizeof(GpuInstance) * std::max<uint64_t>(insts, 1)) != cudaSuccess ||
        cudaMalloc(&b->thit, sizeof(float4) * N) != cudaSuccess ||
        cudaMalloc(&b->prim, sizeof(uint32_t) * N) != cudaSuccess ||
        cudaMalloc(&b->front, sizeof(uint32_t) * N) != cudaSuccess ||
        cudaMalloc(&b->rays, sizeof(float4) * N) != cudaSuccess ||
        cudaMalloc(&b->q_idx, sizeof(uint32_t) * N) != cudaSuccess ||
        cudaMalloc(&b->q_pos, sizeof(float4) * N) != cudaSuccess ||
        cudaMalloc(&b->q_sun, sizeof(float4) * N) != cudaSuccess ||
        cudaMalloc(&b->counters, 4 * (1 + kGroups) * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&b->d_ray_base, sizeof(uint32_t) * (count + 1)) != cudaSuccess ||
        cudaMalloc(&b->d_clock, sizeof(unsigned long long) * (count + 1)) != cudaSuccess ||
        cudaMalloc(&b->d_done, sizeof(uint32_t) * count) != cudaSuccess ||
        cudaMalloc(&b->d_err, sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&b->d_lists, sizeof(uint32_t) * (3 * count + 3)) != cudaSuccess) {
        cudaGetLastError();
        return bail(DDGI_ERR_OUT_OF_MEMORY);
    }
    b->off_order = align_up(sizeof(float4) * b->dir_total, 256);
    b->off_vols = align_up(b->off_order + sizeof(uint32_t) * b->dir_total, 256);
    b->stage_bytes = b->off_vols + sizeof(BatchVolume) * count;
    if (cudaMallocHost(&b->h_stage, b->stage_bytes) != cudaSuccess ||
        cudaMalloc(&b->d_stage, b->stage_bytes) != cudaSuccess) {
        cudaGetLastError();
        return bail(DDGI_ERR_OUT_OF_MEMORY);
    }
    memset(b->h_stage, 0, b->stage_bytes);
    if (cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->done_ev, cudaEventDisableTiming) != cudaSuccess)
        return bail(DDGI_ERR_CUDA);
    for (int i = 0; i < 6; ++i)
        if (cudaEventCreate(&b->ev[i]) != cudaSuccess) return bail(DDGI_ERR_CUDA);

    // ---- tables ----
    std::vector<uint32_t> lists;
    lists.insert(lists.end(), fp32_list.begin(), fp32_list.end());
    lists.insert(lists.end(), fp32_base.begin(), fp32_base.end());
    lists.insert(lists.end(), tc_list.begin(), tc_list.end());
    lists.insert(lists.end(), tc_base.begin(), tc_base.end());
    lists.insert(lists.end(), fp32s_base.begin(), fp32s_base.end());
    if (cudaMemcpyAsync(b->d_lists, lists.data(), sizeof(uint32_t) * lists.size(), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(b->d_ray_base, b->ray_base.data(), sizeof(uint32_t) * (count + 1), cudaMemcpyHostToDevice,
                        st) != cudaSuccess ||
        cudaMemsetAsync(b->d_err, 0, sizeof(uint32_t), st) != cudaSuccess ||
        cudaMemsetAsync(b->d_clock, 0, sizeof(unsigned long long) * (count + 1), st) != cudaSuccess)
        return bail(DDGI_ERR_CUDA);
    const uint32_t nf = (uint32_t)fp32_list.size(), nt = (uint32_t)tc_list.size();
    b->fp32_bl = BatchBlendList{b->d_lists, b->d_lists + nf, nf, fp32_base.back()};
    b->tc_bl = BatchBlendList{b->d_lists + 2 * nf + 1, b->d_lists + 2 * nf + 1 + nt, nt, tc_base.back()};
    b->fp32s_bl = BatchBlendList{b->d_lists, b->d_lists + 2 * nf + 2 * nt + 2, nf, fp32s_base.back()};

    // ---- volume groups: equal volume counts, their own blend lists ----
    {
        const uint32_t K = std::min<uint32_t>(kGroups, count);
        std::vector<uint32_t> gl;
        struct Off {
            size_t fl, fb, tl, tb, sb;
            uint32_t nf, nt, fbt, tbt, sbt;
        };
        std::vector<Off> offs;
        for (uint32_t k = 0; k < K; ++k) {
            ddgi_batch::Group G{};
            G.v0 = (uint32_t)((uint64_t)count * k / K);
            G.v1 = (uint32_t)((uint64_t)count * (k + 1) / K);
            G.first = b->ray_base[G.v0];
            G.total = b->ray_base[G.v1] - G.first;
            std::vector<uint32_t> fl, fb{0}, tl, tb{0}, sb{0};
            for (uint32_t v = G.v0; v < G.v1; ++v) {
                const ddgi_ctx* c = b->vols[v];
                const uint32_t P = (uint32_t)c->grid.resolution[0] * c->grid.resolution[1] * c->grid.resolution[2];
                if (c->fp16) {
                    tl.push_back(v);
                    tb.push_back(tb.back() + tc_tiles(P));
                } else {
                    fl.push_back(v);
                    fb.push_back(fb.back() + P);
                    sb.push_back(sb.back() + fp32_shared_tiles(P));
                }
            }
            Off o;
            o.nf = (uint32_t)fl.size();
            o.nt = (uint32_t)tl.size();
            o.fbt = fb.back();
            o.tbt = tb.back();
            o.sbt = sb.back();
            o.fl = gl.size(), gl.insert(gl.end(), fl.begin(), fl.end());
            o.fb = gl.size(), gl.insert(gl.end(), fb.begin(), fb.end());
            o.tl = gl.size(), gl.insert(gl.end(), tl.begin(), tl.end());
            o.tb = gl.size(), gl.insert(gl.end(), tb.begin(), tb.end());
            o.sb = gl.size(), gl.insert(gl.end(), sb.begin(), sb.end());
            offs.push_back(o);
            b->groups.push_back(G);
        }
        if (cudaMalloc(&b->d_glists, sizeof(uint32_t) * std::max<size_t>(gl.size(), 1)) != cudaSuccess ||
            cudaMemcpyAsync(b->d_glists, gl.data(), sizeof(uint32_t) * gl.size(), cudaMemcpyHostToDevice, st) !=
                cudaSuccess) {
            cudaGetLastError();
            return bail(DDGI_ERR_OUT_OF_MEMORY);
        }
        for (uint32_t k = 0; k < K; ++k) {
            const Off& o = offs[k];
            ddgi_batch::Group& G = b->groups[k];
            G.fp32_bl = BatchBlendList{b->d_glists + o.fl, b->d_glists + o.fb, o.nf, o.fbt};
            G.tc_bl = BatchBlendList{b->d_glists + o.tl, b->d_glists + o.tb, o.nt, o.tbt};
            G.fp32s_bl = BatchBlendList{b->d_glists + o.fl, b->d_glists + o.sb, o.nf, o.sbt};
        }
    }

    // ---- arena: copy every volume's trees with rebased references ----
    uint64_t node_off = 0, tri_off = 0, inst_off = 0, wnode_off = 0;
    for (uint32_t v = 0; v < count; ++v) {
        const ddgi_ctx* c = b->vols[v];
        const SceneBuffers& S = c->scene;
        const uint32_t n = (uint32_t)S.node_count;
        if (n > 0) {
            const uint32_t tlas_start = S.tlas_root >= 0 ? (uint32_t)S.tlas_root : n;
            k_rebase_nodes<<<(n + 255) / 256, 256, 0, st>>>(S.nodes, n, tlas_start, (int)node_off, (int)tri_off,
                                                            (int)inst_off, b->nodes + node_off);
        }
        if (S.tri_count > 0 &&
            cudaMemcpyAsync(b->tris + tri_off, S.tris, sizeof(BvhTri) * S.tri_count, cudaMemcpyDeviceToDevice, st) !=
                cudaSuccess)
            return bail(DDGI_ERR_CUDA);
        if (S.instance_count > 0)
            k_rebase_instances<<<(S.instance_count + 255) / 256, 256, 0, st>>>(S.inst_leaf, S.instance_count,
                                                                               (int)node_off, b->insts + inst_off);
        b->roots.push_back(S.tlas_root >= 0 ? (int32_t)(S.tlas_root + node_off) : -1);
        if (b->wstack_cap > 0) {
            if (launch_rebase_wide(S.wnodes, S.wnode_count, S.wide_tlas_start, (int)wnode_off, (int)tri_off,
                                   (int)inst_off, b->wnodes + wnode_off, st) != cudaSuccess)
                return bail(DDGI_ERR_CUDA);
            if (S.instance_count > 0)
                k_rebase_instances<<<(S.instance_count + 255) / 256, 256, 0, st>>>(
                    S.winst_leaf, S.instance_count, (int)wnode_off, b->winsts + inst_off);
        }
        b->wroots.push_back(S.wtlas_root >= 0 ? (int32_t)(S.wtlas_root + wnode_off) : -1);
        wnode_off += S.wnode_count;
        node_off += S.node_count;
        tri_off += S.tri_count;
        inst_off += S.instance_count;
    }
    if (cudaGetLastError() != cudaSuccess || prepare_batch_kernels() != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return bail(DDGI_ERR_CUDA);
    *out = b;
    return DDGI_OK;
}

ddgi_status ddgi_batch_destroy(ddgi_batch* b) {
    if (!b) return DDGI_OK;
    if (b->pending) wait_event(b, b->done_ev, 60000);
    drop_graph(b);
    bfree(b->nodes);
    bfree(b->tris);
    bfree(b->insts);
    bfree(b->wnodes);
    bfree(b->winsts);
    bfree(b->thit);
    bfree(b->prim);
    bfree(b->front);
    bfree(b->rays);
    bfree(b->q_idx);
    bfree(b->q_pos);
    bfree(b->q_sun);
    bfree(b->counters);
    bfree(b->d_ray_base);
    bfree(b->d_clock);
    bfree(b->d_done);
    bfree(b->d_err);
    bfree(b->d_lists);
    bfree(b->d_glists);
    bfree(b->d_stage);
    if (b->h_stage) cudaFreeHost(b->h_stage);
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->join_ev) cudaEventDestroy(b->join_ev);
    if (b->done_ev) cudaEventDestroy(b->done_ev);
    for (int i = 0; i < 6; ++i)
        if (b->ev[i]) cudaEventDestroy(b->ev[i]);
    delete b;
    return DDGI_OK;
}

const char* ddgi_batch_last_error(const ddgi_batch* b) { return b ? b->msg : "null batch"; }

uint64_t ddgi_batch_ray_count(const ddgi_batch* b) { return b ? b->total : 0; }

ddgi_status ddgi_batch_get_tuning(const ddgi_batch* b, ddgi_batch_tuning* out) {
    if (!b || !out) return DDGI_ERR_INVALID_ARGUMENT;
    *out = b->tuning;
    return DDGI_OK;
}

ddgi_status ddgi_batch_set_tuning(ddgi_batch* b, const ddgi_batch_tuning* t) {
    if (!b || !t) return DDGI_ERR_INVALID_ARGUMENT;
    if (t->refill_lanes < 1 || t->refill_lanes > 32)
        return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "refill_lanes = %u outside [1, 32]", t->refill_lanes);
    if (t->blend_threads != 0 && (t->blend_threads < 32 || t->blend_threads > 256 || t->blend_threads % 32))
        return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "blend_threads = %u: want 0 or a multiple of 32 in [32, 256]",
                     t->blend_threads);
    if (t->smem_stack > (uint32_t)kSpillMax || t->trace_ctas_per_sm > 32)
        return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "smem_stack or trace_ctas_per_sm out of range");
    const uint32_t r = t->rays_per_warp;
    if (!(r == 0 || r == 1 || r == 2 || r == 4 || r == 8 || r == 16 || r == 32))
        return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "rays_per_warp = %u: want 0, 1, 2, 4, 8, 16 or 32", r);
    if (t->node_width != 2 && t->node_width != 8)
        return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "node_width = %u: want 2 or 8", t->node_width);
    if (t->straggler_lanes > 31)
        return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "straggler_lanes = %u outside [0, 31]", t->straggler_lanes);
    ddgi_status s = wait_previous(b);
    if (s != DDGI_OK) return s;
    b->tuning = *t;
    drop_graph(b);  // recaptured with the new launch shapes
    return DDGI_OK;
}

ddgi_status ddgi_batch_use_graph(ddgi_batch* b, int enable) {
    if (!b) return DDGI_ERR_INVALID_ARGUMENT;
    b->use_graph = enable != 0;
    return DDGI_OK;
}

ddgi_status ddgi_batch_update(ddgi_batch* b, const float* orientations, ddgi_stream stream) {
    ddgi::NvtxRange nvtx_range("ddgi_batch_update");
    if (!b || !orientations) return DDGI_ERR_INVALID_ARGUMENT;
    return run_update(b, orientations, reinterpret_cast<cudaStream_t>(stream), false);
}

ddgi_status ddgi_batch_synchronize(ddgi_batch* b, ddgi_stream stream, int timeout_ms) {
    if (!b) return DDGI_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return bcuda(b, e, "stream");
        if (timeout_ms >= 0) {
            auto el = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            if (el >= timeout_ms) return bfail(b, DDGI_ERR_TIMEOUT, "stream not idle after %d ms", timeout_ms);
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    if (b->pending && cudaEventQuery(b->done_ev) == cudaSuccess) b->pending = false;
    return check_batch_error(b);
}

ddgi_status ddgi_batch_completion_ms(ddgi_batch* b, float* ms, uint32_t count) {
    if (!b || !ms) return DDGI_ERR_INVALID_ARGUMENT;
    const uint32_t V = (uint32_t)b->vols.size();
    if (count < V) return bfail(b, DDGI_ERR_INVALID_ARGUMENT, "need room for %u volumes", V);
    ddgi_status s = wait_previous(b);
    if (s != DDGI_OK) return s;
    std::vector<unsigned long long> clk(V + 1);
    BCK(cudaMemcpy(clk.data(), b->d_clock, sizeof(unsigned long long) * (V + 1), cudaMemcpyDeviceToHost), "read clock");
    for (uint32_t v = 0; v < V; ++v)  // internal volume v is the caller's order[v]
        ms[b->order[v]] =
            clk[1 + v] >= clk[0] && clk[1 + v] != 0 ? (float)((double)(clk[1 + v] - clk[0]) * 1e-6) : -1.0f;
    return DDGI_OK;
}

ddgi_status ddgi_batch_autotune(ddgi_batch* b, const float* orientations, uint32_t reps, ddgi_stream stream,
                                ddgi_batch_tuning* chosen) {
    if (!b || !orientations) return DDGI_ERR_INVALID_ARGUMENT;
    if (reps == 0) reps = 3;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    ddgi_status s = check_volumes(b);
    if (s != DDGI_OK) return s;
    s = wait_previous(b);
    if (s != DDGI_OK) return s;
    // ---- save what the trial updates overwrite ----
    struct Saved {
        void* dst;
        void* copy;
        size_t bytes;
    };
    std::vector<Saved> saved;
    auto save = [&](void* p, size_t bytes) -> bool {
        if (!p || bytes == 0) return true;
        void* c = nullptr;
        if (cudaMalloc(&c, bytes) != cudaSuccess) return false;
        saved.push_back({p, c, bytes});
        return cudaMemcpyAsync(c, p, bytes, cudaMemcpyDeviceToDevice, st) == cudaSuccess;
    };
    auto release = [&]() {
        for (auto& x : saved) cudaFree(x.copy);
        saved.clear();
    };
    bool ok = true;
    for (ddgi_ctx* c : b->vols) {
        const DeviceGrid& g = c->dg;
        const size_t ct = (size_t)g.color_w * g.color_h, dt = (size_t)g.depth_w * g.depth_h;
        const uint32_t P = (uint32_t)g.res[0] * g.res[1] * g.res[2];
        ok = ok && save(c->color, ct * (c->fp16 ? 8 : 16)) && save(c->depth, dt * (c->fp16 ? 4 : 8)) &&
             save(c->states, sizeof(uint32_t) * P);
        if (c->fp16) ok = ok && save(c->acc_color, ct * 16) && save(c->acc_depth, dt * 8);
    }
    if (!ok) {
        cudaStreamSynchronize(st);
        release();
        cudaGetLastError();
        return bfail(b, DDGI_ERR_OUT_OF_MEMORY, "autotune: no room to save the volumes' atlases");
    }
    const ddgi_batch_tuning start = b->tuning;
    // time of one candidate: median over reps of the phase it tunes
    auto measure = [&](const ddgi_batch_tuning& t, int phase, float* out) -> ddgi_status {
        b->tuning = t;
        std::vector<float> v;
        for (uint32_t r = 0; r <= reps; ++r) {  // first run untimed
            ddgi_status q = run_update(b, orientations, st, true);
            if (q != DDGI_OK) return q;
            q = wait_event(b, b->ev[5], 60000);
            if (q != DDGI_OK) return q;
            b->pending = false;
            float a = 0.0f;
            if (phase == 0) cudaEventElapsedTime(&a, b->ev[0], b->ev[3]);  // traversal + shading
            else cudaEventElapsedTime(&a, b->ev[3], b->ev[4]);             // FP32 blend
            if (r > 0) v.push_back(a);
        }
        std::sort(v.begin(), v.end());
        *out = v[v.size() / 2];
        return check_batch_error(b);
    };
    ddgi_batch_tuning best = start;
    ddgi_status err = DDGI_OK;
    float best_t = 0.0f;
    err = measure(best, 0, &best_t);
    const uint32_t width_c[] = {8u, 2u};
    const uint32_t rpw_c[] = {0u, 32u, 16u, 8u, 4u, 2u, 1u};
    const uint32_t split_c[] = {0u, 32u, 24u, 16u};
    const uint32_t refill_c[] = {4u, 8u, 16u, 24u};
    const uint32_t ctas_c[] = {0u, 6u, 4u};
    const uint32_t wait_c[] = {6u, 8u, 10u, 12u, 14u};
    for (int p = 0; p < 6 && err == DDGI_OK; ++p) {
        const uint32_t* cand = p == 0   ? width_c
                               : p == 1 ? rpw_c
                               : p == 2 ? split_c
                               : p == 3 ? refill_c
                               : p == 4 ? ctas_c
                                        : wait_c;
        const int nc = p == 0 ? 2 : p == 1 ? 7 : p == 4 ? 3 : p == 5 ? 5 : 4;
        for (int i = 0; i < nc && err == DDGI_OK; ++i) {
            ddgi_batch_tuning t = best;
            uint32_t* field = p == 0   ? &t.node_width
                              : p == 1 ? &t.rays_per_warp
                              : p == 2 ? &t.smem_stack
                              : p == 3 ? &t.refill_lanes
                              : p == 4 ? &t.trace_ctas_per_sm
                                       : &t.straggler_lanes;
            if (*field == cand[i]) continue;
            const int cap = t.node_width == 8 && b->wstack_cap > 0 ? b->wstack_cap : b->stack_cap;
            if (p == 2 && cand[i] != 0 && (int)cand[i] >= cap) continue;
            *field = cand[i];
            float tt = 0.0f;
            err = measure(t, 0, &tt);
            if (err == DDGI_OK && tt < best_t) {
                best_t = tt;
                best = t;
            }
        }
    }
    if (err == DDGI_OK && b->fp32_bl.ntiles > 0) {
        float bt = 0.0f;
        err = measure(best, 1, &bt);
        const uint32_t thr_c[] = {0u, 64u, 128u, 256u};
        for (int i = 0; i < 4 && err == DDGI_OK; ++i) {
            if (thr_c[i] == best.blend_threads) continue;
            ddgi_batch_tuning t = best;
            t.blend_threads = thr_c[i];
            float tt = 0.0f;
            err = measure(t, 1, &tt);
            if (err == DDGI_OK && tt < bt) {
                bt = tt;
                best = t;
            }
        }
    }
    // ---- restore the volumes ----
    for (auto& x : saved) cudaMemcpyAsync(x.dst, x.copy, x.bytes, cudaMemcpyDeviceToDevice, st);
    cudaError_t e = cudaStreamSynchronize(st);
    release();
    b->tuning = err == DDGI_OK ? best : start;
    drop_graph(b);
    if (err != DDGI_OK) return err;
    if (e != cudaSuccess) return bcuda(b, e, "autotune restore");
    if (chosen) *chosen = best;
    return DDGI_OK;
}

}  // extern "C"

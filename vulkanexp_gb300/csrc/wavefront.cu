// wavefront.cu — the probe trace as three kernels instead of one.
//
//  1. k_primary: closest hit of every probe ray.  Persistent warps; a lane
//     whose ray finishes is handed the next ray from a global counter, so the
//     warp keeps its lanes busy instead of waiting for its longest ray.
//  2. k_shade: one thread per ray record, coalesced: miss -> sky, backface ->
//     (0, 0.8 t), front face -> shading split around the shadow query; the
//     front hits are appended (warp-aggregated) to a shadow-ray queue.
//  3. k_shadow: any-hit query of the queued rays toward the sun, persistent
//     like k_primary; an unshadowed ray gets (base + sun) * fade.
//
// Results are identical to the single fused kernel (same traversal, same
// shading arithmetic); only the schedule differs.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "shade.cuh"
#include "traverse.cuh"

namespace ddgi {

namespace {

constexpr int kPersistThreads = kWalkerThreads;  // the walkers' shared-memory stacks assume it
constexpr unsigned kFull = 0xffffffffu;

// Work item `id` of a grouped order: groups of G = 32 / rpw probes (in perm
// order) take rpw consecutive directions of the ray order each per 32 items,
// so a warp traces similar directions from neighbouring probes.  Returns the
// probe slot and the position in the ray order.
__device__ __forceinline__ void grouped_ray(uint32_t id, uint32_t R, uint32_t rpw, uint32_t n,
                                            const uint32_t* perm, uint32_t* slot, uint32_t* j) {
    const uint32_t G = 32u / rpw;
    const uint32_t first = (id / (G * R)) * G;
    const uint32_t m = min(G, n - first);
    const uint32_t local = id - first * R;
    const uint32_t span = m * rpw;
    const uint32_t c = local / span, r = local - c * span;
    const uint32_t q = r / rpw;
    *j = c * rpw + (r - q * rpw);
    *slot = __ldg(perm + first + q);
}

struct PrimaryJob {
    DeviceGrid g;
    const uint32_t* probe_list;
    const float4* dirs;
    const uint32_t* ray_order;
    WaveHits hits;
    uint32_t total;
    const uint32_t* dev_count;  // listed probes, read on the device (NULL: total / rays)
    const uint32_t* perm;       // grouped order over all probes (NULL: a warp per probe slot)
    uint32_t rpw, nprobes;

    template <class W>
    __device__ __forceinline__ bool start(W& w, const DeviceScene& sc, uint32_t id, uint32_t* out) const {
        const uint32_t R = g.rays;
        uint32_t slot, j;
        if (perm) {
            grouped_ray(id, R, rpw, nprobes, perm, &slot, &j);
        } else {
            slot = id / R;
            j = id - slot * R;
        }
        uint32_t ray = __ldg(ray_order + j);
        uint32_t probe = probe_list ? __ldg(probe_list + slot) : slot;
        *out = slot * R + ray;
        float4 d4 = __ldg(dirs + ray);
        return w.start(sc, probe_origin_exact(g, probe), f3(d4.x, d4.y, d4.z), 0.01f, g.tmax, 0x3u);
    }
    template <class W>
    __device__ __forceinline__ void finish(const W& w, uint32_t out) const {
        const HitRec& h = w.best;
        hits.thit[out] = make_float4(h.t, h.b1, h.b2, __uint_as_float(h.inst));
        hits.prim[out] = h.prim | (h.back ? 0x80000000u : 0u);
    }
};

struct ShadowJob {
    const ShadowQueue q;
    float3 dir;
    float4* rays;
    uint32_t* prim;  // hit words: bit 30 marks a shadowed front hit (kept for replays)
    uint32_t total;

    template <class W>
    __device__ __forceinline__ bool start(W& w, const DeviceScene& sc, uint32_t id, uint32_t* out) const {
        *out = id;
        float4 p = q.pos[id];
        return w.start(sc, f3(p.x, p.y, p.z), dir, 0.1f, 10000.0f, 0xFFu);
    }
    template <class W>
    __device__ __forceinline__ void finish(const W& w, uint32_t id) const {
        uint32_t idx = q.idx[id];
        if (w.best.inst != kNoHit) {  // shadowed: the record keeps the base colour
            prim[idx] |= 1u << 30;
            return;
        }
        float4 sun = q.sun[id];
        float4 rec = rays[idx];
        float3 c = (f3(rec.x, rec.y, rec.z) + f3(sun.x, sun.y, sun.z)) * sun.w;
        rays[idx] = make_float4(c.x, c.y, c.z, rec.w);
    }
};

__device__ __forceinline__ void init_stack(SmemStack& s, int* base, int, int*) { s.base = base; }
__device__ __forceinline__ void init_stack(SplitStack& s, int* base, int split, int* spill) {
    s.base = base;
    s.split = split;
    s.spill = spill;
}
template <class Stack>
struct SpillArea {  // local-memory tail of a SplitStack
    __device__ __forceinline__ int* ptr() { return nullptr; }
};
template <>
struct SpillArea<SplitStack> {
    int a[kSpillMax];
    __device__ __forceinline__ int* ptr() { return a; }
};

// Persistent traversal loop with per-lane refill.  A warp refills when at
// least `refill` of its lanes are idle (or all are), taking as many rays as
// it has idle lanes with one atomic.
template <bool ANY, class Stack, template <bool, class> class Walker, class Job>
__device__ __forceinline__ void persistent_walk(const DeviceScene& sc, const Job& job, uint32_t total,
                                                uint32_t* counter, int stack_cap, int split, WalkKnobs knobs,
                                                uint32_t* err) {
    const int refill = knobs.refill;
    extern __shared__ int s_stack[];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    SpillArea<Stack> spill;
    Walker<ANY, Stack> w;
    init_stack(w.stk, s_stack + threadIdx.x, split, spill.ptr());
    w.cap = stack_cap;
    w.clear();
    w.wait_max = knobs.wait;
    bool active = false;
    bool drained = false;  // warp-uniform: the work counter has passed `total`
    uint32_t out = 0;
    for (;;) {
        unsigned busy = __ballot_sync(kFull, active);
        const unsigned idle = ~busy;
        if (!drained && (__popc(idle) >= refill || busy == 0)) {
            int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            drained = base >= total;  // the counter only grows: every later request fails too
            if (!active) {
                uint32_t id = base + (uint32_t)__popc(idle & lt);
                if (id < total) {
                    if (job.start(w, sc, id, &out)) active = true;
                    else job.finish(w, out);  // empty scene: immediate miss
                }
            }
            busy = __ballot_sync(kFull, active);
        }
        if (busy == 0) {
            if (drained) break;
            continue;
        }
        bool fin = w.advance(sc, err, active);  // every lane takes part (warp votes)
        if (active && fin) {
            job.finish(w, out);
            active = false;
        }
    }
}

template <class Stack, template <bool, class> class Walker>
__global__ void __launch_bounds__(kPersistThreads, Walker<false, Stack>::kMinBlocks) k_primary(DeviceScene sc, PrimaryJob job, uint32_t* counter,
                                                                int stack_cap, int split, WalkKnobs knobs, uint32_t* err) {
    const uint32_t total = job.dev_count ? *job.dev_count * job.g.rays : job.total;
    persistent_walk<false, Stack, Walker>(sc, job, total, counter, stack_cap, split, knobs, err);
}

template <class Stack, template <bool, class> class Walker>
__global__ void __launch_bounds__(kPersistThreads, Walker<false, Stack>::kMinBlocks) k_shadow(DeviceScene sc, ShadowJob job, const uint32_t* qcount,
                                                               uint32_t* counter, int stack_cap, int split, WalkKnobs knobs,
                                                               uint32_t* err) {
    persistent_walk<true, Stack, Walker>(sc, job, *qcount, counter, stack_cap, split, knobs, err);
}

// Warp-aggregated append: the lanes with `flag` get consecutive slots of a
// queue whose length is *count; returns this lane's slot (valid if flag).
__device__ __forceinline__ uint32_t warp_append(bool flag, uint32_t* count) {
    const unsigned m = __ballot_sync(kFull, flag);
    if (!m) return 0;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(kFull, base, leader);
    return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

// Shading, pass 1, one thread per record: a miss gets the sky radiance
// (miss.rmiss:17-23), a back face (0, 0, 0, 0.8 t) (closesthit.glsl:137-141);
// front faces go to a compacted queue so that pass 2 runs in full warps.
__global__ void __launch_bounds__(128) k_shade_classify(DeviceGrid g, DeviceLight L, uint32_t total, WaveHits hits,
                                                        float4* rays_out, ddgi_hit* hits_out, uint32_t* front_count,
                                                        const uint32_t* dev_count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (dev_count) total = *dev_count * g.rays;
    bool is_front = false;
    if (i < total) {
        const float4 th = hits.thit[i];
        const uint32_t pb = hits.prim[i];
        const uint32_t inst = __float_as_uint(th.w), prim = pb & 0x0fffffffu;
        const bool back = (pb >> 31) != 0;
        if (inst == kNoHit) rays_out[i] = make_float4(L.sky[0], L.sky[1], L.sky[2], -1.0f);
        else if (back) rays_out[i] = make_float4(0.0f, 0.0f, 0.0f, th.x * 0.80f);
        else is_front = true;
        if (hits_out) {
            ddgi_hit hr;
            hr.instance = inst;
            hr.primitive = inst == kNoHit ? 0u : prim;
            hr.t = inst == kNoHit ? 0.0f : th.x;
            hr.backface = (inst != kNoHit && back) ? 1u : 0u;
            hits_out[i] = hr;
        }
    }
    const uint32_t k = warp_append(is_front, front_count);
    if (is_front) hits.front[k] = i;
}

// Shading, pass 2, one thread per queued front hit: closesthit.glsl
// (NO_REFLECTION) up to the shadow query, whose rays are appended to the
// shadow queue (an unshadowed ray later adds the sun term).
// Built for eight resident blocks per SM (64 registers): 0.05 ms faster per
// update than six (80 registers, no spill) on the 1M-triangle terrain.
template <class AV>
__global__ void __launch_bounds__(128, 8) k_shade_front(DeviceScene sc, DeviceGrid g, DeviceLight L,
                                                        const uint32_t* __restrict__ probe_list,
                                                        const float4* __restrict__ dirs,
                                                        const uint32_t* __restrict__ states, AV at, WaveHits hits,
                                                        const uint32_t* front_count, float4* rays_out, ShadowQueue q,
                                                        uint32_t* err) {
    const uint32_t n = *front_count;
    if (blockIdx.x * blockDim.x >= n) return;  // whole block
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    bool enqueue = false;
    SurfaceShade s;
    uint32_t i = 0;
    if (k < n) {
        i = hits.front[k];
        const uint32_t R = g.rays;
        const uint32_t slot = i / R, ray = i - slot * R;
        const float4 th = hits.thit[i];
        const uint32_t inst = __float_as_uint(th.w), prim = hits.prim[i] & 0x0fffffffu;
        const uint32_t probe = probe_list ? __ldg(probe_list + slot) : slot;
        const float4 d4 = __ldg(dirs + ray);
        if (shade_surface(sc, g, L, states, at, probe_origin_exact(g, probe), f3(d4.x, d4.y, d4.z), th.x, th.y, th.z,
                          inst, prim, &s, err))
            enqueue = true;
        rays_out[i] = make_float4(s.base.x, s.base.y, s.base.z, th.x);
    }
    const uint32_t qk = warp_append(enqueue, q.count);
    if (enqueue) {
        q.idx[qk] = i;
        q.pos[qk] = make_float4(s.position.x, s.position.y, s.position.z, 0.0f);
        q.sun[qk] = make_float4(s.sun.x, s.sun.y, s.sun.z, s.fade);
    }
}

// ---------------------------------------------------------------------------
// Probe classification (src/shaders/probesInit.rgen:31-64 with
// probeInitMiss.rmiss and backfaceTest.rchit): 512 closest-hit rays per
// probe among INSTANCE_STATIC (mask 1) instances, t in [0.01, 1.5 |cell|].
// A hit closer than |cell| counts as a back-face hit when back-facing, and
// marks the probe as near geometry when it lies within one cell of the probe
// on every axis (hit position rounded product, then sum).
// ---------------------------------------------------------------------------
struct InitJob {
    DeviceGrid g;
    const float4* dirs;  // kInitRays directions
    float tmax;
    uint32_t* back;  // per probe
    uint32_t* near;  // per probe

    template <class W>
    __device__ __forceinline__ bool start(W& w, const DeviceScene& sc, uint32_t id, uint32_t* out) const {
        *out = id;
        const uint32_t probe = id / kInitRays, i = id - probe * kInitRays;
        float4 d4 = __ldg(dirs + i);
        return w.start(sc, probe_origin_exact(g, probe), f3(d4.x, d4.y, d4.z), 0.01f, tmax, 0x1u);
    }
    template <class W>
    __device__ __forceinline__ void finish(const W& w, uint32_t id) const {
        const HitRec& h = w.best;
        if (h.inst == kNoHit || !(h.t < g.cell_len)) return;
        const uint32_t probe = id / kInitRays;
        if (h.back) atomicAdd(back + probe, 1u);
        const float3 o = w.wr.o, d = w.wr.d;
        const float dx = fabsf(__fsub_rn(__fadd_rn(__fmul_rn(d.x, h.t), o.x), o.x));
        const float dy = fabsf(__fsub_rn(__fadd_rn(__fmul_rn(d.y, h.t), o.y), o.y));
        const float dz = fabsf(__fsub_rn(__fadd_rn(__fmul_rn(d.z, h.t), o.z), o.z));
        if (dx < g.cell[0] && dy < g.cell[1] && dz < g.cell[2]) near[probe] = 1u;
    }
};

__global__ void __launch_bounds__(kPersistThreads) k_init_probes(DeviceScene sc, InitJob job, uint32_t total,
                                                                 uint32_t* counter, int stack_cap, uint32_t* err) {
    persistent_walk<false, SmemStack, WarpWalker>(sc, job, total, counter, stack_cap, stack_cap,
                                                  WalkKnobs{8, kDefaultWait}, err);
}

// State per probe: OFF (0) when more than half of raysPerProbe back-face
// hits, else 1 near geometry, else 8.
__global__ void k_init_states(uint32_t P, uint32_t R, const uint32_t* back, const uint32_t* near, uint32_t* states) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    states[p] = 2u * back[p] > R ? 0u : (near[p] ? 1u : 8u);
}

// ---------------------------------------------------------------------------
// Batched form: the records of all volumes form one index space; the volume
// of record `id` is found by binary search of the record offsets.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t batch_volume(const BatchTables& bt, uint32_t id) {
    uint32_t lo = 0, hi = bt.nvol;  // ray_base[lo] <= id < ray_base[hi]
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(bt.ray_base + mid) <= id) lo = mid;
        else hi = mid;
    }
    return lo;
}

struct BatchPrimaryJob {
    BatchTables bt;
    WaveHits hits;

    template <class W>
    __device__ __forceinline__ bool start(W& w, const DeviceScene& sc, uint32_t id, uint32_t* out) const {
        id += bt.first;  // records of the launch's volumes
        const uint32_t v = batch_volume(bt, id);
        const BatchVolume& vol = bt.vols[v];
        const uint32_t R = vol.g.rays;
        const uint32_t base = __ldg(bt.ray_base + v);
        const uint32_t local = id - base;
        uint32_t slot, j;
        if (vol.perm) {
            grouped_ray(local, R, vol.rays_per_warp,
                        (uint32_t)vol.g.res[0] * (uint32_t)vol.g.res[1] * (uint32_t)vol.g.res[2], vol.perm, &slot, &j);
        } else {
            slot = local / R;
            j = local - slot * R;
        }
        const uint32_t ray = __ldg(bt.ray_order + vol.dir_base + j);
        *out = base + slot * R + ray;
        float4 d4 = __ldg(bt.dirs + vol.dir_base + ray);
        return w.start_at(sc, W::kWide ? vol.wroot : vol.root, probe_origin_exact(vol.g, slot), f3(d4.x, d4.y, d4.z),
                          0.01f, vol.g.tmax, 0x3u);
    }
    template <class W>
    __device__ __forceinline__ void finish(const W& w, uint32_t out) const {
        const HitRec& h = w.best;
        hits.thit[out] = make_float4(h.t, h.b1, h.b2, __uint_as_float(h.inst));
        hits.prim[out] = h.prim | (h.back ? 0x80000000u : 0u);
    }
};

struct BatchShadowJob {
    const ShadowQueue q;
    BatchTables bt;
    float4* rays;
    uint32_t* prim;

    template <class W>
    __device__ __forceinline__ bool start(W& w, const DeviceScene& sc, uint32_t id, uint32_t* out) const {
        *out = id;
        float4 p = q.pos[id];
        uint32_t v = __float_as_uint(p.w);
        if (v >= bt.nvol) {
            raise_error(bt.err, DEV_BAD_INDEX);
            v = 0;
        }
        const BatchVolume& vol = bt.vols[v];
        return w.start_at(sc, W::kWide ? vol.wroot : vol.root, f3(p.x, p.y, p.z),
                          f3(vol.L.dir[0], vol.L.dir[1], vol.L.dir[2]), 0.1f, 10000.0f, 0xFFu);
    }
    template <class W>
    __device__ __forceinline__ void finish(const W& w, uint32_t id) const {
        uint32_t idx = q.idx[id];
        if (w.best.inst != kNoHit) {
            prim[idx] |= 1u << 30;
            return;
        }
        float4 sun = q.sun[id];
        float4 rec = rays[idx];
        float3 c = (f3(rec.x, rec.y, rec.z) + f3(sun.x, sun.y, sun.z)) * sun.w;
        rays[idx] = make_float4(c.x, c.y, c.z, rec.w);
    }
};

template <class Stack, template <bool, class> class Walker>
__global__ void __launch_bounds__(kPersistThreads, Walker<false, Stack>::kMinBlocks) k_batch_primary(DeviceScene arena, BatchPrimaryJob job,
                                                                   uint32_t total, uint32_t* counter, int stack_cap,
                                                                   int split, WalkKnobs knobs) {
    persistent_walk<false, Stack, Walker>(arena, job, total, counter, stack_cap, split, knobs, job.bt.err);
}

template <class Stack, template <bool, class> class Walker>
__global__ void __launch_bounds__(kPersistThreads, Walker<false, Stack>::kMinBlocks) k_batch_shadow(DeviceScene arena, BatchShadowJob job,
                                                                  const uint32_t* qcount, uint32_t* counter,
                                                                  int stack_cap, int split, WalkKnobs knobs) {
    persistent_walk<true, Stack, Walker>(arena, job, *qcount, counter, stack_cap, split, knobs, job.bt.err);
}

// Batched shading, pass 1 (k_shade_classify with the record's volume).
__global__ void __launch_bounds__(128) k_batch_classify(BatchTables bt, uint32_t total, WaveHits hits,
                                                        float4* rays_out, uint32_t* front_count) {
    const uint32_t i = bt.first + blockIdx.x * blockDim.x + threadIdx.x;
    bool is_front = false;
    if (i < bt.first + total) {
        const float4 th = hits.thit[i];
        const uint32_t pb = hits.prim[i];
        const uint32_t inst = __float_as_uint(th.w);
        const bool back = (pb >> 31) != 0;
        if (inst == kNoHit) {
            const BatchVolume& vol = bt.vols[batch_volume(bt, i)];
            rays_out[i] = make_float4(vol.L.sky[0], vol.L.sky[1], vol.L.sky[2], -1.0f);
        } else if (back) {
            rays_out[i] = make_float4(0.0f, 0.0f, 0.0f, th.x * 0.80f);
        } else {
            is_front = true;
        }
    }
    const uint32_t k = warp_append(is_front, front_count);
    if (is_front) hits.front[k] = i;
}

// Batched shading, pass 2 (k_shade_front with the volume's scene, grid,
// light, states and atlas; the shadow-queue entry carries the volume).
// Eight resident blocks per SM, like k_shade_front: the 48-volume batch
// update 30.4 -> 29.9 ms against six.
__global__ void __launch_bounds__(128, 8) k_batch_shade_front(BatchTables bt, WaveHits hits,
                                                              const uint32_t* front_count, float4* rays_out,
                                                              ShadowQueue q) {
    const uint32_t n = *front_count;
    if (blockIdx.x * blockDim.x >= n) return;  // whole block
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    bool enqueue = false;
    SurfaceShade s;
    uint32_t i = 0, v = 0;
    if (k < n) {
        i = hits.front[k];
        v = batch_volume(bt, i);
        const BatchVolume& vol = bt.vols[v];
        const uint32_t R = vol.g.rays;
        const uint32_t local = i - __ldg(bt.ray_base + v);
        const uint32_t slot = local / R, ray = local - slot * R;
        const float4 th = hits.thit[i];
        const uint32_t inst = __float_as_uint(th.w), prim = hits.prim[i] & 0x0fffffffu;
        const float4 d4 = __ldg(bt.dirs + vol.dir_base + ray);
        const float3 d = f3(d4.x, d4.y, d4.z);
        const float3 o = probe_origin_exact(vol.g, slot);
        const bool half = vol.fp16 != 0;
        AtlasView<ColorTexDyn, DepthTexDyn> at{{vol.color, half}, {vol.depth, half}};
        enqueue = shade_surface(vol.sc, vol.g, vol.L, vol.states, at, o, d, th.x, th.y, th.z, inst, prim, &s, bt.err);
        rays_out[i] = make_float4(s.base.x, s.base.y, s.base.z, th.x);
    }
    const uint32_t qk = warp_append(enqueue, q.count);
    if (enqueue) {
        q.idx[qk] = i;
        q.pos[qk] = make_float4(s.position.x, s.position.y, s.position.z, __uint_as_float(v));
        q.sun[qk] = make_float4(s.sun.x, s.sun.y, s.sun.z, s.fade);
    }
}

uint32_t persistent_blocks(const void* kernel, size_t smem, uint32_t cap_per_sm = 0) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kPersistThreads, smem);
    if (per <= 0) per = 1;
    if (cap_per_sm > 0 && (uint32_t)per > cap_per_sm) per = (int)cap_per_sm;
    return (uint32_t)(sms * per);
}

}  // namespace

namespace {

template <class Stack, template <bool, class> class Walker>
cudaError_t wavefront_kernels(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L,
                              const uint32_t* probe_list, uint32_t total, const float4* dirs, const uint32_t* states,
                              const void* color, const void* depth, bool fp16_atlas, WaveHits hits, ShadowQueue q,
                              uint32_t* counters, float4* rays_out, ddgi_hit* hits_out, int stack_cap, int split,
                              uint32_t* err, cudaStream_t st, cudaEvent_t after_primary, const uint32_t* dev_count,
                              const TraceTuning& tune, const PrimaryJob& pj) {
    const size_t smem = (size_t)split * kPersistThreads * sizeof(int);
    const WalkKnobs knobs = walk_knobs(tune);
    k_primary<Stack, Walker><<<persistent_blocks((const void*)k_primary<Stack, Walker>, smem, tune.ctas_per_sm),
                               kPersistThreads, smem, st>>>(sc, pj, counters, stack_cap, split, knobs, err);
    if (after_primary) cudaEventRecord(after_primary, st);
    ShadowQueue qq = q;
    qq.count = counters + 1;
    uint32_t blocks = (total + 127) / 128;
    k_shade_classify<<<blocks, 128, 0, st>>>(g, L, total, hits, rays_out, hits_out, counters + 3, dev_count);
    if (fp16_atlas) {
        AtlasView<ColorTexF16, DepthTexF16> at{{static_cast<const uint2*>(color)},
                                               {static_cast<const uint32_t*>(depth)}};
        k_shade_front<<<blocks, 128, 0, st>>>(sc, g, L, probe_list, dirs, states, at, hits, counters + 3, rays_out, qq,
                                              err);
    } else {
        AtlasView<ColorTexF32, DepthTexF32> at{{static_cast<const float4*>(color)},
                                               {static_cast<const float2*>(depth)}};
        k_shade_front<<<blocks, 128, 0, st>>>(sc, g, L, probe_list, dirs, states, at, hits, counters + 3, rays_out, qq,
                                              err);
    }
    ShadowJob sj{qq, make_float3(L.dir[0], L.dir[1], L.dir[2]), rays_out, hits.prim, 0};
    k_shadow<Stack, Walker><<<persistent_blocks((const void*)k_shadow<Stack, Walker>, smem, tune.ctas_per_sm),
                              kPersistThreads, smem, st>>>(sc, sj, counters + 1, counters + 2, stack_cap, split, knobs,
                                                           err);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_wavefront(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L,
                             const uint32_t* probe_list, uint32_t nprobes, const float4* dirs,
                             const uint32_t* ray_order, const uint32_t* states, const void* color, const void* depth,
                             bool fp16_atlas, WaveHits hits, ShadowQueue q, uint32_t* counters, float4* rays_out,
                             ddgi_hit* hits_out, int stack_cap, int wstack_cap, uint32_t* err, cudaStream_t st,
                             cudaEvent_t after_primary, const uint32_t* dev_count, const TraceTuning& tune,
                             const uint32_t* perm) {
    uint32_t total = nprobes * g.rays;
    if (total == 0) return cudaSuccess;
    // counters[0]: primary work, [1]: shadow queue length, [2]: shadow work, [3]: front-hit queue length
    cudaError_t e = cudaMemsetAsync(counters, 0, 4 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    const uint32_t rpw = grouped_rays_per_warp(tune.rays_per_warp, g.rays);
    // the grouped order covers all probes in perm order: no list, no device count
    const uint32_t* pm = (perm && !probe_list && !dev_count && rpw != 0u) ? perm : nullptr;
    PrimaryJob pj{g, probe_list, dirs, ray_order, hits, total, dev_count, pm, rpw, nprobes};
    const bool wide = tune.wide && sc.wnodes && sc.winstances && wstack_cap > 0;
    const int cap = wide ? wstack_cap : stack_cap;
    const bool split = !(tune.split == 0 || (int)tune.split >= cap);
    const int sp = split ? (int)tune.split : cap;
#define DDGI_WAVE(STACK, WALKER)                                                                                       \
    return wavefront_kernels<STACK, WALKER>(sc, g, L, probe_list, total, dirs, states, color, depth, fp16_atlas, hits, \
                                            q, counters, rays_out, hits_out, cap, sp, err, st, after_primary,         \
                                            dev_count, tune, pj)
    if (wide) {
        if (split) DDGI_WAVE(SplitStack, WideWalker);
        DDGI_WAVE(SmemStack, WideWalker);
    }
    if (split) DDGI_WAVE(SplitStack, WarpWalker);
    DDGI_WAVE(SmemStack, WarpWalker);
#undef DDGI_WAVE
}

namespace {

template <class Stack, template <bool, class> class Walker>
cudaError_t batch_trace_kernels(const DeviceScene& arena, const BatchTables& bt, uint32_t total, WaveHits hits,
                                ShadowQueue q, uint32_t* counters, float4* rays_out, int stack_cap, int split,
                                const TraceTuning& tune, cudaStream_t st, cudaEvent_t after_primary,
                                cudaEvent_t after_shade) {
    const size_t smem = (size_t)split * kPersistThreads * sizeof(int);
    const WalkKnobs knobs = walk_knobs(tune);
    BatchPrimaryJob pj{bt, hits};
    k_batch_primary<Stack, Walker>
        <<<persistent_blocks((const void*)k_batch_primary<Stack, Walker>, smem, tune.ctas_per_sm), kPersistThreads,
           smem, st>>>(arena, pj, total, counters, stack_cap, split, knobs);
    if (after_primary) cudaEventRecord(after_primary, st);
    ShadowQueue qq = q;
    qq.count = counters + 1;
    k_batch_classify<<<(total + 127) / 128, 128, 0, st>>>(bt, total, hits, rays_out, counters + 3);
    k_batch_shade_front<<<(total + 127) / 128, 128, 0, st>>>(bt, hits, counters + 3, rays_out, qq);
    if (after_shade) cudaEventRecord(after_shade, st);
    BatchShadowJob sj{qq, bt, rays_out, hits.prim};
    k_batch_shadow<Stack, Walker>
        <<<persistent_blocks((const void*)k_batch_shadow<Stack, Walker>, smem, tune.ctas_per_sm), kPersistThreads,
           smem, st>>>(arena, sj, counters + 1, counters + 2, stack_cap, split, knobs);
    return cudaGetLastError();
}

}  // namespace

// counters[0..3] (primary work, shadow queue length, shadow work, front-hit
// queue length) must be zero when the launch sequence starts.
cudaError_t launch_batch_trace(const DeviceScene& arena, const BatchTables& bt, uint32_t total, WaveHits hits,
                               ShadowQueue q, uint32_t* counters, float4* rays_out, int stack_cap, int wstack_cap,
                               const TraceTuning& tune, cudaStream_t st, cudaEvent_t after_primary,
                               cudaEvent_t after_shade) {
    if (total == 0) return cudaSuccess;
    const bool wide = tune.wide && arena.wnodes && arena.winstances && wstack_cap > 0;
    const int cap = wide ? wstack_cap : stack_cap;
    const bool split = !(tune.split == 0 || (int)tune.split >= cap);
    const int sp = split ? (int)tune.split : cap;
#define DDGI_BATCH(STACK, WALKER)                                                                            \
    return batch_trace_kernels<STACK, WALKER>(arena, bt, total, hits, q, counters, rays_out, cap, sp, tune, \
                                              st, after_primary, after_shade)
    if (wide) {
        if (split) DDGI_BATCH(SplitStack, WideWalker);
        DDGI_BATCH(SmemStack, WideWalker);
    }
    if (split) DDGI_BATCH(SplitStack, WarpWalker);
    DDGI_BATCH(SmemStack, WarpWalker);
#undef DDGI_BATCH
}

// Probe classification of all P probes into `states`.  `dirs` holds the
// kInitRays init directions; back/near are P-entry scratch arrays.
cudaError_t launch_init_probes(const DeviceScene& sc, const DeviceGrid& g, const float4* dirs, uint32_t P,
                               uint32_t* back, uint32_t* near, uint32_t* states, uint32_t* counters, int stack_cap,
                               uint32_t* err, cudaStream_t st) {
    if (P == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(back, 0, sizeof(uint32_t) * P, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(near, 0, sizeof(uint32_t) * P, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    const size_t smem = (size_t)stack_cap * kPersistThreads * sizeof(int);
    InitJob job{g, dirs, 1.5f * g.cell_len, back, near};
    k_init_probes<<<persistent_blocks((const void*)k_init_probes, smem), kPersistThreads, smem, st>>>(
        sc, job, P * kInitRays, counters, stack_cap, err);
    k_init_states<<<(P + 255) / 256, 256, 0, st>>>(P, g.rays, back, near, states);
    return cudaGetLastError();
}

}  // namespace ddgi

// schedule.cu — which probes an update refreshes, decided on the device.
//
// Restates IrradianceProbes::selectProbesToUpdate
// (src/IrradianceProbes.cpp:396-424) without the host readback of the probe
// states: probes are visited cyclically starting at the offset where the
// previous selection stopped; probe `idx` is selected when its state s is
// not 0 (OFF) and (idx + loop) % s == 0, where `loop` counts the wraps of
// the visit past the last probe; with a cap (ProbesPerUpdate) the visit stops
// right after the cap-th selection.  The offset, loop index and the selected
// count live in device memory, so the trace and blend launches that follow
// read the count there.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"

namespace ddgi {

namespace {

constexpr int kThreads = 1024;

// One CTA: the visit in chunks of kThreads positions, a block-wide scan of
// the selection flags per chunk.
__global__ void __launch_bounds__(kThreads) k_select_probes(const uint32_t* __restrict__ states, uint32_t P,
                                                            uint32_t cap, uint32_t* sched, uint32_t* list) {
    __shared__ uint32_t s_cnt[kThreads / 32], s_pre[kThreads / 32];
    __shared__ uint32_t s_total, s_stop;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t off = sched[0] < P ? sched[0] : 0u, loop = sched[1];
    if (tid == 0) s_stop = P;  // visit position of the cap-th selection (P: none)
    uint32_t count = 0;        // selections so far (the same in every thread)
    for (uint32_t base = 0; base < P; base += kThreads) {
        const uint32_t j = base + tid;
        bool pick = false;
        uint32_t idx = 0;
        if (j < P) {
            idx = off + j;
            uint32_t lj = loop;
            if (idx >= P) {  // past the wrap
                idx -= P;
                lj = loop + 1u;
            }
            const uint32_t s = states[idx];
            pick = s != 0u && (idx + lj) % s == 0u;
        }
        const unsigned m = __ballot_sync(0xffffffffu, pick);
        if (lane == 0) s_cnt[warp] = (uint32_t)__popc(m);
        __syncthreads();
        if (warp == 0) {  // scan of the warp counts
            const uint32_t c = s_cnt[lane];
            uint32_t x = c;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= (uint32_t)o) x += y;
            }
            s_pre[lane] = x - c;
            if (lane == 31) s_total = x;
        }
        __syncthreads();
        const uint32_t rank = count + s_pre[warp] + (uint32_t)__popc(m & ((1u << lane) - 1u));
        if (pick && (cap == 0u || rank < cap)) list[rank] = idx;
        if (pick && cap != 0u && rank == cap - 1u) s_stop = j;
        count += s_total;
        __syncthreads();
        if (s_stop < P) break;  // the same in every thread
    }
    if (tid == 0) {
        const uint32_t visited = s_stop < P ? s_stop + 1u : P;
        uint32_t next = off + visited;
        uint32_t wraps = 0;
        if (next >= P) {
            next -= P;
            wraps = 1;
        }
        sched[0] = next;
        sched[1] = loop + wraps;
        sched[2] = cap != 0u && count > cap ? cap : count;
    }
}

// IrradianceProbes::update's hysteresis ramp (src/IrradianceProbes.cpp:462-476)
// for one update, one thread.  sched[4..7] hold the ramp: the hysteresis the
// blend uses (the reference's uniform buffer), the host-side
// GridParameters.hysteresis, TargetHysteresis (float bits) and the probes
// counted since the last step (the reference's static updatedProbes).  The
// host's changes since the last update (cmd) apply first.  Once a full probe
// count has been refreshed, a step either uploads the current value and then
// moves it a tenth of the way towards the target (updateUniforms() comes
// before the increment, so the blend sees the value one step late) or, within
// 0.05 of the target, sets and uploads the target itself; then this update's
// probe count is added.  Float operations are rounded one by one as the
// reference's host code computes them; the 0.05 comparison is in double.
__global__ void k_hysteresis_ramp(uint32_t* sched, RampCmd cmd, const uint32_t* dev_count, uint32_t count,
                                  uint32_t P) {
    float* f = reinterpret_cast<float*>(sched + 4);
    float blended = f[0], h = f[1], target = f[2];
    uint32_t counted = sched[7];
    if (cmd.set & kRampSetBlended) blended = cmd.blended;
    if (cmd.set & kRampSetParam) h = cmd.param;
    if (cmd.set & kRampSetTarget) target = cmd.target;
    if (cmd.set & kRampZeroCount) counted = 0;
    if (counted >= P) {
        if ((double)fabsf(__fsub_rn(h, target)) > 0.05) {
            blended = h;
            h = __fadd_rn(h, __fmul_rn(0.1f, __fsub_rn(target, h)));
        } else if (h != target) {
            h = target;
            blended = h;
        }
        counted -= P;
    }
    counted += dev_count ? *dev_count : count;
    f[0] = blended;
    f[1] = h;
    f[2] = target;
    sched[7] = counted;
}

}  // namespace

cudaError_t launch_hysteresis_ramp(uint32_t* sched, const RampCmd& cmd, const uint32_t* dev_count, uint32_t count,
                                   uint32_t P, cudaStream_t st) {
    k_hysteresis_ramp<<<1, 1, 0, st>>>(sched, cmd, dev_count, count, P);
    return cudaGetLastError();
}

cudaError_t launch_select_probes(const uint32_t* states, uint32_t P, uint32_t max_probes, uint32_t* sched,
                                 uint32_t* list, cudaStream_t st) {
    if (P == 0) return cudaSuccess;
    k_select_probes<<<1, kThreads, 0, st>>>(states, P, max_probes, sched, list);
    return cudaGetLastError();
}

}  // namespace ddgi

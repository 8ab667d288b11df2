// noalloc.cu — the BF16 tensor-core atlas blend for callers that cannot
// allocate device memory.
//
// Some hosts of this library own every byte of device memory themselves: a
// renderer running with a fixed, pre-reserved memory budget, or a frame loop
// where a cudaMalloc/cudaFree (which can synchronise the whole device) would
// stall a frame.  ddgi_blend_records_noalloc serves them: the caller passes
// device pointers to every input and output, and the only other memory the
// blend needs (the ray-direction table, the per-update BF16 weight
// matrices, their row sums and an error word) lives in one file-scope
// __device__ array of fixed size, loaded with this library on every GPU that
// uses it and kept until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "../../include/ddgi.h"
#include "../../include/ddgi_exact.h"
#include "common.cuh"
#include "kernels.h"

using namespace ddgi;

namespace {

// Scratch layout: direction table (1024 x float4 = 16 KB), row sums
// (512 floats in a 4 KB slot), error word (256-byte slot), then the weight
// matrices (at most 2 MB: 16 chunks of 64 rays x 2 parts x 512 rows x 128 B).
constexpr size_t kDirsOff = 0;
constexpr size_t kRowsumOff = 16u << 10;
constexpr size_t kErrOff = kRowsumOff + (4u << 10);
constexpr size_t kWeightsOff = kErrOff + 256;
constexpr size_t kWeightsMax = 2u << 20;
constexpr size_t kScratchBytes = kWeightsOff + kWeightsMax;

__device__ __align__(256) static unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch array in the caller's current context.
// The address belongs to the CUDA context that loaded this library's module
// on the current device, so it is looked up on every call instead of being
// remembered: a context made again after cudaDeviceReset, or another device,
// has its own copy of the array at its own address.  The lookup is a host
// call with no stream work, cheap next to the synchronisation at the end of
// the call.
ddgi_status scratch_address(void** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return DDGI_ERR_CUDA;
    }
    *out = p;
    return DDGI_OK;
}

bool grid_ok(const ddgi_grid_desc* g) {
    for (int k = 0; k < 3; ++k) {
        if (g->resolution[k] < 2) return false;
        if (!std::isfinite(g->extent_min[k]) || !std::isfinite(g->extent_max[k]) ||
            !(g->extent_max[k] > g->extent_min[k]))
            return false;
    }
    if (g->rays_per_probe < 1 || g->rays_per_probe > DDGI_MAX_RAYS_PER_PROBE) return false;
    if (g->color_res < 3 || g->depth_res < 3) return false;
    if (!std::isfinite(g->hysteresis) || !std::isfinite(g->depth_sharpness)) return false;
    return true;
}

}  // namespace

extern "C" ddgi_status ddgi_blend_records_noalloc(const ddgi_grid_desc* grid, const float orientation[9],
                                                  const uint32_t* probe_list, uint32_t probe_count,
                                                  const float* records, uint32_t* states, void* color, void* depth,
                                                  float* acc_color, float* acc_depth, ddgi_stream stream) {
    if (!grid || !orientation || !records || !states || !color || !depth || !acc_color || !acc_depth)
        return DDGI_ERR_INVALID_ARGUMENT;
    if (!grid_ok(grid)) return DDGI_ERR_INVALID_ARGUMENT;
    if (!tc_blend_supported(grid->color_res, grid->depth_res)) return DDGI_ERR_UNSUPPORTED;
    if (tc_weight_bytes(grid->rays_per_probe, grid->color_res, grid->depth_res) > kWeightsMax)
        return DDGI_ERR_UNSUPPORTED;  // beyond the fixed scratch: too many rays or texels
    for (int k = 0; k < 9; ++k)
        if (!std::isfinite(orientation[k])) return DDGI_ERR_INVALID_ARGUMENT;
    const uint32_t P = (uint32_t)grid->resolution[0] * (uint32_t)grid->resolution[1] * (uint32_t)grid->resolution[2];
    const uint32_t n = probe_list ? probe_count : P;
    if (n > P) return DDGI_ERR_INVALID_ARGUMENT;
    if (n == 0) return DDGI_OK;

    void* base = nullptr;
    ddgi_status s = scratch_address(&base);
    if (s != DDGI_OK) return s;
    unsigned char* sc = static_cast<unsigned char*>(base);
    float4* dirs = reinterpret_cast<float4*>(sc + kDirsOff);
    float* rowsum = reinterpret_cast<float*>(sc + kRowsumOff);
    uint32_t* err = reinterpret_cast<uint32_t*>(sc + kErrOff);
    uint8_t* weights = reinterpret_cast<uint8_t*>(sc + kWeightsOff);

    // The direction table follows the exact host definition shared with the
    // other entry points; it lives on this call's stack.
    const uint32_t R = grid->rays_per_probe;
    float host_dirs[4 * DDGI_MAX_RAYS_PER_PROBE];
    ddgi_ray_direction_table(orientation, R, host_dirs);

    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    DeviceGrid dg{};
    for (int k = 0; k < 3; ++k) {
        dg.mn[k] = grid->extent_min[k];
        dg.mx[k] = grid->extent_max[k];
        dg.res[k] = grid->resolution[k];
        volatile float diff = grid->extent_max[k] - grid->extent_min[k];
        dg.cell[k] = diff / (float)(grid->resolution[k] - 1);
    }
    {
        volatile float a = dg.cell[0] * dg.cell[0];
        volatile float b = dg.cell[1] * dg.cell[1];
        volatile float c = dg.cell[2] * dg.cell[2];
        volatile float t = a + b;
        t = t + c;
        dg.cell_len = std::sqrt((float)t);
    }
    dg.rays = R;
    dg.color_res = grid->color_res;
    dg.depth_res = grid->depth_res;
    dg.sharp = grid->depth_sharpness;
    dg.hyst = grid->hysteresis;
    dg.bias = grid->shadow_bias;
    dg.color_w = grid->color_res * grid->resolution[0] * grid->resolution[1];
    dg.color_h = grid->color_res * grid->resolution[2];
    dg.depth_w = grid->depth_res * grid->resolution[0] * grid->resolution[1];
    dg.depth_h = grid->depth_res * grid->resolution[2];
    dg.quant = 0;

    // The scratch keeps the previous call's contents: the error word must
    // start at zero; the table, weights and row sums are rewritten in full.
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dirs, host_dirs, sizeof(float4) * R, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = launch_blend_tc(dg, probe_list, n, reinterpret_cast<const float4*>(records), dirs, weights, rowsum, states,
                            color, depth, reinterpret_cast<float4*>(acc_color), reinterpret_cast<float2*>(acc_depth),
                            err, st);
    uint32_t herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return DDGI_ERR_CUDA;
    }
    return herr ? DDGI_ERR_DEVICE : DDGI_OK;
}

// gbuild.h — surface-area-heuristic trees built on the GPU (see gbuild.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace ddgi {

// Builds binary trees over several primitive sets at once on the device and
// writes them in the layout of sah.cu / sbvh.cu (depth-first nodes, leaf
// references into a per-set leaf order).
//
// Triangle sets (build_triangles): the spatial-split builder of sbvh.cu —
// binned object splits, and spatial splits where the object split's
// children overlap by more than `alpha` of the set root's surface area.
// Box sets (build_boxes): the object splits of sah.cu, binned above
// kSweepMax primitives and by an exact sweep below.  Every decision uses the
// host builders' arithmetic (same bins, same separately rounded operations,
// the reference splits of tri_split.h in float interval arithmetic), and
// partitions keep the references' order, so a set's tree is the host
// builder's tree.
class GpuTreeBuilder {
  public:
    GpuTreeBuilder() = default;
    ~GpuTreeBuilder();
    GpuTreeBuilder(const GpuTreeBuilder&) = delete;
    GpuTreeBuilder& operator=(const GpuTreeBuilder&) = delete;

    // tris: 9 floats (v0, v1, v2) per triangle, the sets' triangles one set
    // after the other (counts[s] triangles for set s).  Device pointers.
    cudaError_t build_triangles(const float* tris, const std::vector<uint32_t>& counts, int leaf_max, float alpha,
                                uint32_t* err, cudaStream_t st);
    // One set of n boxes (xyz of lo/hi).  Device pointers.
    cudaError_t build_boxes(const float4* lo, const float4* hi, uint32_t n, int leaf_max, uint32_t* err,
                            cudaStream_t st);

    // After a build: per set, inner nodes written (max(n - 1, 1) for box
    // sets; 0 for an empty set), leaf references, inner nodes on the longest
    // root-to-leaf path.
    const std::vector<uint32_t>& node_counts() const { return nodes_; }
    const std::vector<uint32_t>& ref_counts() const { return refs_; }
    const std::vector<uint32_t>& depths() const { return depth_; }
    // Levels processed and device milliseconds of the last build (events on
    // the build stream).
    uint32_t levels() const { return levels_; }
    float build_ms() const { return build_ms_; }

    // Set s's tree at nodes[node_base[s] ...] (references to inner nodes
    // node_base[s] + index, to leaves prim_base[s] + position) and its leaf
    // order at order[order_base[s] ...] (set-local primitive indices).
    // Host arrays of one entry per set.
    cudaError_t write(BvhNode* nodes, const std::vector<int>& node_base, const std::vector<int>& prim_base,
                      uint32_t* order, const std::vector<uint32_t>& order_base, cudaStream_t st);

  private:
    cudaError_t run(bool triangles, const float* tris, const float4* lo, const float4* hi,
                    const std::vector<uint32_t>& counts, int leaf_max, float alpha, uint32_t* err, cudaStream_t st);
    cudaError_t attempt(bool triangles, const float* tris, const float4* lo, const float4* hi,
                        const std::vector<uint32_t>& counts, int leaf_max, float alpha, uint32_t* err,
                        cudaStream_t st, size_t cap, bool* overflow);
    void release();

    // device state of the last build
    void* mem_ = nullptr;
    size_t mem_bytes_ = 0;
    struct Layout {
        size_t nodes, refs0, refs1, pool, chunks0, chunks1, chunk_cnt, chunk_off, bins0, bins1, ctr, sets, levels,
            sweep0, sweep1;
        size_t cap, cap_chunks, cap_bins;
    } L_{};
    std::vector<uint32_t> level_begin_;  // node ids of each level (levels + 1 entries)
    std::vector<uint32_t> set_root_;     // root node id per set (~0u: fewer than 2 primitives)
    std::vector<uint32_t> set_n_, set_off_;
    std::vector<uint32_t> nodes_, refs_, depth_;
    const float* tris_ = nullptr;
    const float4* box_lo_ = nullptr;
    const float4* box_hi_ = nullptr;
    bool triangles_ = true;
    uint32_t levels_ = 0;
    float build_ms_ = 0.0f;
};

// Triangles of one mesh as 9 floats each (v0, v1, v2), the input of
// GpuTreeBuilder::build_triangles: out[9 t ...] for t < ntri.
cudaError_t gather_triangle_soup(const float4* pos, const uint32_t* indices, uint32_t vbase, uint32_t ibase,
                                 uint32_t ntri, float* out, cudaStream_t st);

}  // namespace ddgi

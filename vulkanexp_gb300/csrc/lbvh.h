// lbvh.h — GPU LBVH construction entry points (see lbvh.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace ddgi {

// Device scratch needed by lbvh_build for n primitives.
size_t lbvh_scratch_bytes(uint32_t n);

// Builds a tree over n primitive boxes (float4 lo/hi, xyz used).  Writes
// max(n - 1, 1) nodes at nodes[node_base ...]; leaf references point at
// prim_base + sorted position.  sorted_ids[s] = original primitive of sorted
// position s.  Root = node_base.
cudaError_t lbvh_build(const float4* prim_lo, const float4* prim_hi, uint32_t n, int leaf_max, BvhNode* nodes,
                       int node_base, int prim_base, uint32_t* sorted_ids, void* scratch, uint32_t* err, uint32_t* depth,
                       cudaStream_t st);

// Bottom-level build of one mesh: triangle boxes from the vertex positions and
// indices, the tree, and the triangles gathered in leaf order at
// tris[tri_base ...].  box_lo/box_hi/sorted_ids hold ntri entries of scratch.
cudaError_t build_mesh_blas(const float4* pos, const uint32_t* indices, uint32_t vbase, uint32_t vcount,
                            uint32_t ibase, uint32_t ntri, int leaf_max, BvhNode* nodes, int node_base, BvhTri* tris,
                            int tri_base, float4* box_lo, float4* box_hi, uint32_t* sorted_ids, void* scratch,
                            uint32_t* err, uint32_t* depth, cudaStream_t st);

// Triangles of one mesh (ntri of them) gathered in leaf order
// (sorted_ids[s] = triangle of leaf position s) at tris[0, nref), for a tree
// built elsewhere; a triangle may fill several positions.
cudaError_t gather_mesh_tris(const float4* pos, const uint32_t* indices, uint32_t vbase, uint32_t vcount,
                             uint32_t ibase, uint32_t ntri, uint32_t nref, const uint32_t* sorted_ids, BvhTri* tris,
                             cudaStream_t st);

// Refit of a top-level tree whose topology is kept: new boxes for its n
// leaf slots (leaf order); leaf_parent[s] / node_parent[k] = parent node
// (relative to node_base) << 1 | side, 0xFFFFFFFF for the root; flags
// (n - 1 entries) and sub_lo/sub_hi (2 (n - 1) entries) are scratch.
cudaError_t lbvh_refit_top(BvhNode* nodes, int node_base, const float4* leaf_lo, const float4* leaf_hi, uint32_t n,
                           const uint32_t* leaf_parent, const uint32_t* node_parent, uint32_t* flags, float4* sub_lo,
                           float4* sub_hi, uint32_t* err, cudaStream_t st);

}  // namespace ddgi

// sah.h — surface-area-heuristic trees built on the host (see sah.cu).
#pragma once

#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace ddgi {

// Binary tree over n primitive boxes (xyz of lo/hi) split by the surface-area
// heuristic; every subtree of at most leaf_max primitives becomes a leaf.
// Writes max(n - 1, 1) nodes: the tree depth first from nodes[0] (inner
// references node_base + index, leaf references prim_base + leaf position,
// every box enlarged like the GPU builder's), then never-hit filler nodes.
// order[s] = primitive at leaf position s; *depth = inner nodes on the
// longest root-to-leaf path.  Uses up to `threads` host threads.  Returns
// false when n == 0.
bool sah_build(const float4* lo, const float4* hi, uint32_t n, int leaf_max, int node_base, int prim_base,
               BvhNode* nodes, uint32_t* order, uint32_t* depth, unsigned threads);

// Mesh tree over n triangles (9 floats each: v0, v1, v2) with object splits
// and, where the object split's children overlap by more than alpha of the
// root's surface area, spatial splits (sbvh.cu); alpha <= 0: object splits
// only.  A triangle may be referenced by several leaves: order (resized to
// the reference count) holds the triangle of each leaf position, nodes
// (resized to the inner-node count) the tree depth first, references as in
// sah_build.  Returns false when n == 0.
bool sbvh_build(const float* tris, uint32_t n, int leaf_max, float alpha, int node_base, int prim_base,
                std::vector<BvhNode>& nodes, std::vector<uint32_t>& order, uint32_t* depth, unsigned threads);

// The spatial-split builder's reference split (tri_split.h): the bounds of
// the part of triangle `tri` (9 floats) between slab_lo[axis] and
// slab_hi[axis], widened outwards, intersected with the slab in every axis
// (lo > hi in some axis when the triangle misses it).
void sbvh_clip_box(const float* tri, int axis, const float slab_lo[3], const float slab_hi[3], float out_lo[3],
                   float out_hi[3]);

}  // namespace ddgi

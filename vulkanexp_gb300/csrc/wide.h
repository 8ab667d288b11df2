// wide.h — eight-wide quantised trees collapsed from the binary trees (wide.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace ddgi {

// Appends the wide nodes of the binary tree rooted at bin[root] to `out`
// and returns the wide root (-1 for an empty tree); *levels = wide levels
// on the longest path; *ok is cleared on a malformed reference.
int collapse_wide(const std::vector<BvhNode>& bin, int root, std::vector<WideNode>& out, uint32_t* levels, bool* ok);

// Wide nodes of one scene copied into a batch arena with rebased references.
cudaError_t launch_rebase_wide(const WideNode* src, uint32_t n, uint32_t tlas_start, int node_off, int tri_off,
                               int inst_off, WideNode* dst, cudaStream_t st);

}  // namespace ddgi

// wide.cu — four-wide trees collapsed from the binary LBVH trees.
//
// A wide node is made for the root and for every binary inner node two
// levels below a wide node's binary node: its up-to-four slots are the
// binary node's children, with an inner child replaced by that child's two
// children (the grandchildren), each with the box its parent stores.  Empty
// boxes (the unused side of a one-primitive tree) are dropped.  Boxes are
// copied, not recomputed, so they stay exactly as conservative as the binary
// tree's; leaf references keep their encoding.  Wide nodes of a tree are
// laid out parent before children, siblings together.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "traverse.cuh"
#include "wide.h"

namespace ddgi {

namespace {

struct Slot {
    int ref;
    float lo[3], hi[3];
};

bool box_empty(const float lo[3], const float hi[3]) {
    for (int k = 0; k < 3; ++k)
        if (!(lo[k] <= hi[k])) return true;  // also NaN
    return false;
}

void child_slot(const BvhNode& n, int side, Slot* s) {
    if (side == 0) {
        s->ref = n.d.x;
        s->lo[0] = n.a.x, s->hi[0] = n.a.y, s->lo[1] = n.a.z, s->hi[1] = n.a.w, s->lo[2] = n.c.x, s->hi[2] = n.c.y;
    } else {
        s->ref = n.d.y;
        s->lo[0] = n.b.x, s->hi[0] = n.b.y, s->lo[1] = n.b.z, s->hi[1] = n.b.w, s->lo[2] = n.c.z, s->hi[2] = n.c.w;
    }
}

}  // namespace

int collapse_wide(const std::vector<BvhNode>& bin, int root, std::vector<WideNode>& out, uint32_t* levels,
                  bool* ok) {
    *levels = 0;
    if (root < 0) return -1;
    struct Work {
        int bin, wide;
        uint32_t level;
    };
    std::vector<Work> work;
    const int wroot = (int)out.size();
    out.emplace_back();
    work.push_back({root, wroot, 1});
    while (!work.empty()) {
        Work w = work.back();
        work.pop_back();
        *levels = std::max(*levels, w.level);
        if (w.bin < 0 || (size_t)w.bin >= bin.size()) {
            *ok = false;
            return wroot;
        }
        Slot slots[4];
        int ns = 0;
        const BvhNode& b = bin[(size_t)w.bin];
        for (int side = 0; side < 2; ++side) {
            Slot c;
            child_slot(b, side, &c);
            if (box_empty(c.lo, c.hi)) continue;
            if (c.ref >= 0) {
                if ((size_t)c.ref >= bin.size()) {
                    *ok = false;
                    return wroot;
                }
                for (int s2 = 0; s2 < 2; ++s2) {
                    Slot g;
                    child_slot(bin[(size_t)c.ref], s2, &g);
                    if (!box_empty(g.lo, g.hi)) slots[ns++] = g;
                }
            } else {
                slots[ns++] = c;
            }
        }
        WideNode n;
        float* lo[3] = {&n.lox.x, &n.loy.x, &n.loz.x};
        float* hi[3] = {&n.hix.x, &n.hiy.x, &n.hiz.x};
        int refs[4] = {kNone, kNone, kNone, kNone};
        for (int k = 0; k < 4; ++k)
            for (int a = 0; a < 3; ++a) {
                lo[a][k] = INFINITY;
                hi[a][k] = -INFINITY;
            }
        for (int k = 0; k < ns; ++k) {
            for (int a = 0; a < 3; ++a) {
                lo[a][k] = slots[k].lo[a];
                hi[a][k] = slots[k].hi[a];
            }
            if (slots[k].ref >= 0) {
                const int nw = (int)out.size();
                out.emplace_back();
                work.push_back({slots[k].ref, nw, w.level + 1});
                refs[k] = nw;
            } else {
                refs[k] = slots[k].ref;
            }
        }
        n.ref = make_int4(refs[0], refs[1], refs[2], refs[3]);
        n.unused = make_int4(0, 0, 0, 0);
        out[(size_t)w.wide] = n;
    }
    return wroot;
}

namespace {

// Wide-node references moved into a batch arena: inner + node offset,
// mesh-tree leaves + triangle offset, top-level leaves (wide index >=
// tlas_start) + instance offset; empty slots stay empty.
__global__ void k_rebase_wide(const WideNode* __restrict__ src, uint32_t n, uint32_t tlas_start, int node_off,
                              int tri_off, int inst_off, WideNode* __restrict__ dst) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    WideNode w = src[i];
    const int prim_off = i >= tlas_start ? inst_off : tri_off;
    int r[4] = {w.ref.x, w.ref.y, w.ref.z, w.ref.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (r[k] == kNone) continue;
        if (r[k] >= 0) {
            r[k] += node_off;
        } else {
            int first = (~r[k]) >> 3, cnt = (~r[k]) & 7;
            r[k] = ~(((first + prim_off) << 3) | cnt);
        }
    }
    w.ref = make_int4(r[0], r[1], r[2], r[3]);
    dst[i] = w;
}

}  // namespace

cudaError_t launch_rebase_wide(const WideNode* src, uint32_t n, uint32_t tlas_start, int node_off, int tri_off,
                               int inst_off, WideNode* dst, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_rebase_wide<<<(n + 255) / 256, 256, 0, st>>>(src, n, tlas_start, node_off, tri_off, inst_off, dst);
    return cudaGetLastError();
}

}  // namespace ddgi

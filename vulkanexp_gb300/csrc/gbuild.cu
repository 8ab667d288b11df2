// gbuild.cu — surface-area-heuristic trees built on the GPU.
//
// The device counterpart of the host builders sah.cu (top level over
// instance boxes) and sbvh.cu (mesh trees with spatial splits).  The
// reference asks the driver for static bottom-level structures built for
// trace speed (VK_BUILD_ACCELERATION_STRUCTURE_PREFER_FAST_TRACE_BIT_KHR,
// src/Renderer.cpp:334); these kernels build them on the GPU with the host
// builders' algorithm, breadth first: every level of all sets' trees is one
// round of passes over the level's nodes, cut into chunks of kChunk
// references (one block each).
//
//   k_bin_object   centroids binned into kBins slabs per axis (counts and
//                  boxes, shared-memory atomics, merged into the node's
//                  global bins); the node's last block picks the object
//                  split (a warp: one lane per plane, prefix/suffix unions
//                  by shuffles, the lowest cost with the lowest axis and
//                  plane on ties, as the host's strict-less scan picks it)
//                  and whether its children overlap enough for spatial
//                  splits (Stich, Friedrich & Dietrich 2009);
//   k_bin_spatial  for those nodes: references binned by their extent,
//                  chopped at the bin planes (the reference splits of
//                  tri_split.h, one plane per thread); the last block
//                  keeps a spatial plane only if its cost is lower;
//   k_count        each chunk counts the references going left and right
//                  (both the spatial and the object partition); the node's
//                  last block scans the chunks, falls back from a spatial
//                  split with an empty side, and allocates the children:
//                  leaves (at most leaf_max references) in the leaf pool,
//                  inner children as next-level nodes with their chunks;
//   k_scatter      each chunk writes its references to the children in
//                  their order (ballot ranks), straddling triangles clipped
//                  to each side, and reduces the children's boxes and
//                  centroid bounds.
//
// The box sets' nodes of at most kSweepMax references are split by k_sweep
// instead (one block per node): references sorted by centroid along each
// axis (ties by primitive), the cost at every position from prefix and
// suffix box scans, the lowest cost with the most balanced position, then
// the earliest axis and position, exactly as sah.cu's sweep.
//
// Every decision uses the host builders' arithmetic: float operations
// separately rounded in the host's order (__fadd_rn / __fmul_rn, no
// contraction), unions by min/max (exact in any order; ordered-integer
// atomics), the reference split of tri_split.h shared with the host, and
// partitions that keep the references' order, so a set's tree equals the
// host builder's tree node for node.  A finishing pass numbers each tree
// depth first (subtree sizes bottom-up, positions top-down), as the host
// writers do, and writes the nodes with the boxes enlarged by the same
// formula.
//
// The level passes need buffers sized before the build; spatial splits add
// references, so a build that runs out of them (an overflow word set
// instead of a write) is started again with twice the capacity.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gbuild.h"
#include "kernels.h"
#include "traverse.cuh"
#include "tri_split.h"

namespace ddgi {

namespace {

constexpr int kBins = 32;
constexpr uint32_t kChunk = 1024;  // references per block of a level pass
constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr uint32_t kMaxSplitDepth = 40;  // sbvh.cu: no spatial split below this depth
constexpr uint32_t kSweepMax = 4096;     // sah.cu: exact sweep at or below this many references
constexpr int kSweepThreads = 512;
constexpr int kObjWords = 7;   // count, lo keys xyz, hi keys xyz
constexpr int kSpWords = 8;    // enter, leave, lo keys xyz, hi keys xyz
constexpr int kBinWords = 3 * kBins * (kObjWords + kSpWords);
constexpr uint32_t kKeyPosInf = 0xFF800000u, kKeyNegInf = 0x007FFFFFu;

enum Kind : int32_t { kObject = 0, kSpatial = 1, kHalve = 2 };
enum Ctr : int { kCtrNodes = 0, kCtrRefs, kCtrChunks, kCtrBins, kCtrPool, kCtrOverflow, kCtrSweep, kCtrs = 8 };

struct Ref {
    float4 lo, hi;  // box; lo.w holds the primitive (global index) as bits
};

// One node of the trees being built (ids are global over all sets).
struct BNode {
    uint32_t nb[6];     // bounds of the node's references (ordered keys: lo xyz, hi xyz)
    uint32_t cb[6];     // bounds of their centroids
    uint32_t lb[2][6];  // boxes of leaf children
    uint32_t begin, count, set, depth;
    uint32_t chunk_first, nchunks;
    int32_t bins;     // global bin slot of a node of several chunks (-1: one chunk)
    uint32_t ctr[3];  // blocks finished: object bins, spatial bins, counts
    int32_t kind, oax, oplane, sax;
    float ocost, splane;
    uint32_t spatial;  // spatial splits evaluated
    int32_t child[2];  // inner child id, -1: leaf
    uint32_t leaf_first[2], leaf_cnt[2];
    uint32_t sub_nodes, sub_refs, dfs, leaf_base;
};

struct DBox {
    float lo[3], hi[3];
};

__host__ __device__ __forceinline__ uint32_t fkey(float f) {
#ifdef __CUDA_ARCH__
    const uint32_t u = __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float kval(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

__device__ __forceinline__ void box_reset(DBox& b) {
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = INFINITY;
        b.hi[k] = -INFINITY;
    }
}
__device__ __forceinline__ void box_grow(DBox& b, const DBox& o) {
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = fminf(b.lo[k], o.lo[k]);
        b.hi[k] = fmaxf(b.hi[k], o.hi[k]);
    }
}
__device__ __forceinline__ bool box_empty(const DBox& b) {
    return !(b.lo[0] <= b.hi[0] && b.lo[1] <= b.hi[1] && b.lo[2] <= b.hi[2]);
}
// Half the surface area, 0 for an empty or degenerate box: the host's
// dx * dy + dy * dz + dz * dx, each operation rounded separately.
__device__ __forceinline__ float half_area(const DBox& b) {
    const float dx = __fsub_rn(b.hi[0], b.lo[0]), dy = __fsub_rn(b.hi[1], b.lo[1]), dz = __fsub_rn(b.hi[2], b.lo[2]);
    if (!(dx >= 0.0f && dy >= 0.0f && dz >= 0.0f)) return 0.0f;
    const float a = __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
    return a == a ? a : 0.0f;
}
__device__ __forceinline__ float centroid(const DBox& b, int k) {
    const float c = __fmul_rn(0.5f, __fadd_rn(b.lo[k], b.hi[k]));
    return c == c ? c : -INFINITY;
}
__device__ __forceinline__ int bin_of(float x, float lo, float scale) {
    const float f = __fmul_rn(__fsub_rn(x, lo), scale);
    if (!(f >= 0.0f)) return 0;
    return f < (float)(kBins - 1) ? __float2int_rz(f) : kBins - 1;
}
__device__ __forceinline__ DBox ref_box(const Ref& r) {
    DBox b;
    b.lo[0] = r.lo.x, b.lo[1] = r.lo.y, b.lo[2] = r.lo.z;
    b.hi[0] = r.hi.x, b.hi[1] = r.hi.y, b.hi[2] = r.hi.z;
    return b;
}
__device__ __forceinline__ Ref make_ref(const DBox& b, uint32_t prim) {
    Ref r;
    r.lo = make_float4(b.lo[0], b.lo[1], b.lo[2], __uint_as_float(prim));
    r.hi = make_float4(b.hi[0], b.hi[1], b.hi[2], 0.0f);
    return r;
}
__device__ __forceinline__ uint32_t ref_prim(const Ref& r) { return __float_as_uint(r.lo.w); }
__device__ __forceinline__ DBox key_box(const uint32_t* k) {
    DBox b;
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = kval(k[a]);
        b.hi[a] = kval(k[3 + a]);
    }
    return b;
}

__device__ __forceinline__ void load_tri(const float* __restrict__ tri, float t[9]) {
    for (int i = 0; i < 9; ++i) t[i] = __ldg(tri + i);
}
__device__ __forceinline__ void box_clip(DBox& b, const DBox& o) {
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = fmaxf(b.lo[k], o.lo[k]);
        b.hi[k] = fminf(b.hi[k], o.hi[k]);
    }
}

// The host writers' box enlargement, each operation rounded separately.
__device__ __forceinline__ void enlarge_exact(DBox& b) {
    for (int k = 0; k < 3; ++k) {
        const float e = __fadd_rn(__fadd_rn(__fmul_rn(__fsub_rn(b.hi[k], b.lo[k]), 1e-5f),
                                            __fmul_rn(__fadd_rn(fabsf(b.lo[k]), fabsf(b.hi[k])), 1e-6f)),
                                  1e-7f);
        b.lo[k] = __fsub_rn(b.lo[k], e);
        b.hi[k] = __fadd_rn(b.hi[k], e);
    }
}

__device__ __forceinline__ DBox shfl_box(const DBox& b, int src) {
    DBox r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = __shfl_sync(0xFFFFFFFFu, b.lo[k], src);
        r.hi[k] = __shfl_sync(0xFFFFFFFFu, b.hi[k], src);
    }
    return r;
}
__device__ __forceinline__ DBox shfl_up_box(const DBox& b, int d) {
    DBox r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = __shfl_up_sync(0xFFFFFFFFu, b.lo[k], d);
        r.hi[k] = __shfl_up_sync(0xFFFFFFFFu, b.hi[k], d);
    }
    return r;
}
__device__ __forceinline__ DBox shfl_down_box(const DBox& b, int d) {
    DBox r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = __shfl_down_sync(0xFFFFFFFFu, b.lo[k], d);
        r.hi[k] = __shfl_down_sync(0xFFFFFFFFu, b.hi[k], d);
    }
    return r;
}

// Lowest (cost, lane) of the warp: lane of the minimum, the lowest lane on ties.
__device__ __forceinline__ int warp_argmin(float cost, float* best) {
    int lane = threadIdx.x & 31;
    float c = cost;
    int l = lane;
    for (int o = 16; o > 0; o >>= 1) {
        const float oc = __shfl_xor_sync(0xFFFFFFFFu, c, o);
        const int ol = __shfl_xor_sync(0xFFFFFFFFu, l, o);
        if (oc < c || (oc == c && ol < l)) {
            c = oc;
            l = ol;
        }
    }
    *best = c;
    return l;
}

// Bins of a warp's 32 lanes: the union of the bins below the lane
// (exclusive prefix) and of the bins from the lane up (inclusive suffix).
template <class T>
__device__ __forceinline__ void scan_bins(const DBox& b, T cnt_left, T cnt_right, DBox& left, T& nleft, DBox& right,
                                          T& nright) {
    const int lane = threadIdx.x & 31;
    DBox r = b;
    T rc = cnt_right;
    for (int o = 1; o < 32; o <<= 1) {
        const DBox t = shfl_down_box(r, o);
        const T tc = __shfl_down_sync(0xFFFFFFFFu, rc, o);
        if (lane + o < 32) {
            box_grow(r, t);
            rc += tc;
        }
    }
    DBox l = b;
    T lc = cnt_left;
    for (int o = 1; o < 32; o <<= 1) {
        const DBox t = shfl_up_box(l, o);
        const T tc = __shfl_up_sync(0xFFFFFFFFu, lc, o);
        if (lane >= o) {
            box_grow(l, t);
            lc += tc;
        }
    }
    left = shfl_up_box(l, 1);
    nleft = __shfl_up_sync(0xFFFFFFFFu, lc, 1);
    if (lane == 0) {
        box_reset(left);
        nleft = 0;
    }
    right = r;
    nright = rc;
}

struct Pass {
    BNode* nodes;
    const Ref* in;
    Ref* out;
    const uint32_t* chunk_node;  // this level's chunks (node of each)
    uint32_t* chunk_cnt;         // 4 per chunk: spatial left/right, object left/right
    uint32_t* chunk_off;         // 2 per chunk: offsets of the chunk's references in the children
    uint32_t* chunk_out;         // next level's chunks
    uint32_t* bins;              // this level's bin slots
    uint32_t* bins_out;          // next level's
    const uint32_t* sweep_in;    // this level's swept nodes (box sets)
    uint32_t* sweep_out;
    uint32_t* pool;              // leaf references (primitive, global index)
    uint32_t* ctr;
    uint32_t cap_refs, cap_chunks, cap_bins;
    const float* tris;           // triangle sets: 9 floats per primitive; null for box sets
    const uint32_t* set_root;    // root node of each set
    int leaf_max;
    float alpha;
    uint32_t sweep_max;
};

__device__ __forceinline__ void chunk_range(const BNode& N, uint32_t c, uint32_t& p0, uint32_t& p1) {
    p0 = N.begin + (c - N.chunk_first) * kChunk;
    p1 = min(N.begin + N.count, p0 + kChunk);
}

__device__ __forceinline__ void init_bin_words(uint32_t* b, int words) {
    const int nc = words - 6;
    for (int w = 0; w < nc; ++w) b[w] = 0u;
    b[nc] = b[nc + 1] = b[nc + 2] = kKeyPosInf;
    b[nc + 3] = b[nc + 4] = b[nc + 5] = kKeyNegInf;
}

// Adds a block's bins to the node's global bins; true in the node's last
// block, which then holds the merged bins in shared memory.
__device__ bool merge_bins(uint32_t* s, uint32_t* g, int nbins, int words, uint32_t* ctr, uint32_t nblocks,
                           int* s_last) {
    const int nc = words - 6;
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) {
        const uint32_t* b = s + words * i;
        uint32_t* d = g + words * i;
        for (int w = 0; w < nc; ++w)
            if (b[w]) atomicAdd(d + w, b[w]);
        if (b[nc] != kKeyPosInf)
            for (int a = 0; a < 3; ++a) {
                atomicMin(d + nc + a, b[nc + a]);
                atomicMax(d + nc + 3 + a, b[nc + 3 + a]);
            }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) *s_last = atomicAdd(ctr, 1u) == nblocks - 1;
    __syncthreads();
    if (!*s_last) return false;
    __threadfence();
    for (int i = threadIdx.x; i < nbins * words; i += blockDim.x) s[i] = __ldcg(g + i);
    __syncthreads();
    return true;
}

// ---------------------------------------------------------------------------
// Level 0: the roots' references and bounds
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_init_refs(Pass P, Ref* refs, const float4* blo, const float4* bhi) {
    const uint32_t c = blockIdx.x;
    BNode& N = P.nodes[P.chunk_node[c]];
    uint32_t p0, p1;
    chunk_range(N, c, p0, p1);
    DBox nb, cb;
    box_reset(nb);
    box_reset(cb);
    for (uint32_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        DBox b;
        if (P.tris) {
            const float* t = P.tris + 9 * (size_t)p;
            for (int k = 0; k < 3; ++k) {
                b.lo[k] = fminf(fminf(t[k], t[3 + k]), t[6 + k]);
                b.hi[k] = fmaxf(fmaxf(t[k], t[3 + k]), t[6 + k]);
            }
        } else {
            const float4 l = blo[p], h = bhi[p];
            b.lo[0] = l.x, b.lo[1] = l.y, b.lo[2] = l.z;
            b.hi[0] = h.x, b.hi[1] = h.y, b.hi[2] = h.z;
        }
        refs[p] = make_ref(b, p);
        box_grow(nb, b);
        for (int k = 0; k < 3; ++k) {
            const float ce = centroid(b, k);
            if (ce > -INFINITY && ce < INFINITY) {
                cb.lo[k] = fminf(cb.lo[k], ce);
                cb.hi[k] = fmaxf(cb.hi[k], ce);
            }
        }
    }
    __shared__ uint32_t s_red[kWarps][12];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = 0; k < 3; ++k) {
        const uint32_t v[4] = {__reduce_min_sync(0xFFFFFFFFu, fkey(nb.lo[k])), __reduce_max_sync(0xFFFFFFFFu, fkey(nb.hi[k])),
                               __reduce_min_sync(0xFFFFFFFFu, fkey(cb.lo[k])), __reduce_max_sync(0xFFFFFFFFu, fkey(cb.hi[k]))};
        if (lane == 0) {
            s_red[w][k] = v[0];
            s_red[w][3 + k] = v[1];
            s_red[w][6 + k] = v[2];
            s_red[w][9 + k] = v[3];
        }
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        const int i = threadIdx.x;
        const bool is_min = (i % 6) < 3;
        uint32_t v = s_red[0][i];
        for (int q = 1; q < kWarps; ++q) v = is_min ? min(v, s_red[q][i]) : max(v, s_red[q][i]);
        uint32_t* dst = i < 6 ? &N.nb[i] : &N.cb[i - 6];
        if (is_min) atomicMin(dst, v);
        else atomicMax(dst, v);
    }
}

// ---------------------------------------------------------------------------
// Object split
// ---------------------------------------------------------------------------
__device__ void eval_object(const Pass& P, BNode& N, const uint32_t* s_bin, const float* s_scale) {
    const int lane = threadIdx.x & 31;
    const uint32_t n = N.count;
    float best = INFINITY;
    int bax = -1, bplane = 0;
    DBox bl, br;
    box_reset(bl);
    box_reset(br);
    for (int k = 0; k < 3; ++k) {
        if (s_scale[k] == 0.0f) continue;
        const uint32_t* q = s_bin + kObjWords * (k * kBins + lane);
        const uint32_t cnt = q[0];
        DBox left, right;
        uint32_t nl, nr;
        scan_bins<uint32_t>(key_box(q + 1), cnt, cnt, left, nl, right, nr);
        float cost = INFINITY;
        if (lane >= 1 && nl != 0 && nl != n) {
            const float rcost = __fmul_rn(half_area(right), __uint2float_rn(nr));
            cost = __fadd_rn(__fmul_rn(half_area(left), __uint2float_rn(nl)), rcost);
        }
        float m;
        const int j = warp_argmin(cost, &m);
        const DBox jl = shfl_box(left, j), jr = shfl_box(right, j);
        if (m < best) {
            best = m;
            bax = k;
            bplane = j;
            bl = jl;
            br = jr;
        }
    }
    bool spatial = false;
    if (P.tris && P.alpha > 0.0f && bax >= 0 && N.depth < kMaxSplitDepth) {
        DBox ov;
        for (int k = 0; k < 3; ++k) {
            ov.lo[k] = fmaxf(bl.lo[k], br.lo[k]);
            ov.hi[k] = fminf(bl.hi[k], br.hi[k]);
        }
        const float root_area = half_area(key_box(P.nodes[P.set_root[N.set]].nb));
        spatial = half_area(ov) > __fmul_rn(P.alpha, root_area);
    }
    if (lane == 0) {
        N.oax = bax;
        N.oplane = bplane;
        N.ocost = best;
        N.spatial = spatial ? 1u : 0u;
        N.kind = bax >= 0 ? kObject : kHalve;
        N.sax = -1;
    }
}

__global__ void __launch_bounds__(kThreads) k_bin_object(Pass P) {
    __shared__ uint32_t s_bin[3 * kBins * kObjWords];
    __shared__ float s_clo[3], s_scale[3];
    __shared__ int s_last;
    const uint32_t c = blockIdx.x;
    BNode& N = P.nodes[P.chunk_node[c]];
    for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) init_bin_words(s_bin + kObjWords * i, kObjWords);
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        const float lo = kval(N.cb[k]), hi = kval(N.cb[3 + k]);
        const float ext = __fsub_rn(hi, lo);
        s_clo[k] = lo;
        s_scale[k] = ext > 0.0f && ext < INFINITY ? __fdiv_rn((float)kBins, ext) : 0.0f;  // 0: axis skipped
    }
    __syncthreads();
    uint32_t p0, p1;
    chunk_range(N, c, p0, p1);
    for (uint32_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const DBox b = ref_box(P.in[p]);
        for (int k = 0; k < 3; ++k) {
            if (s_scale[k] == 0.0f) continue;
            uint32_t* q = s_bin + kObjWords * (k * kBins + bin_of(centroid(b, k), s_clo[k], s_scale[k]));
            atomicAdd(q, 1u);
            for (int a = 0; a < 3; ++a) {
                atomicMin(q + 1 + a, fkey(b.lo[a]));
                atomicMax(q + 4 + a, fkey(b.hi[a]));
            }
        }
    }
    __syncthreads();
    if (N.nchunks > 1 &&
        !merge_bins(s_bin, P.bins + (size_t)N.bins * kBinWords, 3 * kBins, kObjWords, &N.ctr[0], N.nchunks, &s_last))
        return;
    if (threadIdx.x < 32) eval_object(P, N, s_bin, s_scale);
}

// ---------------------------------------------------------------------------
// Spatial split
// ---------------------------------------------------------------------------
__device__ __forceinline__ float plane_at(float lo, float hi, float w, int j) {
    return j == kBins ? hi : __fadd_rn(lo, __fmul_rn((float)j, w));
}

__device__ __forceinline__ void grow_bin(uint32_t* q, const DBox& b) {
    for (int a = 0; a < 3; ++a) {
        atomicMin(q + a, fkey(b.lo[a]));
        atomicMax(q + 3 + a, fkey(b.hi[a]));
    }
}

__global__ void __launch_bounds__(kThreads) k_bin_spatial(Pass P) {
    __shared__ uint32_t s_bin[3 * kBins * kSpWords];
    __shared__ float s_lo[3], s_hi[3], s_w[3], s_scale[3];
    __shared__ uint32_t s_cnt[3 * kThreads], s_off[3 * kThreads], s_total;
    __shared__ uint8_t s_b0[3 * kThreads];
    __shared__ float s_above[kThreads][6];
    __shared__ float s_carry[6];
    __shared__ int s_last;
    const uint32_t c = blockIdx.x;
    BNode& N = P.nodes[P.chunk_node[c]];
    if (!N.spatial) return;  // the whole block
    for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) init_bin_words(s_bin + kSpWords * i, kSpWords);
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        const float lo = kval(N.nb[k]), hi = kval(N.nb[3 + k]);
        const float ext = __fsub_rn(hi, lo);
        const bool ok = ext > 0.0f && ext < INFINITY;
        s_lo[k] = lo;
        s_hi[k] = hi;
        s_w[k] = ok ? __fdiv_rn(ext, (float)kBins) : 0.0f;
        s_scale[k] = ok ? __fdiv_rn((float)kBins, ext) : 0.0f;
    }
    __syncthreads();
    uint32_t p0, p1;
    chunk_range(N, c, p0, p1);
    // Rounds of kThreads references.  A reference spanning bins b0 < b1
    // along axis k has the m = b1 - b0 inner bin planes p_(b0+1) .. p_(b1);
    // the (reference, axis, plane) triples of a round are numbered
    // axis-major and dealt out one per thread, each thread computing the
    // triangle's bounds below and above its plane (tri_split.h).  Bin
    // b0 + i then gets the reference's box cut to "below plane i" and
    // "above plane i - 1" (the previous triple, the neighbouring thread or
    // the previous sub-round's last one), bin b1 the box cut to "above plane
    // m - 1": sbvh.cu's binning, dealt out evenly.
    for (uint32_t r0 = p0; r0 < p1; r0 += kThreads) {
        const uint32_t nr = min((uint32_t)kThreads, p1 - r0);
        __syncthreads();  // the previous round's tables are read
        {
            const uint32_t t = threadIdx.x;
            for (int k = 0; k < 3; ++k) {
                uint32_t m = 0;
                int b0 = 0;
                if (t < nr && s_scale[k] != 0.0f) {
                    const DBox rb = ref_box(P.in[r0 + t]);
                    b0 = bin_of(rb.lo[k], s_lo[k], s_scale[k]);
                    const int b1 = max(b0, bin_of(rb.hi[k], s_lo[k], s_scale[k]));
                    uint32_t* sb = s_bin + kSpWords * kBins * k;
                    atomicAdd(sb + kSpWords * b0, 1u);
                    atomicAdd(sb + kSpWords * b1 + 1, 1u);
                    if (b0 == b1) grow_bin(sb + kSpWords * b0 + 2, rb);
                    m = (uint32_t)(b1 - b0);
                }
                s_cnt[k * kThreads + t] = m;
                s_b0[k * kThreads + t] = (uint8_t)b0;
            }
        }
        __syncthreads();
        if (threadIdx.x < 32) {  // exclusive scan of the 3 x kThreads plane counts
            uint32_t run = 0;
            for (int base = 0; base < 3 * kThreads; base += 32) {
                const uint32_t v = s_cnt[base + threadIdx.x];
                uint32_t x = v;
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                    if ((int)threadIdx.x >= o) x += y;
                }
                s_off[base + threadIdx.x] = run + x - v;
                run += __shfl_sync(0xFFFFFFFFu, x, 31);
            }
            if (threadIdx.x == 0) s_total = run;
        }
        __syncthreads();
        const uint32_t total = s_total;
        for (uint32_t g0 = 0; g0 < total; g0 += kThreads) {
            const uint32_t g = g0 + threadIdx.x;
            DBox below, above, rb;
            int bin = -1, k = 0;
            bool last = false;
            uint32_t i = 0;
            if (g < total) {
                // the triple holding plane g: the last entry with s_off <= g
                int lo = 0, hi = 3 * kThreads - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_off[mid] <= g) lo = mid;
                    else hi = mid - 1;
                }
                // (an entry without planes shares its offset with the next
                // one, so the last entry at or below g has planes)
                k = lo / kThreads;
                const uint32_t t = (uint32_t)(lo % kThreads);
                i = g - s_off[lo];
                last = i + 1 == s_cnt[lo];
                const int b0 = s_b0[lo];
                bin = b0 + (int)i;
                const Ref r = P.in[r0 + t];
                rb = ref_box(r);
                float tri[9];
                load_tri(P.tris + 9 * (size_t)ref_prim(r), tri);
                const float pl = plane_at(s_lo[k], s_hi[k], s_w[k], bin + 1);
                if (k == 0) tri_plane_bounds_k<0>(tri, pl, below.lo, below.hi, above.lo, above.hi);
                else if (k == 1) tri_plane_bounds_k<1>(tri, pl, below.lo, below.hi, above.lo, above.hi);
                else tri_plane_bounds_k<2>(tri, pl, below.lo, below.hi, above.lo, above.hi);
                for (int a = 0; a < 3; ++a) {
                    s_above[threadIdx.x][a] = above.lo[a];
                    s_above[threadIdx.x][3 + a] = above.hi[a];
                }
            }
            __syncthreads();
            DBox prev;
            if (g < total && i > 0) {
                const float* q = threadIdx.x > 0 ? s_above[threadIdx.x - 1] : s_carry;
                for (int a = 0; a < 3; ++a) {
                    prev.lo[a] = q[a];
                    prev.hi[a] = q[3 + a];
                }
            }
            __syncthreads();
            if (threadIdx.x == kThreads - 1)
                for (int a = 0; a < 6; ++a) s_carry[a] = s_above[kThreads - 1][a];
            if (g < total) {
                uint32_t* sb = s_bin + kSpWords * kBins * k;
                DBox part = rb;
                if (i > 0) box_clip(part, prev);
                box_clip(part, below);
                if (!box_empty(part)) grow_bin(sb + kSpWords * bin + 2, part);
                if (last) {
                    DBox tail = rb;
                    box_clip(tail, above);
                    if (!box_empty(tail)) grow_bin(sb + kSpWords * (bin + 1) + 2, tail);
                }
            }
        }
    }
    __syncthreads();
    if (N.nchunks > 1 && !merge_bins(s_bin, P.bins + (size_t)N.bins * kBinWords + 3 * kBins * kObjWords, 3 * kBins,
                                     kSpWords, &N.ctr[1], N.nchunks, &s_last))
        return;
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    float best = N.ocost;
    int sax = -1;
    float splane = 0.0f;
    for (int k = 0; k < 3; ++k) {
        if (s_scale[k] == 0.0f) continue;
        const uint32_t* q = s_bin + kSpWords * (k * kBins + lane);
        DBox left, right;
        uint32_t nl, nr;
        scan_bins<uint32_t>(key_box(q + 2), q[0], q[1], left, nl, right, nr);
        float cost = INFINITY;
        if (lane >= 1 && nl != 0 && nr != 0) {
            const float rcost = __fmul_rn(half_area(right), __uint2float_rn(nr));
            cost = __fadd_rn(__fmul_rn(half_area(left), __uint2float_rn(nl)), rcost);
        }
        float m;
        const int j = warp_argmin(cost, &m);
        if (m < best) {
            best = m;
            sax = k;
            splane = plane_at(s_lo[k], s_hi[k], s_w[k], j);
        }
    }
    if (lane == 0 && sax >= 0) {
        N.kind = kSpatial;
        N.sax = sax;
        N.splane = splane;
    }
}

// ---------------------------------------------------------------------------
// Partition: counts, children, scatter
// ---------------------------------------------------------------------------
struct ObjectPlane {
    float lo, scale;
    int axis, plane;
};
__device__ __forceinline__ ObjectPlane object_plane(const BNode& N) {
    ObjectPlane o{0.0f, 0.0f, N.oax, N.oplane};
    if (o.axis >= 0) {
        o.lo = kval(N.cb[o.axis]);
        o.scale = __fdiv_rn((float)kBins, __fsub_rn(kval(N.cb[3 + o.axis]), o.lo));
    }
    return o;
}

// Where one reference goes under the spatial split (sbvh.cu's partition):
// entirely left or right of the plane, or clipped to both sides (a side
// whose part is empty gets nothing; both empty: left, unclipped).
__device__ __forceinline__ void spatial_side(const Ref& r, const float* tris, int ax, float pl, bool& to_l, bool& to_r,
                                             DBox& bl, DBox& br) {
    const DBox b = ref_box(r);
    bl = br = b;
    if (b.hi[ax] <= pl) {
        to_l = true, to_r = false;
    } else if (b.lo[ax] >= pl) {
        to_l = false, to_r = true;
    } else {
        float t[9];
        load_tri(tris + 9 * (size_t)ref_prim(r), t);
        DBox below, above;
        tri_plane_bounds(t, ax, pl, below.lo, below.hi, above.lo, above.hi);
        box_clip(bl, below);
        box_clip(br, above);
        to_l = !box_empty(bl);
        to_r = !box_empty(br);
        if (!to_l && !to_r) {
            to_l = true;
            bl = b;
        }
    }
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* s_tmp) {
    v = __reduce_add_sync(0xFFFFFFFFu, v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_tmp[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t t = 0;
    for (int w = 0; w < kWarps; ++w) t += s_tmp[w];
    return t;
}

__global__ void __launch_bounds__(kThreads) k_count(Pass P) {
    __shared__ uint32_t s_tmp[kWarps];
    __shared__ uint32_t s_scan[4][kThreads];
    __shared__ int s_last;
    __shared__ int32_t s_child[2];
    __shared__ uint32_t s_cf[2], s_nch[2], s_slot[2], s_begin[2], s_cnt[2], s_sweep[2];
    const uint32_t c = blockIdx.x;
    const uint32_t id = P.chunk_node[c];
    BNode& N = P.nodes[id];
    const int kind = N.kind;
    const ObjectPlane op = object_plane(N);
    uint32_t p0, p1;
    chunk_range(N, c, p0, p1);
    uint32_t cnt[4] = {0, 0, 0, 0};
    for (uint32_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const Ref r = P.in[p];
        if (kind == kSpatial) {
            bool l, rr;
            DBox bl, br;
            spatial_side(r, P.tris, N.sax, N.splane, l, rr, bl, br);
            cnt[0] += l;
            cnt[1] += rr;
        }
        if (op.axis >= 0) {
            const bool l = bin_of(centroid(ref_box(r), op.axis), op.lo, op.scale) < op.plane;
            cnt[2] += l;
            cnt[3] += !l;
        }
    }
    for (int q = 0; q < 4; ++q) cnt[q] = block_sum(cnt[q], s_tmp);
    if (N.nchunks > 1) {
        if (threadIdx.x < 4) P.chunk_cnt[4 * c + threadIdx.x] = cnt[threadIdx.x];
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(&N.ctr[2], 1u) == N.nchunks - 1;
        __syncthreads();
        if (!s_last) return;
        __threadfence();
    }
    // ---- the node's last block: totals, decision, offsets ----
    const uint32_t nch = N.nchunks, n = N.count;
    const uint32_t per = (nch + kThreads - 1) / kThreads;
    const uint32_t c0 = N.chunk_first + threadIdx.x * per, c1 = min(N.chunk_first + nch, c0 + per);
    uint32_t mine[4] = {0, 0, 0, 0};
    if (nch > 1) {
        for (uint32_t q = c0; q < c1; ++q)
            for (int w = 0; w < 4; ++w) mine[w] += __ldcg(P.chunk_cnt + 4 * q + w);
    } else if (threadIdx.x == 0) {
        for (int w = 0; w < 4; ++w) mine[w] = cnt[w];
    }
    for (int w = 0; w < 4; ++w) s_scan[w][threadIdx.x] = mine[w];
    __syncthreads();
    if (threadIdx.x < 4) {  // exclusive scan of the threads' sums, one word per thread
        uint32_t run = 0;
        for (int t = 0; t < kThreads; ++t) {
            const uint32_t v = s_scan[threadIdx.x][t];
            s_scan[threadIdx.x][t] = run;
            run += v;
        }
        s_tmp[threadIdx.x] = run;  // totals
    }
    __syncthreads();
    int k = kind;
    if (k == kSpatial && (s_tmp[0] == 0 || s_tmp[1] == 0)) k = op.axis >= 0 ? kObject : kHalve;
    const uint32_t nl = k == kSpatial ? s_tmp[0] : (k == kObject ? s_tmp[2] : n / 2);
    const uint32_t nr = k == kSpatial ? s_tmp[1] : (k == kObject ? s_tmp[3] : n - n / 2);
    {
        const int wl = k == kSpatial ? 0 : 2;
        uint32_t ol = s_scan[wl][threadIdx.x], orr = s_scan[wl + 1][threadIdx.x];
        for (uint32_t q = c0; q < c1; ++q) {
            uint32_t a, b;
            if (k == kHalve) {
                const uint32_t start = (q - N.chunk_first) * kChunk;
                a = min(start, n / 2);
                b = start - a;
            } else {
                a = ol;
                b = orr;
                if (nch > 1) {
                    ol += __ldcg(P.chunk_cnt + 4 * q + wl);
                    orr += __ldcg(P.chunk_cnt + 4 * q + wl + 1);
                }
            }
            P.chunk_off[2 * q] = a;
            P.chunk_off[2 * q + 1] = b;
        }
    }
    if (threadIdx.x == 0) {
        N.kind = k;
        for (int s = 0; s < 2; ++s) {
            const uint32_t m = s ? nr : nl;
            s_child[s] = -1;
            s_nch[s] = 0;
            s_sweep[s] = 0;
            if (m <= (uint32_t)P.leaf_max) {
                const uint32_t first = atomicAdd(&P.ctr[kCtrPool], m);
                const bool fits = first + m <= P.cap_refs;
                if (!fits) atomicExch(&P.ctr[kCtrOverflow], 1u);
                N.child[s] = -1;
                N.leaf_first[s] = fits ? first : 0u;
                N.leaf_cnt[s] = fits ? m : 0u;
                continue;
            }
            const uint32_t nid = atomicAdd(&P.ctr[kCtrNodes], 1u);
            const uint32_t begin = atomicAdd(&P.ctr[kCtrRefs], m);
            bool ok = nid < P.cap_refs && begin + m <= P.cap_refs;
            uint32_t cf = 0, nchild = 0, slot = 0xFFFFFFFFu;
            if (m <= P.sweep_max) {
                cf = atomicAdd(&P.ctr[kCtrSweep], 1u);
                ok = ok && cf < P.cap_chunks;
                s_sweep[s] = 1;
            } else {
                nchild = (m + kChunk - 1) / kChunk;
                cf = atomicAdd(&P.ctr[kCtrChunks], nchild);
                ok = ok && cf + nchild <= P.cap_chunks;
                if (nchild > 1) {
                    slot = atomicAdd(&P.ctr[kCtrBins], 1u);
                    ok = ok && slot < P.cap_bins;
                }
            }
            if (!ok) {
                atomicExch(&P.ctr[kCtrOverflow], 1u);
                N.child[s] = -1;
                N.leaf_first[s] = 0;
                N.leaf_cnt[s] = 0;
                continue;
            }
            N.child[s] = (int32_t)nid;
            s_child[s] = (int32_t)nid;
            s_cf[s] = cf;
            s_nch[s] = nchild;
            s_slot[s] = slot;
            s_begin[s] = begin;
            s_cnt[s] = m;
        }
        N.leaf_cnt[0] = N.child[0] >= 0 ? 0u : N.leaf_cnt[0];
        N.leaf_cnt[1] = N.child[1] >= 0 ? 0u : N.leaf_cnt[1];
    }
    __syncthreads();
    for (int s = 0; s < 2; ++s) {
        if (s_child[s] < 0) continue;
        BNode& C = P.nodes[s_child[s]];
        if (threadIdx.x < 6) {
            const uint32_t init = threadIdx.x < 3 ? kKeyPosInf : kKeyNegInf;
            C.nb[threadIdx.x] = init;
            C.cb[threadIdx.x] = init;
            C.lb[0][threadIdx.x] = init;
            C.lb[1][threadIdx.x] = init;
        }
        if (threadIdx.x == 0) {
            C.begin = s_begin[s];
            C.count = s_cnt[s];
            C.set = N.set;
            C.depth = N.depth + 1;
            C.chunk_first = s_cf[s];
            C.nchunks = s_nch[s];
            C.bins = s_slot[s] == 0xFFFFFFFFu ? -1 : (int32_t)s_slot[s];
            C.ctr[0] = C.ctr[1] = C.ctr[2] = 0;
            C.kind = kObject;
            C.oax = C.sax = -1;
            C.spatial = 0;
            C.child[0] = C.child[1] = -1;
            C.leaf_cnt[0] = C.leaf_cnt[1] = 0;
            if (s_sweep[s]) P.sweep_out[s_cf[s]] = (uint32_t)s_child[s];
        }
        for (uint32_t q = threadIdx.x; q < s_nch[s]; q += blockDim.x) P.chunk_out[s_cf[s] + q] = (uint32_t)s_child[s];
        if (s_slot[s] != 0xFFFFFFFFu) {
            uint32_t* g = P.bins_out + (size_t)s_slot[s] * kBinWords;
            for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) {
                init_bin_words(g + kObjWords * i, kObjWords);
                init_bin_words(g + 3 * kBins * kObjWords + kSpWords * i, kSpWords);
            }
        }
    }
}

// Block-wide min/max of 24 keys per thread (two sides x node box and
// centroid bounds) folded into global words by atomics.
__device__ void reduce_side_boxes(const DBox* box, const DBox* cen, uint32_t (*s_red)[24], uint32_t* const dst_box[2],
                                  uint32_t* const dst_cen[2]) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 3; ++k) {
            const uint32_t v0 = __reduce_min_sync(0xFFFFFFFFu, fkey(box[s].lo[k]));
            const uint32_t v1 = __reduce_max_sync(0xFFFFFFFFu, fkey(box[s].hi[k]));
            const uint32_t v2 = __reduce_min_sync(0xFFFFFFFFu, fkey(cen[s].lo[k]));
            const uint32_t v3 = __reduce_max_sync(0xFFFFFFFFu, fkey(cen[s].hi[k]));
            if (lane == 0) {
                s_red[w][12 * s + k] = v0;
                s_red[w][12 * s + 3 + k] = v1;
                s_red[w][12 * s + 6 + k] = v2;
                s_red[w][12 * s + 9 + k] = v3;
            }
        }
    __syncthreads();
    if (threadIdx.x < 24) {
        const int i = threadIdx.x, s = i / 12, j = i % 12;
        const bool is_min = (j % 6) < 3;
        uint32_t v = s_red[0][i];
        for (int q = 1; q < kWarps; ++q) v = is_min ? min(v, s_red[q][i]) : max(v, s_red[q][i]);
        uint32_t* d = j < 6 ? dst_box[s] : dst_cen[s];
        if (d && (is_min ? v != kKeyPosInf : v != kKeyNegInf)) {
            if (is_min) atomicMin(d + (j % 6), v);
            else atomicMax(d + (j % 6), v);
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_scatter(Pass P) {
    __shared__ uint32_t s_wl[kWarps], s_wr[kWarps];
    __shared__ uint32_t s_red[kWarps][24];
    const uint32_t c = blockIdx.x;
    BNode& N = P.nodes[P.chunk_node[c]];
    const int kind = N.kind;
    const ObjectPlane op = object_plane(N);
    uint32_t p0, p1;
    chunk_range(N, c, p0, p1);
    const uint32_t half = N.count / 2;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t run[2] = {P.chunk_off[2 * c], P.chunk_off[2 * c + 1]};
    Ref* dst_ref[2] = {nullptr, nullptr};
    uint32_t* dst_leaf[2] = {nullptr, nullptr};
    uint32_t lim[2];
    for (int s = 0; s < 2; ++s) {
        if (N.child[s] >= 0) {
            const BNode& C = P.nodes[N.child[s]];
            dst_ref[s] = P.out + C.begin;
            lim[s] = C.count;
        } else {
            dst_leaf[s] = P.pool + N.leaf_first[s];
            lim[s] = N.leaf_cnt[s];
        }
    }
    DBox acc[2], cen[2];
    for (int s = 0; s < 2; ++s) {
        box_reset(acc[s]);
        box_reset(cen[s]);
    }
    for (uint32_t base = p0; base < p1; base += blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        bool to[2] = {false, false};
        DBox b[2];
        Ref r;
        if (p < p1) {
            r = P.in[p];
            if (kind == kSpatial) {
                spatial_side(r, P.tris, N.sax, N.splane, to[0], to[1], b[0], b[1]);
            } else {
                b[0] = b[1] = ref_box(r);
                const bool l = kind == kObject ? bin_of(centroid(b[0], op.axis), op.lo, op.scale) < op.plane
                                               : (p - N.begin) < half;
                to[0] = l;
                to[1] = !l;
            }
        }
        const uint32_t bl = __ballot_sync(0xFFFFFFFFu, to[0]), br = __ballot_sync(0xFFFFFFFFu, to[1]);
        if (lane == 0) {
            s_wl[w] = __popc(bl);
            s_wr[w] = __popc(br);
        }
        __syncthreads();
        uint32_t off[2] = {run[0], run[1]}, tot[2] = {0, 0};
        for (int q = 0; q < kWarps; ++q) {
            if (q < w) {
                off[0] += s_wl[q];
                off[1] += s_wr[q];
            }
            tot[0] += s_wl[q];
            tot[1] += s_wr[q];
        }
        const uint32_t lt = (1u << lane) - 1u;
        off[0] += __popc(bl & lt);
        off[1] += __popc(br & lt);
        for (int s = 0; s < 2; ++s) {
            if (!to[s]) continue;
            if (off[s] >= lim[s]) {
                atomicExch(&P.ctr[kCtrOverflow], 1u);
                continue;
            }
            if (dst_ref[s]) {
                dst_ref[s][off[s]] = make_ref(b[s], ref_prim(r));
                for (int k = 0; k < 3; ++k) {
                    const float ce = centroid(b[s], k);
                    if (ce > -INFINITY && ce < INFINITY) {
                        cen[s].lo[k] = fminf(cen[s].lo[k], ce);
                        cen[s].hi[k] = fmaxf(cen[s].hi[k], ce);
                    }
                }
            } else {
                dst_leaf[s][off[s]] = ref_prim(r);
            }
            box_grow(acc[s], b[s]);
        }
        run[0] += tot[0];
        run[1] += tot[1];
        __syncthreads();
    }
    uint32_t* dbox[2];
    uint32_t* dcen[2];
    for (int s = 0; s < 2; ++s) {
        dbox[s] = N.child[s] >= 0 ? P.nodes[N.child[s]].nb : N.lb[s];
        dcen[s] = N.child[s] >= 0 ? P.nodes[N.child[s]].cb : nullptr;
    }
    reduce_side_boxes(acc, cen, s_red, dbox, dcen);
}

// ---------------------------------------------------------------------------
// Exact sweep of small box-set nodes (sah.cu's sweep_split), one block each
// ---------------------------------------------------------------------------
constexpr int kSweepPer = (int)(kSweepMax / kSweepThreads);  // references per thread

// Bitonic sort of s_key[0, n2) (n2 a power of two) with the payload s_val.
__device__ void block_sort(unsigned long long* s_key, uint16_t* s_val, uint32_t n2) {
    for (uint32_t size = 2; size <= n2; size <<= 1)
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = threadIdx.x; i < n2 / 2; i += blockDim.x) {
                const uint32_t lo = 2 * i - (i & (stride - 1));
                const uint32_t hi = lo + stride;
                const bool up = (lo & size) == 0;
                const unsigned long long a = s_key[lo], b = s_key[hi];
                if ((a > b) == up) {
                    s_key[lo] = b;
                    s_key[hi] = a;
                    const uint16_t t = s_val[lo];
                    s_val[lo] = s_val[hi];
                    s_val[hi] = t;
                }
            }
            __syncthreads();
        }
}

__device__ __forceinline__ float canon_zero(float x) { return x == 0.0f ? 0.0f : x; }

// Inclusive block scan of boxes (kSweepPer consecutive elements per thread),
// forward (prefix unions) or backward (suffix unions); out[i] gets the half
// area of the union of elements [0, i] (forward) or [i, n) (backward).
__device__ void box_scan_areas(const Ref* refs, const uint16_t* order, uint32_t n, bool forward, float* out,
                               float (*s_part)[6]) {
    const int t = threadIdx.x;
    DBox mine;
    box_reset(mine);
    const int i0 = t * kSweepPer;
    for (int e = 0; e < kSweepPer; ++e) {
        const int i = forward ? i0 + e : (int)n - 1 - (i0 + e);
        if (i < 0 || (uint32_t)i >= n) continue;
        box_grow(mine, ref_box(refs[order[i]]));
    }
    for (int k = 0; k < 3; ++k) {
        s_part[t][k] = mine.lo[k];
        s_part[t][3 + k] = mine.hi[k];
    }
    __syncthreads();
    // exclusive prefix over threads (serial per component; 512 entries)
    if (t < 6) {
        float run = t < 3 ? INFINITY : -INFINITY;
        for (int q = 0; q < kSweepThreads; ++q) {
            const float v = s_part[q][t];
            s_part[q][t] = run;
            run = t < 3 ? fminf(run, v) : fmaxf(run, v);
        }
    }
    __syncthreads();
    DBox acc;
    for (int k = 0; k < 3; ++k) {
        acc.lo[k] = s_part[t][k];
        acc.hi[k] = s_part[t][3 + k];
    }
    for (int e = 0; e < kSweepPer; ++e) {
        const int i = forward ? i0 + e : (int)n - 1 - (i0 + e);
        if (i < 0 || (uint32_t)i >= n) continue;
        box_grow(acc, ref_box(refs[order[i]]));
        out[i] = half_area(acc);
    }
    __syncthreads();
}

// Dynamic shared memory of k_sweep: sort keys, prefix and suffix areas,
// per-thread partial boxes, the sorted order of the current and best axis.
constexpr size_t kSweepSmem = sizeof(unsigned long long) * kSweepMax + 2 * sizeof(float) * kSweepMax +
                              sizeof(float) * 6 * kSweepThreads + 2 * sizeof(uint16_t) * kSweepMax;

__global__ void __launch_bounds__(kSweepThreads) k_sweep(Pass P) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    unsigned long long* s_key = reinterpret_cast<unsigned long long*>(s_dyn);
    float* s_pre = reinterpret_cast<float*>(s_key + kSweepMax);
    float* s_suf = s_pre + kSweepMax;
    float(*s_part)[6] = reinterpret_cast<float(*)[6]>(s_suf + kSweepMax);
    uint16_t* s_val = reinterpret_cast<uint16_t*>(s_suf + kSweepMax + 6 * kSweepThreads);
    uint16_t* s_best = s_val + kSweepMax;
    __shared__ float s_rc[kSweepThreads / 32];
    __shared__ uint32_t s_ro[kSweepThreads / 32], s_ri[kSweepThreads / 32];
    __shared__ int32_t s_child[2];
    __shared__ uint32_t s_begin[2], s_cnt[2], s_sw[2];
    __shared__ uint32_t s_red[kSweepThreads / 32][24];
    const uint32_t id = P.sweep_in[blockIdx.x];
    BNode& N = P.nodes[id];
    const uint32_t n = N.count;
    const Ref* refs = P.in + N.begin;
    uint32_t n2 = 1;
    while (n2 < n) n2 <<= 1;
    float best = INFINITY;
    int best_axis = -1;
    uint32_t best_pos = n / 2;
    const uint32_t half = n / 2;
    for (int k = 0; k < 3; ++k) {
        for (uint32_t i = threadIdx.x; i < n2; i += blockDim.x) {
            if (i < n) {
                const Ref r = refs[i];
                const float ce = canon_zero(centroid(ref_box(r), k));
                s_key[i] = (unsigned long long)fkey(ce) << 32 | ref_prim(r);
                s_val[i] = (uint16_t)i;
            } else {
                s_key[i] = ~0ull;
                s_val[i] = 0;
            }
        }
        __syncthreads();
        block_sort(s_key, s_val, n2);
        box_scan_areas(refs, s_val, n, true, s_pre, s_part);
        box_scan_areas(refs, s_val, n, false, s_suf, s_part);
        // lowest (cost, |i - n/2|, i) over positions 1..n-1
        float bc = INFINITY;
        uint32_t bo = 0xFFFFFFFFu, bi = 0xFFFFFFFFu;
        for (uint32_t i = 1 + threadIdx.x; i < n; i += blockDim.x) {
            const float cost = __fadd_rn(__fmul_rn(s_pre[i - 1], __uint2float_rn(i)),
                                         __fmul_rn(s_suf[i], __uint2float_rn(n - i)));
            const uint32_t off = i > half ? i - half : half - i;
            if (cost < bc || (cost == bc && (off < bo || (off == bo && i < bi)))) {
                bc = cost;
                bo = off;
                bi = i;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float oc = __shfl_xor_sync(0xFFFFFFFFu, bc, o);
            const uint32_t oo = __shfl_xor_sync(0xFFFFFFFFu, bo, o), oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
            if (oc < bc || (oc == bc && (oo < bo || (oo == bo && oi < bi)))) {
                bc = oc;
                bo = oo;
                bi = oi;
            }
        }
        if ((threadIdx.x & 31) == 0) {
            s_rc[threadIdx.x >> 5] = bc;
            s_ro[threadIdx.x >> 5] = bo;
            s_ri[threadIdx.x >> 5] = bi;
        }
        __syncthreads();
        bc = s_rc[0], bo = s_ro[0], bi = s_ri[0];
        for (int q = 1; q < kSweepThreads / 32; ++q)
            if (s_rc[q] < bc || (s_rc[q] == bc && (s_ro[q] < bo || (s_ro[q] == bo && s_ri[q] < bi)))) {
                bc = s_rc[q];
                bo = s_ro[q];
                bi = s_ri[q];
            }
        // the host's scan: strictly lower cost, or equal cost and more balanced
        const uint32_t best_off = best_pos > half ? best_pos - half : half - best_pos;
        const bool take = bi != 0xFFFFFFFFu && (bc < best || (bc == best && bo < best_off));
        if (take) {
            best = bc;
            best_axis = k;
            best_pos = bi;
        }
        if (take || (k == 0 && best_axis < 0))  // the order the references end in
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) s_best[i] = s_val[i];
        __syncthreads();
    }
    // children: [0, best_pos) and [best_pos, n) of the best axis's order
    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; ++s) {
            const uint32_t m = s ? n - best_pos : best_pos;
            s_child[s] = -1;
            s_sw[s] = 0;
            if (m <= (uint32_t)P.leaf_max) {
                const uint32_t first = atomicAdd(&P.ctr[kCtrPool], m);
                const bool fits = first + m <= P.cap_refs;
                if (!fits) atomicExch(&P.ctr[kCtrOverflow], 1u);
                N.child[s] = -1;
                N.leaf_first[s] = fits ? first : 0u;
                N.leaf_cnt[s] = fits ? m : 0u;
                continue;
            }
            const uint32_t nid = atomicAdd(&P.ctr[kCtrNodes], 1u);
            const uint32_t begin = atomicAdd(&P.ctr[kCtrRefs], m);
            const uint32_t slot = atomicAdd(&P.ctr[kCtrSweep], 1u);
            if (!(nid < P.cap_refs && begin + m <= P.cap_refs && slot < P.cap_chunks)) {
                atomicExch(&P.ctr[kCtrOverflow], 1u);
                N.child[s] = -1;
                N.leaf_cnt[s] = 0;
                continue;
            }
            N.child[s] = (int32_t)nid;
            N.leaf_cnt[s] = 0;
            s_child[s] = (int32_t)nid;
            s_begin[s] = begin;
            s_cnt[s] = m;
            s_sw[s] = slot;
        }
        N.kind = kObject;
    }
    __syncthreads();
    for (int s = 0; s < 2; ++s) {
        if (s_child[s] < 0) continue;
        BNode& C = P.nodes[s_child[s]];
        if (threadIdx.x < 6) {
            const uint32_t init = threadIdx.x < 3 ? kKeyPosInf : kKeyNegInf;
            C.nb[threadIdx.x] = init;
            C.cb[threadIdx.x] = init;
            C.lb[0][threadIdx.x] = init;
            C.lb[1][threadIdx.x] = init;
        }
        if (threadIdx.x == 0) {
            C.begin = s_begin[s];
            C.count = s_cnt[s];
            C.set = N.set;
            C.depth = N.depth + 1;
            C.chunk_first = 0;
            C.nchunks = 0;
            C.bins = -1;
            C.ctr[0] = C.ctr[1] = C.ctr[2] = 0;
            C.kind = kObject;
            C.oax = C.sax = -1;
            C.spatial = 0;
            C.child[0] = C.child[1] = -1;
            C.leaf_cnt[0] = C.leaf_cnt[1] = 0;
            P.sweep_out[s_sw[s]] = (uint32_t)s_child[s];
        }
    }
    __syncthreads();
    DBox acc[2], cen[2];
    for (int s = 0; s < 2; ++s) {
        box_reset(acc[s]);
        box_reset(cen[s]);
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const int s = i < best_pos ? 0 : 1;
        const uint32_t pos = s ? i - best_pos : i;
        const Ref r = refs[s_best[i]];
        const DBox b = ref_box(r);
        if (s_child[s] >= 0) {
            P.out[s_begin[s] + pos] = r;
        } else if (N.leaf_cnt[s] > pos) {
            P.pool[N.leaf_first[s] + pos] = ref_prim(r);
        }
        box_grow(acc[s], b);
    }
    // block reduction (16 warps)
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 3; ++k) {
            const uint32_t v0 = __reduce_min_sync(0xFFFFFFFFu, fkey(acc[s].lo[k]));
            const uint32_t v1 = __reduce_max_sync(0xFFFFFFFFu, fkey(acc[s].hi[k]));
            if (lane == 0) {
                s_red[w][6 * s + k] = v0;
                s_red[w][6 * s + 3 + k] = v1;
            }
        }
    __syncthreads();
    if (threadIdx.x < 12) {
        const int i = threadIdx.x, s = i / 6, j = i % 6;
        const bool is_min = j < 3;
        uint32_t v = s_red[0][i];
        for (int q = 1; q < kSweepThreads / 32; ++q) v = is_min ? min(v, s_red[q][i]) : max(v, s_red[q][i]);
        uint32_t* d = s_child[s] >= 0 ? P.nodes[s_child[s]].nb : N.lb[s];
        d[j] = v;  // this block alone writes them
    }
}

// ---------------------------------------------------------------------------
// Depth-first numbering and output
// ---------------------------------------------------------------------------
__global__ void k_subtree(BNode* nodes, uint32_t b, uint32_t e, uint32_t* set_depth) {
    const uint32_t i = b + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e) return;
    BNode& N = nodes[i];
    uint32_t sn = 1, sr = 0;
    for (int s = 0; s < 2; ++s) {
        if (N.child[s] >= 0) {
            sn += nodes[N.child[s]].sub_nodes;
            sr += nodes[N.child[s]].sub_refs;
        } else {
            sr += N.leaf_cnt[s];
        }
    }
    N.sub_nodes = sn;
    N.sub_refs = sr;
    if (N.depth == 1) {  // a root: first in its set's depth-first order
        N.dfs = 0;
        N.leaf_base = 0;
    }
    atomicMax(set_depth + N.set, N.depth);
}

struct WriteArgs {
    BNode* nodes;
    const uint32_t* pool;
    BvhNode* out;
    uint32_t* order;
    const int* node_base;
    const int* prim_base;
    const uint32_t* order_base;
    const uint32_t* set_off;
};

__global__ void k_place(WriteArgs A, uint32_t b, uint32_t e) {
    const uint32_t i = b + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e) return;
    const BNode& N = A.nodes[i];
    const int nbase = A.node_base[N.set], pbase = A.prim_base[N.set];
    uint32_t dfs = N.dfs + 1, leaf = N.leaf_base;
    int32_t ref[2];
    DBox box[2];
    for (int s = 0; s < 2; ++s) {
        if (N.child[s] >= 0) {
            BNode& C = A.nodes[N.child[s]];
            C.dfs = dfs;
            C.leaf_base = leaf;
            ref[s] = nbase + (int32_t)dfs;
            box[s] = key_box(C.nb);
            dfs += C.sub_nodes;
            leaf += C.sub_refs;
        } else {
            const uint32_t cnt = N.leaf_cnt[s];
            ref[s] = ~(int32_t)((((uint32_t)pbase + leaf) << 3) | (cnt - 1));
            box[s] = key_box(N.lb[s]);
            uint32_t* o = A.order + A.order_base[N.set] + leaf;
            for (uint32_t q = 0; q < cnt; ++q) o[q] = A.pool[N.leaf_first[s] + q] - A.set_off[N.set];
            leaf += cnt;
        }
        enlarge_exact(box[s]);
    }
    BvhNode nd;
    nd.a = make_float4(box[0].lo[0], box[0].hi[0], box[0].lo[1], box[0].hi[1]);
    nd.b = make_float4(box[1].lo[0], box[1].hi[0], box[1].lo[1], box[1].hi[1]);
    nd.c = make_float4(box[0].lo[2], box[0].hi[2], box[1].lo[2], box[1].hi[2]);
    nd.d = make_int4(ref[0], ref[1], 0, 0);
    A.out[nbase + N.dfs] = nd;
}

// Sets of one primitive: one node, a leaf on the left and a never-hit box on
// the right (the host builders' special case); fillers after the used nodes
// of a box set.
__global__ void k_single(const uint32_t* sets, uint32_t count, const float* tris, const float4* blo,
                         const float4* bhi, const uint32_t* set_off, const int* node_base, const int* prim_base,
                         const uint32_t* order_base, BvhNode* out, uint32_t* order) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t s = sets[i], p = set_off[s];
    DBox b;
    if (tris) {
        const float* t = tris + 9 * (size_t)p;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = fminf(fminf(t[k], t[3 + k]), t[6 + k]);
            b.hi[k] = fmaxf(fmaxf(t[k], t[3 + k]), t[6 + k]);
        }
    } else {
        b.lo[0] = blo[p].x, b.lo[1] = blo[p].y, b.lo[2] = blo[p].z;
        b.hi[0] = bhi[p].x, b.hi[1] = bhi[p].y, b.hi[2] = bhi[p].z;
    }
    enlarge_exact(b);
    const int32_t leaf = ~(prim_base[s] << 3);
    BvhNode nd;
    nd.a = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
    nd.b = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    nd.c = make_float4(b.lo[2], b.hi[2], INFINITY, -INFINITY);
    nd.d = make_int4(leaf, leaf, 0, 0);
    out[node_base[s]] = nd;
    order[order_base[s]] = 0;
}

__global__ void k_filler(BvhNode* out, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BvhNode nd;
    nd.a = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    nd.b = nd.a;
    nd.c = nd.a;
    nd.d = make_int4(kNone, kNone, 0, 0);
    out[i] = nd;
}

__global__ void k_reset_level(uint32_t* ctr) {
    ctr[kCtrRefs] = 0;
    ctr[kCtrChunks] = 0;
    ctr[kCtrBins] = 0;
    ctr[kCtrSweep] = 0;
}

__global__ void k_init_bins(uint32_t* bins, uint32_t slots) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slots * 3 * kBins) return;
    const uint32_t slot = i / (3 * kBins), b = i % (3 * kBins);
    uint32_t* g = bins + (size_t)slot * kBinWords;
    init_bin_words(g + kObjWords * b, kObjWords);
    init_bin_words(g + 3 * kBins * kObjWords + kSpWords * b, kSpWords);
}

__global__ void k_soup(const float4* __restrict__ pos, const uint32_t* __restrict__ indices, uint32_t vbase,
                       uint32_t ibase, uint32_t ntri, float* __restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    for (int v = 0; v < 3; ++v) {
        const float4 p = pos[vbase + indices[ibase + 3 * t + v]];
        out[9 * (size_t)t + 3 * v] = p.x;
        out[9 * (size_t)t + 3 * v + 1] = p.y;
        out[9 * (size_t)t + 3 * v + 2] = p.z;
    }
}

inline uint32_t div_up(size_t a, size_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace

cudaError_t gather_triangle_soup(const float4* pos, const uint32_t* indices, uint32_t vbase, uint32_t ibase,
                                 uint32_t ntri, float* out, cudaStream_t st) {
    if (ntri == 0) return cudaSuccess;
    k_soup<<<div_up(ntri, 256), 256, 0, st>>>(pos, indices, vbase, ibase, ntri, out);
    return cudaGetLastError();
}

GpuTreeBuilder::~GpuTreeBuilder() { release(); }

void GpuTreeBuilder::release() {
    if (mem_) cudaFree(mem_);
    mem_ = nullptr;
    mem_bytes_ = 0;
}

cudaError_t GpuTreeBuilder::build_triangles(const float* tris, const std::vector<uint32_t>& counts, int leaf_max,
                                            float alpha, uint32_t* err, cudaStream_t st) {
    return run(true, tris, nullptr, nullptr, counts, leaf_max, alpha, err, st);
}

cudaError_t GpuTreeBuilder::build_boxes(const float4* lo, const float4* hi, uint32_t n, int leaf_max, uint32_t* err,
                                        cudaStream_t st) {
    return run(false, nullptr, lo, hi, std::vector<uint32_t>{n}, leaf_max, 0.0f, err, st);
}

cudaError_t GpuTreeBuilder::run(bool triangles, const float* tris, const float4* lo, const float4* hi,
                                const std::vector<uint32_t>& counts, int leaf_max, float alpha, uint32_t* err,
                                cudaStream_t st) {
    triangles_ = triangles;
    tris_ = tris;
    box_lo_ = lo;
    box_hi_ = hi;
    size_t total = 0;
    for (uint32_t n : counts) total += n;
    // spatial splits reference some triangles more than once
    // (the 1M-triangle terrain ends with 3.2 references per triangle)
    size_t cap = triangles && alpha > 0.0f ? 4 * total + 4096 : total + 4096;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    cudaError_t e = cudaSuccess;
    for (int tries = 0; tries < 6; ++tries) {
        bool overflow = false;
        e = attempt(triangles, tris, lo, hi, counts, leaf_max, alpha, err, st, cap, &overflow);
        if (e != cudaSuccess || !overflow) break;
        cap *= 2;
        e = cudaErrorMemoryAllocation;
    }
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&build_ms_, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return e;
}

cudaError_t GpuTreeBuilder::attempt(bool triangles, const float* tris, const float4* blo, const float4* bhi,
                                    const std::vector<uint32_t>& counts, int leaf_max, float alpha, uint32_t* err,
                                    cudaStream_t st, size_t cap, bool* overflow) {
    (void)err;
    const uint32_t nsets = (uint32_t)counts.size();
    set_n_ = counts;
    set_off_.assign(nsets, 0);
    size_t total = 0;
    for (uint32_t s = 0; s < nsets; ++s) {
        set_off_[s] = (uint32_t)total;
        total += counts[s];
    }
    nodes_.assign(nsets, 0);
    refs_.assign(nsets, 0);
    depth_.assign(nsets, 0);
    set_root_.assign(nsets, 0xFFFFFFFFu);
    levels_ = 0;
    const uint32_t sweep_max = triangles ? 0u : kSweepMax;

    // ---- layout ----
    const size_t cap_chunks = cap / 2 + 1024, cap_bins = cap / kChunk + 64;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = (off + bytes + 255) / 256 * 256;
        return o;
    };
    L_.cap = cap;
    L_.cap_chunks = cap_chunks;
    L_.cap_bins = cap_bins;
    L_.nodes = take(sizeof(BNode) * cap);
    L_.refs0 = take(sizeof(Ref) * cap);
    L_.refs1 = take(sizeof(Ref) * cap);
    L_.pool = take(sizeof(uint32_t) * cap);
    L_.chunks0 = take(sizeof(uint32_t) * cap_chunks);
    L_.chunks1 = take(sizeof(uint32_t) * cap_chunks);
    L_.chunk_cnt = take(sizeof(uint32_t) * 4 * cap_chunks);
    L_.chunk_off = take(sizeof(uint32_t) * 2 * cap_chunks);
    L_.bins0 = take(sizeof(uint32_t) * kBinWords * cap_bins);
    L_.bins1 = take(sizeof(uint32_t) * kBinWords * cap_bins);
    L_.sweep0 = take(sizeof(uint32_t) * cap_chunks);
    L_.sweep1 = take(sizeof(uint32_t) * cap_chunks);
    L_.ctr = take(sizeof(uint32_t) * kCtrs);
    L_.sets = take(sizeof(uint32_t) * 3 * std::max<uint32_t>(nsets, 1));  // root, offset, depth
    if (off > mem_bytes_) {
        release();
        cudaError_t e = cudaMalloc(&mem_, off);
        if (e != cudaSuccess) return e;
        mem_bytes_ = off;
    }
    char* m = static_cast<char*>(mem_);
    BNode* nodes = reinterpret_cast<BNode*>(m + L_.nodes);
    Ref* refs[2] = {reinterpret_cast<Ref*>(m + L_.refs0), reinterpret_cast<Ref*>(m + L_.refs1)};
    uint32_t* chunks[2] = {reinterpret_cast<uint32_t*>(m + L_.chunks0), reinterpret_cast<uint32_t*>(m + L_.chunks1)};
    uint32_t* bins[2] = {reinterpret_cast<uint32_t*>(m + L_.bins0), reinterpret_cast<uint32_t*>(m + L_.bins1)};
    uint32_t* sweeps[2] = {reinterpret_cast<uint32_t*>(m + L_.sweep0), reinterpret_cast<uint32_t*>(m + L_.sweep1)};
    uint32_t* ctr = reinterpret_cast<uint32_t*>(m + L_.ctr);
    uint32_t* sets = reinterpret_cast<uint32_t*>(m + L_.sets);

    // ---- level 0: a root per set of two or more primitives ----
    std::vector<BNode> roots;
    std::vector<uint32_t> chunk_list, sweep_list;
    uint32_t nbins = 0;
    for (uint32_t s = 0; s < nsets; ++s) {
        const uint32_t n = counts[s];
        if (n < 2) continue;
        BNode r;
        memset(&r, 0, sizeof(r));
        for (int k = 0; k < 6; ++k) {
            const uint32_t init = k < 3 ? fkey(INFINITY) : fkey(-INFINITY);
            r.nb[k] = r.cb[k] = r.lb[0][k] = r.lb[1][k] = init;
        }
        r.begin = set_off_[s];
        r.count = n;
        r.set = s;
        r.depth = 1;
        r.chunk_first = (uint32_t)chunk_list.size();
        r.nchunks = div_up(n, kChunk);
        r.bins = r.nchunks > 1 ? (int32_t)nbins++ : -1;
        r.kind = kObject;
        r.oax = r.sax = -1;
        r.child[0] = r.child[1] = -1;
        set_root_[s] = (uint32_t)roots.size();
        for (uint32_t q = 0; q < r.nchunks; ++q) chunk_list.push_back((uint32_t)roots.size());
        if (n <= sweep_max) sweep_list.push_back((uint32_t)roots.size());
        roots.push_back(r);
    }
    if (roots.size() > cap || chunk_list.size() > cap_chunks || nbins > cap_bins) {
        *overflow = true;
        return cudaSuccess;
    }
    std::vector<uint32_t> set_words(3 * (size_t)std::max<uint32_t>(nsets, 1), 0);
    for (uint32_t s = 0; s < nsets; ++s) {
        set_words[s] = set_root_[s] == 0xFFFFFFFFu ? 0u : set_root_[s];
        set_words[nsets + s] = set_off_[s];
    }
    uint32_t ctr_h[kCtrs] = {};
    ctr_h[kCtrNodes] = (uint32_t)roots.size();
    cudaError_t e = cudaSuccess;
#define GB_CK(call)                    \
    do {                               \
        e = (call);                    \
        if (e != cudaSuccess) return e; \
    } while (0)
    GB_CK(cudaMemcpyAsync(sets, set_words.data(), sizeof(uint32_t) * set_words.size(), cudaMemcpyHostToDevice, st));
    GB_CK(cudaMemcpyAsync(ctr, ctr_h, sizeof(ctr_h), cudaMemcpyHostToDevice, st));
    level_begin_.assign(1, 0);
    if (!roots.empty()) {
        GB_CK(cudaMemcpyAsync(nodes, roots.data(), sizeof(BNode) * roots.size(), cudaMemcpyHostToDevice, st));
        GB_CK(cudaMemcpyAsync(chunks[0], chunk_list.data(), sizeof(uint32_t) * chunk_list.size(),
                              cudaMemcpyHostToDevice, st));
        if (!sweep_list.empty())
            GB_CK(cudaMemcpyAsync(sweeps[0], sweep_list.data(), sizeof(uint32_t) * sweep_list.size(),
                                  cudaMemcpyHostToDevice, st));
        if (nbins) k_init_bins<<<div_up((size_t)nbins * 3 * kBins, 256), 256, 0, st>>>(bins[0], nbins);
        Pass P0{};
        P0.nodes = nodes;
        P0.chunk_node = chunks[0];
        P0.tris = triangles ? tris : nullptr;
        k_init_refs<<<(uint32_t)chunk_list.size(), kThreads, 0, st>>>(P0, refs[0], blo, bhi);
        GB_CK(cudaGetLastError());
    }
    level_begin_.push_back((uint32_t)roots.size());
    // chunks of nodes that are swept are not binned
    uint32_t nchunks = sweep_list.empty() ? (uint32_t)chunk_list.size() : 0u;
    uint32_t nsweep = (uint32_t)sweep_list.size();
    uint32_t* host_ctr = nullptr;
    GB_CK(cudaMallocHost(&host_ctr, sizeof(uint32_t) * kCtrs));
    struct HostFree {
        uint32_t* p;
        ~HostFree() { cudaFreeHost(p); }
    } host_free{host_ctr};
    int cur = 0;
    while (nchunks + nsweep > 0) {
        Pass P{};
        P.nodes = nodes;
        P.in = refs[cur];
        P.out = refs[cur ^ 1];
        P.chunk_node = chunks[cur];
        P.chunk_cnt = reinterpret_cast<uint32_t*>(m + L_.chunk_cnt);
        P.chunk_off = reinterpret_cast<uint32_t*>(m + L_.chunk_off);
        P.chunk_out = chunks[cur ^ 1];
        P.bins = bins[cur];
        P.bins_out = bins[cur ^ 1];
        P.sweep_in = sweeps[cur];
        P.sweep_out = sweeps[cur ^ 1];
        P.pool = reinterpret_cast<uint32_t*>(m + L_.pool);
        P.ctr = ctr;
        P.cap_refs = (uint32_t)std::min<size_t>(cap, 0xFFFFFFF0u);
        P.cap_chunks = (uint32_t)std::min<size_t>(cap_chunks, 0xFFFFFFF0u);
        P.cap_bins = (uint32_t)std::min<size_t>(cap_bins, 0xFFFFFFF0u);
        P.tris = triangles ? tris : nullptr;
        P.set_root = sets;
        P.leaf_max = std::max(leaf_max, 1);
        P.alpha = triangles ? alpha : 0.0f;
        P.sweep_max = sweep_max;
        k_reset_level<<<1, 1, 0, st>>>(ctr);
        if (nchunks) {
            k_bin_object<<<nchunks, kThreads, 0, st>>>(P);
            if (P.tris && P.alpha > 0.0f) k_bin_spatial<<<nchunks, kThreads, 0, st>>>(P);
            k_count<<<nchunks, kThreads, 0, st>>>(P);
            k_scatter<<<nchunks, kThreads, 0, st>>>(P);
        }
        if (nsweep) {
            GB_CK(ensure_dynamic_smem(k_sweep, (int)kSweepSmem));
            k_sweep<<<nsweep, kSweepThreads, kSweepSmem, st>>>(P);
        }
        GB_CK(cudaGetLastError());
        GB_CK(cudaMemcpyAsync(host_ctr, ctr, sizeof(uint32_t) * kCtrs, cudaMemcpyDeviceToHost, st));
        GB_CK(cudaStreamSynchronize(st));
        ++levels_;
        if (host_ctr[kCtrOverflow]) {
            *overflow = true;
            return cudaSuccess;
        }
        nchunks = host_ctr[kCtrChunks];
        nsweep = host_ctr[kCtrSweep];
        level_begin_.push_back(host_ctr[kCtrNodes]);
        cur ^= 1;
        if (levels_ > 4096) return cudaErrorUnknown;  // cannot happen: every level splits nodes
    }
    // ---- subtree sizes bottom-up, depths ----
    uint32_t* set_depth = sets + 2 * nsets;
    for (int lv = (int)level_begin_.size() - 2; lv >= 0; --lv) {
        const uint32_t b = level_begin_[lv], en = level_begin_[lv + 1];
        if (en > b) k_subtree<<<div_up(en - b, 256), 256, 0, st>>>(nodes, b, en, set_depth);
    }
    GB_CK(cudaGetLastError());
    std::vector<uint32_t> depths(nsets);
    if (nsets) {
        GB_CK(cudaMemcpyAsync(depths.data(), set_depth, sizeof(uint32_t) * nsets, cudaMemcpyDeviceToHost, st));
    }
    std::vector<BNode> rec(roots.size());
    if (!roots.empty())
        GB_CK(cudaMemcpyAsync(rec.data(), nodes, sizeof(BNode) * roots.size(), cudaMemcpyDeviceToHost, st));
    GB_CK(cudaStreamSynchronize(st));
    for (uint32_t s = 0; s < nsets; ++s) {
        if (counts[s] == 0) continue;
        if (counts[s] == 1) {
            nodes_[s] = 1;
            refs_[s] = 1;
            depth_[s] = 1;
            continue;
        }
        const BNode& r = rec[set_root_[s]];
        nodes_[s] = triangles ? r.sub_nodes : std::max<uint32_t>(counts[s] - 1, 1);
        refs_[s] = r.sub_refs;
        depth_[s] = depths[s];
    }
    *overflow = false;
    return cudaSuccess;
#undef GB_CK
}

cudaError_t GpuTreeBuilder::write(BvhNode* out, const std::vector<int>& node_base, const std::vector<int>& prim_base,
                                  uint32_t* order, const std::vector<uint32_t>& order_base, cudaStream_t st) {
    const uint32_t nsets = (uint32_t)set_n_.size();
    if (nsets == 0) return cudaSuccess;
    char* m = static_cast<char*>(mem_);
    BNode* nodes = reinterpret_cast<BNode*>(m + L_.nodes);
    // per-set tables: node base, prim base, order base, offset, single-set list
    std::vector<uint32_t> tab(5 * (size_t)nsets, 0);
    std::vector<uint32_t> singles;
    for (uint32_t s = 0; s < nsets; ++s) {
        tab[s] = (uint32_t)node_base[s];
        tab[nsets + s] = (uint32_t)prim_base[s];
        tab[2 * nsets + s] = order_base[s];
        tab[3 * nsets + s] = set_off_[s];
        if (set_n_[s] == 1) singles.push_back(s);
    }
    for (size_t i = 0; i < singles.size(); ++i) tab[4 * nsets + i] = singles[i];
    uint32_t* d_tab = nullptr;
    cudaError_t e = cudaMallocAsync(&d_tab, sizeof(uint32_t) * tab.size(), st);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(d_tab, tab.data(), sizeof(uint32_t) * tab.size(), cudaMemcpyHostToDevice, st);
    // fillers of box sets first (unused node slots), then the trees
    if (e == cudaSuccess && !triangles_)
        for (uint32_t s = 0; s < nsets; ++s)
            if (nodes_[s]) k_filler<<<div_up(nodes_[s], 256), 256, 0, st>>>(out + node_base[s], nodes_[s]);
    WriteArgs A;
    A.nodes = nodes;
    A.pool = reinterpret_cast<const uint32_t*>(m + L_.pool);
    A.out = out;
    A.order = order;
    A.node_base = reinterpret_cast<const int*>(d_tab);
    A.prim_base = reinterpret_cast<const int*>(d_tab + nsets);
    A.order_base = d_tab + 2 * nsets;
    A.set_off = d_tab + 3 * nsets;
    for (size_t lv = 0; lv + 1 < level_begin_.size() && e == cudaSuccess; ++lv) {
        const uint32_t b = level_begin_[lv], en = level_begin_[lv + 1];
        if (en > b) k_place<<<div_up(en - b, 256), 256, 0, st>>>(A, b, en);
    }
    if (e == cudaSuccess && !singles.empty())
        k_single<<<div_up(singles.size(), 128), 128, 0, st>>>(d_tab + 4 * nsets, (uint32_t)singles.size(),
                                                               triangles_ ? tris_ : nullptr, box_lo_, box_hi_,
                                                               d_tab + 3 * nsets, A.node_base, A.prim_base,
                                                               A.order_base, out, order);
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaFreeAsync(d_tab, st);
    return e;
}

}  // namespace ddgi

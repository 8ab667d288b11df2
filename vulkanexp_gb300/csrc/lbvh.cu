// lbvh.cu — linear BVH construction on the GPU.
//
// Replaces the driver-built Vulkan acceleration structures
// (src/Renderer.cpp:272-449 BLAS, 525-642 TLAS) with:
//   1. centroid bounds (reduction),
//   2. 30-bit Morton codes of the primitive centroids,
//   3. a stable LSD radix sort (4 passes of 8 bits; per-block histograms,
//      one scan, warp-match ranked scatter),
//   4. the Karras (HPG 2012) hierarchy: one thread per inner node finds its
//      range and split from the longest common prefix of the sorted codes,
//   5. a bottom-up box refit (one thread per leaf, second arriver continues),
//   6. finalisation into 64-byte two-child nodes, collapsing subtrees of at
//      most `leaf_max` primitives into leaves and enlarging every box so that
//      float slab tests are conservative.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "lbvh.h"

namespace ddgi {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;  // elements per thread per block in the sort
constexpr int kSortTile = kSortThreads * kSortItems;

__device__ __forceinline__ void atomic_min_f(float* a, float v) {
    if (v >= 0.0f) atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
    else atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* a, float v) {
    if (v >= 0.0f) atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
    else atomicMin(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}

__global__ void k_init_bounds(float* b) {
    if (threadIdx.x < 3) b[threadIdx.x] = INFINITY;
    else if (threadIdx.x < 6) b[threadIdx.x] = -INFINITY;
}

__global__ void k_centroid_bounds(const float4* lo, const float4* hi, uint32_t n, float* bounds) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 a = lo[i], b = hi[i];
        float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (c[k] == c[k]) {  // skip NaN
                mn[k] = fminf(mn[k], c[k]);
                mx[k] = fmaxf(mx[k], c[k]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (mn[k] <= mx[k]) {
                atomic_min_f(bounds + k, mn[k]);
                atomic_max_f(bounds + 3 + k, mx[k]);
            }
        }
    }
}

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(const float4* lo, const float4* hi, uint32_t n, const float* bounds, uint32_t* keys,
                         uint32_t* vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = lo[i], b = hi[i];
    float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float ext = bounds[3 + k] - bounds[k];
        float u = ext > 0.0f ? (c[k] - bounds[k]) / ext : 0.5f;
        u = fminf(fmaxf(u, 0.0f), 1.0f);  // NaN -> 0
        q[k] = (uint32_t)fminf(u * 1024.0f, 1023.0f);
    }
    keys[i] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    vals[i] = i;
}

// --- stable LSD radix sort --------------------------------------------------
__global__ void k_radix_hist(const uint32_t* keys, uint32_t n, int shift, uint32_t* hist, uint32_t nblocks) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    uint32_t base = blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; ++k) {
        uint32_t i = base + k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of `n` counters in place, one block of 1024 threads.
__global__ void k_scan_single(uint32_t* data, uint32_t n) {
    __shared__ uint32_t part[1024];
    uint32_t per = (n + 1023) / 1024;
    uint32_t b = threadIdx.x * per, e = min(n, b + per);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; ++i) s += data[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        uint32_t v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (uint32_t i = b; i < e; ++i) {
        uint32_t v = data[i];
        data[i] = run;
        run += v;
    }
}

__global__ void k_radix_scatter(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t n, int shift,
                                const uint32_t* offsets, uint32_t nblocks, uint32_t* keys_out, uint32_t* vals_out) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[kSortThreads / 32][256];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    base[t] = offsets[t * nblocks + blockIdx.x];
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (int k = 0; k < kSortItems; ++k) {
        uint32_t i = blockIdx.x * kSortTile + k * kSortThreads + t;
        bool valid = i < n;
        uint32_t key = valid ? keys_in[i] : 0u, val = valid ? vals_in[i] : 0u;
        uint32_t digit = valid ? ((key >> shift) & 255u) : 256u;
        for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][t] = 0;
        __syncthreads();
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t rank = __popc(peers & lt_mask);
        int leader = __ffs(peers) - 1;
        if (valid && lane == leader) wcnt[warp][digit] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = base[t];
            for (int w = 0; w < kSortThreads / 32; ++w) {
                uint32_t c = wcnt[w][t];
                wcnt[w][t] = run;
                run += c;
            }
            base[t] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = wcnt[warp][digit] + rank;
            if (pos < n) {  // always true for a consistent histogram
                keys_out[pos] = key;
                vals_out[pos] = val;
            }
        }
        __syncthreads();
    }
}

// --- Karras hierarchy --------------------------------------------------------
__device__ __forceinline__ int delta(const uint32_t* codes, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = codes[i], b = codes[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

// child encoding during construction: >= 0 inner node, < 0 leaf ~sorted_pos
__global__ void k_karras(const uint32_t* codes, int n, int2* children, int2* ranges, int* inner_parent,
                         int* leaf_parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(codes, n, i, i - d);
    int lmax = 2;
    while (delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(codes, n, i, j);
    int s = 0, step = l;
    do {
        step = (step + 1) >> 1;
        int ns = s + step;
        if (ns < l && delta(codes, n, i, i + ns * d) > dnode) s = ns;
    } while (step > 1);
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    int left = (lo == gamma) ? ~gamma : gamma;
    int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    children[i] = make_int2(left, right);
    ranges[i] = make_int2(lo, hi);
    if (left >= 0) inner_parent[left] = i;
    else leaf_parent[~left] = i;
    if (right >= 0) inner_parent[right] = i;
    else leaf_parent[~right] = i;
    if (i == 0) inner_parent[0] = -1;
}

// Inner nodes on the path root -> leaf, maximised into *depth (the stack a
// near-first traversal needs within this tree).
__global__ void k_depth(const int* inner_parent, const int* leaf_parent, int n, uint32_t* depth) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t d = 0;
    int p = leaf_parent[j];
    while (p >= 0 && p < n - 1 && d <= (uint32_t)n) {
        ++d;
        p = inner_parent[p];
    }
    atomicMax(depth, d);
}

__global__ void k_refit(const float4* prim_lo, const float4* prim_hi, const uint32_t* sorted_ids, int n,
                        const int2* children, const int* inner_parent, const int* leaf_parent, uint32_t* flags,
                        float4* node_lo, float4* node_hi, uint32_t* err) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int p = leaf_parent[j];
    for (int level = 0; p >= 0; ++level) {
        if (p >= n - 1 || level > n) {  // malformed tree: stop instead of running away
            raise_error(err, DEV_BAD_INDEX);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[p], 1u) == 0) return;  // first arriver stops
        __threadfence();
        int2 c = children[p];
        if (c.x >= n - 1 || c.y >= n - 1 || (c.x < 0 && ~c.x >= n) || (c.y < 0 && ~c.y >= n)) {
            raise_error(err, DEV_BAD_INDEX);
            return;
        }
        float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0);
        int cs[2] = {c.x, c.y};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            float4 a, b;
            if (cs[k] >= 0) {
                a = __ldcg(node_lo + cs[k]);
                b = __ldcg(node_hi + cs[k]);
            } else {
                uint32_t id = sorted_ids[~cs[k]];
                if (id >= (uint32_t)n) id = 0;
                a = prim_lo[id];
                b = prim_hi[id];
            }
            lo.x = fminf(lo.x, a.x);
            lo.y = fminf(lo.y, a.y);
            lo.z = fminf(lo.z, a.z);
            hi.x = fmaxf(hi.x, b.x);
            hi.y = fmaxf(hi.y, b.y);
            hi.z = fmaxf(hi.z, b.z);
        }
        __stcg(node_lo + p, lo);
        __stcg(node_hi + p, hi);
        p = inner_parent[p];
    }
}

__device__ __forceinline__ void enlarge(float4& lo, float4& hi) {
    float e;
    e = (hi.x - lo.x) * 1e-5f + (fabsf(lo.x) + fabsf(hi.x)) * 1e-6f + 1e-7f;
    lo.x -= e;
    hi.x += e;
    e = (hi.y - lo.y) * 1e-5f + (fabsf(lo.y) + fabsf(hi.y)) * 1e-6f + 1e-7f;
    lo.y -= e;
    hi.y += e;
    e = (hi.z - lo.z) * 1e-5f + (fabsf(lo.z) + fabsf(hi.z)) * 1e-6f + 1e-7f;
    lo.z -= e;
    hi.z += e;
}

__device__ __forceinline__ int leaf_ref(int first, int count) { return ~((first << 3) | (count - 1)); }

__global__ void k_finalize(const float4* prim_lo, const float4* prim_hi, const uint32_t* sorted_ids, int n,
                           const int2* children, const int2* ranges, const float4* node_lo, const float4* node_hi,
                           int leaf_max, BvhNode* out, int node_base, int prim_base, uint32_t* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int2 c = children[i];
    if (c.x >= n - 1 || c.y >= n - 1 || (c.x < 0 && ~c.x >= n) || (c.y < 0 && ~c.y >= n)) {
        raise_error(err, DEV_BAD_INDEX);
        c = make_int2(~0, ~0);  // keep the node well-formed
    }
    int cs[2] = {c.x, c.y};
    float4 lo[2], hi[2];
    int ref[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (cs[k] >= 0) {
            lo[k] = node_lo[cs[k]];
            hi[k] = node_hi[cs[k]];
            int2 r = ranges[cs[k]];
            int cnt = r.y - r.x + 1;
            ref[k] = cnt <= leaf_max ? leaf_ref(prim_base + r.x, cnt) : node_base + cs[k];
        } else {
            uint32_t id = sorted_ids[~cs[k]];
            if (id >= (uint32_t)n) id = 0;
            lo[k] = prim_lo[id];
            hi[k] = prim_hi[id];
            ref[k] = leaf_ref(prim_base + ~cs[k], 1);
        }
        enlarge(lo[k], hi[k]);
    }
    BvhNode nd;
    nd.a = make_float4(lo[0].x, hi[0].x, lo[0].y, hi[0].y);
    nd.b = make_float4(lo[1].x, hi[1].x, lo[1].y, hi[1].y);
    nd.c = make_float4(lo[0].z, hi[0].z, lo[1].z, hi[1].z);
    nd.d = make_int4(ref[0], ref[1], 0, 0);
    out[node_base + i] = nd;
}

// A tree of a single primitive: one node with the leaf on the left and an
// empty (never hit) right child.
__global__ void k_single(const float4* prim_lo, const float4* prim_hi, BvhNode* out, int node_base, int prim_base) {
    float4 lo = prim_lo[0], hi = prim_hi[0];
    enlarge(lo, hi);
    BvhNode nd;
    nd.a = make_float4(lo.x, hi.x, lo.y, hi.y);
    nd.b = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    nd.c = make_float4(lo.z, hi.z, INFINITY, -INFINITY);
    nd.d = make_int4(leaf_ref(prim_base, 1), leaf_ref(prim_base, 1), 0, 0);
    out[node_base] = nd;
}

__global__ void k_iota(uint32_t* v, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

inline uint32_t div_up(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

}  // namespace

size_t lbvh_scratch_bytes(uint32_t n) {
    uint32_t nb = div_up(n > 0 ? n : 1, kSortTile);
    size_t s = 0;
    auto add = [&](size_t b) { s += (b + 255) & ~size_t(255); };
    add(6 * sizeof(float));                 // bounds
    add(4 * sizeof(uint32_t) * (size_t)n);  // keys/vals x2
    add(sizeof(uint32_t) * 256 * (size_t)nb);
    add(sizeof(int2) * 2 * (size_t)n);      // children + ranges
    add(sizeof(int) * 2 * (size_t)n);       // parents
    add(sizeof(uint32_t) * (size_t)n);      // flags
    add(sizeof(float4) * 2 * (size_t)n);    // node boxes
    return s;
}

cudaError_t lbvh_build(const float4* prim_lo, const float4* prim_hi, uint32_t n, int leaf_max, BvhNode* nodes,
                       int node_base, int prim_base, uint32_t* sorted_ids, void* scratch, uint32_t* err, uint32_t* depth,
                       cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    if (n == 1) {
        k_iota<<<1, 32, 0, st>>>(sorted_ids, 1);
        k_single<<<1, 1, 0, st>>>(prim_lo, prim_hi, nodes, node_base, prim_base);
        return cudaGetLastError();
    }
    char* p = static_cast<char*>(scratch);
    auto take = [&](size_t b) {
        char* r = p;
        p += (b + 255) & ~size_t(255);
        return r;
    };
    uint32_t nb = div_up(n, kSortTile);
    float* bounds = reinterpret_cast<float*>(take(6 * sizeof(float)));
    uint32_t* keys0 = reinterpret_cast<uint32_t*>(take(4 * sizeof(uint32_t) * (size_t)n));
    uint32_t* vals0 = keys0 + n;
    uint32_t* keys1 = vals0 + n;
    uint32_t* vals1 = keys1 + n;
    uint32_t* hist = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * 256 * (size_t)nb));
    int2* children = reinterpret_cast<int2*>(take(sizeof(int2) * 2 * (size_t)n));
    int2* ranges = children + n;
    int* inner_parent = reinterpret_cast<int*>(take(sizeof(int) * 2 * (size_t)n));
    int* leaf_parent = inner_parent + n;
    uint32_t* flags = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (size_t)n));
    float4* node_lo = reinterpret_cast<float4*>(take(sizeof(float4) * 2 * (size_t)n));
    float4* node_hi = node_lo + n;

    const int T = 256;
    k_init_bounds<<<1, 32, 0, st>>>(bounds);
    k_centroid_bounds<<<min(div_up(n, T), 1024u), T, 0, st>>>(prim_lo, prim_hi, n, bounds);
    k_morton<<<div_up(n, T), T, 0, st>>>(prim_lo, prim_hi, n, bounds, keys0, vals0);
    uint32_t *ki = keys0, *vi = vals0, *ko = keys1, *vo = vals1;
    for (int shift = 0; shift < 32; shift += 8) {
        k_radix_hist<<<nb, kSortThreads, 0, st>>>(ki, n, shift, hist, nb);
        k_scan_single<<<1, 1024, 0, st>>>(hist, 256 * nb);
        k_radix_scatter<<<nb, kSortThreads, 0, st>>>(ki, vi, n, shift, hist, nb, ko, vo);
        uint32_t* t;
        t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
    }
    // 4 passes: the sorted data is back in keys0/vals0
    cudaMemcpyAsync(sorted_ids, vi, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(inner_parent, 0xFF, sizeof(int) * 2 * (size_t)n, st);  // parents = -1
    k_karras<<<div_up(n - 1, T), T, 0, st>>>(ki, (int)n, children, ranges, inner_parent, leaf_parent);
    cudaMemsetAsync(flags, 0, sizeof(uint32_t) * n, st);
    k_refit<<<div_up(n, T), T, 0, st>>>(prim_lo, prim_hi, vi, (int)n, children, inner_parent, leaf_parent, flags,
                                        node_lo, node_hi, err);
    k_finalize<<<div_up(n - 1, T), T, 0, st>>>(prim_lo, prim_hi, vi, (int)n, children, ranges, node_lo, node_hi,
                                               leaf_max, nodes, node_base, prim_base, err);
    if (depth) k_depth<<<div_up(n, T), T, 0, st>>>(inner_parent, leaf_parent, (int)n, depth);
    return cudaGetLastError();
}

// --- refit of a top-level tree with fixed topology -------------------------
namespace {

// One thread per leaf slot: writes the slot's (enlarged) box into its
// parent's child box and climbs; the second thread to reach a node unites
// the two children's subtree bounds (kept un-enlarged in sub_lo/sub_hi, as
// k_refit keeps them) and continues, so every box is the enlarged union of
// its subtree's primitive boxes, as a fresh build makes it.
__global__ void k_refit_top(BvhNode* nodes, int node_base, const float4* lo_in, const float4* hi_in, uint32_t n,
                            const uint32_t* leaf_parent, const uint32_t* node_parent, uint32_t* flags, float4* sub_lo,
                            float4* sub_hi, uint32_t* err) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float4 lo = lo_in[s], hi = hi_in[s];
    uint32_t p = leaf_parent[s];
    const uint32_t inner = n > 1 ? n - 1 : 1;
    for (uint32_t guard = 0; guard < n + 1; ++guard) {
        const uint32_t node = p >> 1, side = p & 1u;
        if (node >= inner) {
            raise_error(err, DEV_BAD_INDEX);
            return;
        }
        float4 elo = lo, ehi = hi;
        enlarge(elo, ehi);
        BvhNode* nd = nodes + node_base + node;
        if (side == 0) {
            nd->a = make_float4(elo.x, ehi.x, elo.y, ehi.y);
            nd->c.x = elo.z;
            nd->c.y = ehi.z;
        } else {
            nd->b = make_float4(elo.x, ehi.x, elo.y, ehi.y);
            nd->c.z = elo.z;
            nd->c.w = ehi.z;
        }
        sub_lo[2 * node + side] = lo;
        sub_hi[2 * node + side] = hi;
        __threadfence();
        if (atomicAdd(flags + node, 1u) == 0u) return;  // the sibling subtree is not finished
        __threadfence();
        const float4 l0 = __ldcg(sub_lo + 2 * node), l1 = __ldcg(sub_lo + 2 * node + 1);
        const float4 h0 = __ldcg(sub_hi + 2 * node), h1 = __ldcg(sub_hi + 2 * node + 1);
        lo = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.0f);
        hi = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f);
        p = node_parent[node];
        if (p == 0xFFFFFFFFu) return;  // root done
    }
    raise_error(err, DEV_BAD_INDEX);  // a cycle in the parent links
}

}  // namespace

cudaError_t lbvh_refit_top(BvhNode* nodes, int node_base, const float4* leaf_lo, const float4* leaf_hi, uint32_t n,
                           const uint32_t* leaf_parent, const uint32_t* node_parent, uint32_t* flags, float4* sub_lo,
                           float4* sub_hi, uint32_t* err, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(flags, 0, sizeof(uint32_t) * (n > 1 ? n - 1 : 1), st);
    if (e != cudaSuccess) return e;
    k_refit_top<<<div_up(n, 256), 256, 0, st>>>(nodes, node_base, leaf_lo, leaf_hi, n, leaf_parent, node_parent,
                                                flags, sub_lo, sub_hi, err);
    return cudaGetLastError();
}

// --- helpers used by the scene build --------------------------------------
namespace {

__global__ void k_tri_boxes(const float4* pos, const uint32_t* indices, uint32_t vbase, uint32_t ibase, uint32_t ntri,
                            uint32_t nvert, float4* lo, float4* hi, uint32_t* err) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    float4 v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        uint32_t idx = indices[ibase + 3 * t + k];
        if (idx >= nvert) {
            raise_error(err, DEV_BAD_INDEX);
            idx = 0;
        }
        v[k] = pos[vbase + idx];
    }
    lo[t] = make_float4(fminf(fminf(v[0].x, v[1].x), v[2].x), fminf(fminf(v[0].y, v[1].y), v[2].y),
                        fminf(fminf(v[0].z, v[1].z), v[2].z), 0.0f);
    hi[t] = make_float4(fmaxf(fmaxf(v[0].x, v[1].x), v[2].x), fmaxf(fmaxf(v[0].y, v[1].y), v[2].y),
                        fmaxf(fmaxf(v[0].z, v[1].z), v[2].z), 0.0f);
}

// nref leaf positions, each holding one of the mesh's ntri triangles (a
// permutation of them, or with repeats for a tree with spatial splits).
__global__ void k_gather_tris(const float4* pos, const uint32_t* indices, uint32_t vbase, uint32_t ibase,
                              uint32_t nref, uint32_t ntri, uint32_t nvert, const uint32_t* sorted_ids, BvhTri* out) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nref) return;
    uint32_t t = sorted_ids[s];
    if (t >= ntri) t = 0;  // cannot happen: the builders write triangle indices
    float4 v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        uint32_t idx = indices[ibase + 3 * t + k];
        if (idx >= nvert) idx = 0;
        v[k] = pos[vbase + idx];
    }
    BvhTri tr;
    tr.v0 = make_float4(v[0].x, v[0].y, v[0].z, __int_as_float((int)t));
    tr.v1 = make_float4(v[1].x, v[1].y, v[1].z, 0.0f);
    tr.v2 = make_float4(v[2].x, v[2].y, v[2].z, 0.0f);
    out[s] = tr;
}

}  // namespace

cudaError_t build_mesh_blas(const float4* pos, const uint32_t* indices, uint32_t vbase, uint32_t vcount,
                            uint32_t ibase, uint32_t ntri, int leaf_max, BvhNode* nodes, int node_base, BvhTri* tris,
                            int tri_base, float4* box_lo, float4* box_hi, uint32_t* sorted_ids, void* scratch,
                            uint32_t* err, uint32_t* depth, cudaStream_t st) {
    if (ntri == 0) return cudaSuccess;
    const int T = 256;
    k_tri_boxes<<<div_up(ntri, T), T, 0, st>>>(pos, indices, vbase, ibase, ntri, vcount, box_lo, box_hi, err);
    cudaError_t e =
        lbvh_build(box_lo, box_hi, ntri, leaf_max, nodes, node_base, tri_base, sorted_ids, scratch, err, depth, st);
    if (e != cudaSuccess) return e;
    k_gather_tris<<<div_up(ntri, T), T, 0, st>>>(pos, indices, vbase, ibase, ntri, ntri, vcount, sorted_ids,
                                                 tris + tri_base);
    return cudaGetLastError();
}

cudaError_t gather_mesh_tris(const float4* pos, const uint32_t* indices, uint32_t vbase, uint32_t vcount,
                             uint32_t ibase, uint32_t ntri, uint32_t nref, const uint32_t* sorted_ids, BvhTri* tris,
                             cudaStream_t st) {
    if (nref == 0) return cudaSuccess;
    const int T = 256;
    k_gather_tris<<<div_up(nref, T), T, 0, st>>>(pos, indices, vbase, ibase, nref, ntri, vcount, sorted_ids, tris);
    return cudaGetLastError();
}

}  // namespace ddgi

// sah.cu — binned surface-area-heuristic trees, built on the host.
//
// The fast-trace counterpart of the GPU LBVH (lbvh.cu).  The reference asks
// the driver for static bottom-level structures built for trace speed
// (VK_BUILD_ACCELERATION_STRUCTURE_PREFER_FAST_TRACE_BIT_KHR,
// src/Renderer.cpp:334) and for fast builds only for dynamic meshes
// (src/Renderer.cpp:364).  Here a fast-trace tree is a top-down SAH build
// (MacDonald & Booth 1990; binned evaluation after Wald 2007):
//   * ranges of more than kSweepMax primitives: centroids binned into kBins
//     slabs per axis, the split plane with the lowest
//     area(left) x count(left) + area(right) x count(right) chosen, an
//     in-place partition;
//   * smaller ranges: the same cost evaluated at every position of the
//     primitives sorted by centroid along each axis;
//   * no valid plane (all centroids equal): the range is halved.
// Ranges of at most leaf_max primitives become leaves, as in the LBVH, so
// the two builders differ only in the grouping.  Children are built in
// parallel on host threads above kSpawnMin primitives; node numbering is a
// depth-first pass afterwards, so the output does not depend on the thread
// schedule.  Boxes are exact unions (min/max) of the primitive boxes,
// enlarged by the formula of the GPU builder.
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <system_error>
#include <thread>
#include <vector>

#include "sah.h"
#include "traverse.cuh"

namespace ddgi {

namespace {

constexpr int kBins = 32;
constexpr uint32_t kSweepMax = 4096;  // exact sweep below: the top level (instance boxes) gets 1.3 % fewer traversal cycles than with binning at 48
constexpr uint32_t kSpawnMin = 16384;

struct Box {
    float lo[3], hi[3];
    void reset() {
        for (int k = 0; k < 3; ++k) {
            lo[k] = INFINITY;
            hi[k] = -INFINITY;
        }
    }
    void grow(const Box& o) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], o.lo[k]);
            hi[k] = fmaxf(hi[k], o.hi[k]);
        }
    }
    // half the surface area; 0 for an empty or degenerate box
    float half_area() const {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0.0f && dy >= 0.0f && dz >= 0.0f)) return 0.0f;
        const float a = dx * dy + dy * dz + dz * dx;
        return a == a ? a : 0.0f;
    }
};

struct Ref {
    Box box;
    uint32_t id;
    float centroid(int k) const {
        const float c = 0.5f * (box.lo[k] + box.hi[k]);
        return c == c ? c : -INFINITY;  // a NaN centroid sorts and bins first
    }
};

// ref >= 0: another temporary node; ref < 0: ~((first << 3) | (count - 1))
// with first relative to the range of the whole build.
struct TempNode {
    Box box[2];
    int32_t ref[2];
};

void enlarge_host(Box& b) {
    for (int k = 0; k < 3; ++k) {
        const float e = (b.hi[k] - b.lo[k]) * 1e-5f + (std::fabs(b.lo[k]) + std::fabs(b.hi[k])) * 1e-6f + 1e-7f;
        b.lo[k] -= e;
        b.hi[k] += e;
    }
}

class SahBuilder {
  public:
    SahBuilder(const float4* lo, const float4* hi, uint32_t n, int leaf_max)
        : n_(n), leaf_max_((uint32_t)std::max(leaf_max, 1)), refs_(n), temp_(n > 1 ? n - 1 : 1) {
        for (uint32_t i = 0; i < n; ++i) {
            Ref& r = refs_[i];
            r.box.lo[0] = lo[i].x, r.box.lo[1] = lo[i].y, r.box.lo[2] = lo[i].z;
            r.box.hi[0] = hi[i].x, r.box.hi[1] = hi[i].y, r.box.hi[2] = hi[i].z;
            r.id = i;
        }
    }

    // Builds the tree of all n (>= 2) primitives; the root is temporary node 0.
    void run(unsigned threads) {
        next_.store(1);
        build_node(0, 0, n_, std::max(threads, 1u));
    }

    uint32_t write(BvhNode* nodes, uint32_t* order, int node_base, int prim_base) const;

  private:
    const uint32_t n_, leaf_max_;
    std::vector<Ref> refs_;
    std::vector<TempNode> temp_;
    std::atomic<uint32_t> next_{0};

    Box range_box(uint32_t b, uint32_t e) const {
        Box bx;
        bx.reset();
        for (uint32_t i = b; i < e; ++i) bx.grow(refs_[i].box);
        return bx;
    }

    int32_t child(uint32_t b, uint32_t e, unsigned threads) {
        const uint32_t cnt = e - b;
        if (cnt <= leaf_max_) return ~(int32_t)((b << 3) | (cnt - 1));
        const uint32_t id = next_.fetch_add(1);
        build_node(id, b, e, threads);
        return (int32_t)id;
    }

    void build_node(uint32_t id, uint32_t b, uint32_t e, unsigned threads) {
        const uint32_t mid = split(b, e);
        TempNode& t = temp_[id];
        t.box[0] = range_box(b, mid);
        t.box[1] = range_box(mid, e);
        if (threads > 1 && e - b >= kSpawnMin) {
            const unsigned tl = threads / 2, tr = threads - tl;
            int32_t left = 0;
            bool spawned = false;
            std::thread worker;
            try {
                worker = std::thread([&, b, mid, tl]() { left = child(b, mid, tl); });
                spawned = true;
            } catch (const std::system_error&) {
                spawned = false;
            }
            if (!spawned) left = child(b, mid, 1);
            const int32_t right = child(mid, e, spawned ? tr : threads);
            if (spawned) worker.join();
            t.ref[0] = left;
            t.ref[1] = right;
        } else {
            t.ref[0] = child(b, mid, 1);
            t.ref[1] = child(mid, e, 1);
        }
    }

    // Position that splits refs_[b, e) (reordered) into two non-empty parts.
    uint32_t split(uint32_t b, uint32_t e) {
        const uint32_t cnt = e - b;
        if (cnt <= kSweepMax) return sweep_split(b, e);
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t i = b; i < e; ++i)
            for (int k = 0; k < 3; ++k) {
                const float c = refs_[i].centroid(k);
                if (c > -INFINITY && c < INFINITY) {
                    clo[k] = std::min(clo[k], c);
                    chi[k] = std::max(chi[k], c);
                }
            }
        float best = INFINITY;
        int best_axis = -1, best_plane = 0;
        float scale[3] = {0.0f, 0.0f, 0.0f};
        for (int k = 0; k < 3; ++k) {
            const float ext = chi[k] - clo[k];
            if (!(ext > 0.0f) || !(ext < INFINITY)) continue;
            scale[k] = (float)kBins / ext;
            Box bins[kBins];
            uint32_t bc[kBins] = {};
            for (auto& bx : bins) bx.reset();
            for (uint32_t i = b; i < e; ++i) {
                const int j = bin_of(refs_[i].centroid(k), clo[k], scale[k]);
                bins[j].grow(refs_[i].box);
                ++bc[j];
            }
            float right_cost[kBins];
            Box acc;
            acc.reset();
            uint32_t nacc = 0;
            for (int j = kBins - 1; j >= 1; --j) {
                acc.grow(bins[j]);
                nacc += bc[j];
                right_cost[j] = acc.half_area() * (float)nacc;
            }
            acc.reset();
            nacc = 0;
            for (int j = 1; j < kBins; ++j) {
                acc.grow(bins[j - 1]);
                nacc += bc[j - 1];
                if (nacc == 0 || nacc == cnt) continue;
                const float cost = acc.half_area() * (float)nacc + right_cost[j];
                if (cost < best) {
                    best = cost;
                    best_axis = k;
                    best_plane = j;
                }
            }
        }
        if (best_axis < 0) return b + cnt / 2;
        const int k = best_axis;
        const float lo = clo[k], sc = scale[k];
        Ref* first = refs_.data() + b;
        Ref* m = std::partition(first, refs_.data() + e,
                                [&](const Ref& r) { return bin_of(r.centroid(k), lo, sc) < best_plane; });
        const uint32_t mid = (uint32_t)(m - refs_.data());
        return mid > b && mid < e ? mid : b + cnt / 2;
    }

    static int bin_of(float c, float lo, float scale) {
        const float f = (c - lo) * scale;
        if (!(f >= 0.0f)) return 0;  // below the range, NaN or -inf
        return f < (float)(kBins - 1) ? (int)f : kBins - 1;
    }

    uint32_t sweep_split(uint32_t b, uint32_t e) {
        const uint32_t cnt = e - b;
        float best = INFINITY;
        int best_axis = -1;
        uint32_t best_pos = cnt / 2;
        std::vector<float> suffix(cnt + 1);
        for (int k = 0; k < 3; ++k) {
            sort_axis(b, e, k);
            Box acc;
            acc.reset();
            for (uint32_t i = cnt; i >= 1; --i) {
                acc.grow(refs_[b + i - 1].box);
                suffix[i - 1] = acc.half_area();
            }
            acc.reset();
            for (uint32_t i = 1; i < cnt; ++i) {
                acc.grow(refs_[b + i - 1].box);
                const float cost = acc.half_area() * (float)i + suffix[i] * (float)(cnt - i);
                // equal costs (coincident boxes): the more balanced split keeps the tree shallow
                const uint32_t off = i > cnt / 2 ? i - cnt / 2 : cnt / 2 - i;
                const uint32_t best_off = best_pos > cnt / 2 ? best_pos - cnt / 2 : cnt / 2 - best_pos;
                if (cost < best || (cost == best && off < best_off)) {
                    best = cost;
                    best_axis = k;
                    best_pos = i;
                }
            }
        }
        sort_axis(b, e, best_axis >= 0 ? best_axis : 0);
        return b + best_pos;
    }

    void sort_axis(uint32_t b, uint32_t e, int k) {
        std::sort(refs_.begin() + b, refs_.begin() + e, [k](const Ref& x, const Ref& y) {
            const float cx = x.centroid(k), cy = y.centroid(k);
            return cx < cy || (cx == cy && x.id < y.id);
        });
    }
};

uint32_t SahBuilder::write(BvhNode* nodes, uint32_t* order, int node_base, int prim_base) const {
    const uint32_t used = next_.load();
    std::vector<int32_t> newidx(used, -1);
    std::vector<uint32_t> seq;
    seq.reserve(used);
    std::vector<std::pair<uint32_t, uint32_t>> stack{{0u, 1u}};  // (temporary node, depth)
    std::vector<uint32_t> depth_of(used, 0);
    uint32_t depth = 0;
    while (!stack.empty()) {
        const auto [k, d] = stack.back();
        stack.pop_back();
        newidx[k] = (int32_t)seq.size();
        seq.push_back(k);
        depth_of[k] = d;
        depth = std::max(depth, d);
        const TempNode& t = temp_[k];
        if (t.ref[1] >= 0) stack.push_back({(uint32_t)t.ref[1], d + 1});  // second child after the first's subtree
        if (t.ref[0] >= 0) stack.push_back({(uint32_t)t.ref[0], d + 1});
    }
    auto final_ref = [&](int32_t r) {
        if (r >= 0) return node_base + newidx[r];
        const int32_t code = ~r;
        return ~((((code >> 3) + prim_base) << 3) | (code & 7));
    };
    for (size_t i = 0; i < seq.size(); ++i) {
        const TempNode& t = temp_[seq[i]];
        Box b0 = t.box[0], b1 = t.box[1];
        enlarge_host(b0);
        enlarge_host(b1);
        BvhNode& nd = nodes[i];
        nd.a = make_float4(b0.lo[0], b0.hi[0], b0.lo[1], b0.hi[1]);
        nd.b = make_float4(b1.lo[0], b1.hi[0], b1.lo[1], b1.hi[1]);
        nd.c = make_float4(b0.lo[2], b0.hi[2], b1.lo[2], b1.hi[2]);
        nd.d = make_int4(final_ref(t.ref[0]), final_ref(t.ref[1]), 0, 0);
    }
    for (uint32_t s = 0; s < n_; ++s) order[s] = refs_[s].id;
    return depth;
}

void filler(BvhNode& nd) {
    nd.a = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    nd.b = nd.a;
    nd.c = nd.a;
    nd.d = make_int4(kNone, kNone, 0, 0);
}

}  // namespace

bool sah_build(const float4* lo, const float4* hi, uint32_t n, int leaf_max, int node_base, int prim_base,
               BvhNode* nodes, uint32_t* order, uint32_t* depth, unsigned threads) {
    if (n == 0) return false;
    const uint32_t slots = n > 1 ? n - 1 : 1;
    for (uint32_t i = 0; i < slots; ++i) filler(nodes[i]);
    if (n == 1) {
        // one leaf on the left, an empty (never hit) box on the right
        Box b;
        b.lo[0] = lo[0].x, b.lo[1] = lo[0].y, b.lo[2] = lo[0].z;
        b.hi[0] = hi[0].x, b.hi[1] = hi[0].y, b.hi[2] = hi[0].z;
        enlarge_host(b);
        const int32_t leaf = ~(prim_base << 3);
        nodes[0].a = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
        nodes[0].b = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
        nodes[0].c = make_float4(b.lo[2], b.hi[2], INFINITY, -INFINITY);
        nodes[0].d = make_int4(leaf, leaf, 0, 0);
        order[0] = 0;
        *depth = 1;
        return true;
    }
    SahBuilder sb(lo, hi, n, leaf_max);
    sb.run(threads);
    *depth = sb.write(nodes, order, node_base, prim_base);
    return true;
}

}  // namespace ddgi

// sbvh.cu — surface-area-heuristic mesh trees with spatial splits, built on
// the host.
//
// A node is split either by an object split (the binned SAH partition of
// sah.cu: primitives by centroid) or by a spatial split (Stich, Friedrich &
// Dietrich 2009): a plane through the node's box, with the triangles that
// straddle it referenced on both sides, each reference bounded by the part
// of its triangle on that side (tri_split.h: the triangle between the
// plane and the reference's own bounds along the split axis, in float
// interval arithmetic, intersected with the reference's box).  Spatial
// splits are evaluated only where the object split's two children overlap
// by more than `alpha` of the root's surface area, and taken when their SAH
// cost is lower.  Overlapping geometry (the box clusters of the at-scale
// workload) then needs far fewer node visits per ray, at the price of
// triangle references in several leaves; meshes whose triangles do not
// overlap (a height field) are built as by sah.cu.
//
// A ray hit at a point p of a triangle is still found: p lies in the part of
// the triangle on one side of every split plane, so some reference's box
// contains it.  Reference boxes contain the exact parts (every operation of
// the split widened outwards), so box tests stay conservative and the hit
// set equals that of any other tree.  The same triangle may be tested twice
// along a ray; the tie rule (t, instance, primitive) makes that harmless.
// The GPU builder (gbuild.cu) runs this algorithm with the same operations
// and builds the same trees.
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <system_error>
#include <thread>
#include <vector>

#include "sah.h"
#include "traverse.cuh"
#include "tri_split.h"

namespace ddgi {

void sbvh_clip_box(const float* tri, int axis, const float slab_lo[3], const float slab_hi[3], float out_lo[3],
                   float out_hi[3]) {
    tri_split_box(tri, axis, slab_lo, slab_hi, out_lo, out_hi);
}

namespace {

constexpr int kBins = 32;
constexpr size_t kSpawnMin = 8192;   // references of a subtree built on another thread
constexpr int kMaxSplitDepth = 40;   // no spatial split below this depth: the traversal stack stays bounded

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
    bool empty() const { return !(lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2]); }
    float half_area() const {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0.0f && dy >= 0.0f && dz >= 0.0f)) return 0.0f;
        const float a = dx * dy + dy * dz + dz * dx;
        return a == a ? a : 0.0f;
    }
};

Box intersect(const Box& a, const Box& b) {
    Box r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = fmaxf(a.lo[k], b.lo[k]);
        r.hi[k] = fminf(a.hi[k], b.hi[k]);
    }
    return r;
}

struct Ref {
    Box box;
    uint32_t prim;
    float centroid(int k) const {
        const float c = 0.5f * (box.lo[k] + box.hi[k]);
        return c == c ? c : -INFINITY;
    }
};

struct Node {
    Box box[2];
    std::unique_ptr<Node> child[2];
    std::vector<uint32_t> leaf[2];  // primitives of a leaf child
};

void enlarge_host(Box& b) {
    for (int k = 0; k < 3; ++k) {
        const float e = (b.hi[k] - b.lo[k]) * 1e-5f + (std::fabs(b.lo[k]) + std::fabs(b.hi[k])) * 1e-6f + 1e-7f;
        b.lo[k] -= e;
        b.hi[k] += e;
    }
}

Box bounds(const std::vector<Ref>& refs) {
    Box b;
    b.reset();
    for (const Ref& r : refs) b.grow(r.box);
    return b;
}

class Sbvh {
  public:
    Sbvh(const float* tris, int leaf_max, float alpha) : tris_(tris), leaf_max_((size_t)std::max(leaf_max, 1)),
                                                          alpha_(alpha) {}

    std::unique_ptr<Node> run(std::vector<Ref>& refs, unsigned threads) {
        root_area_ = bounds(refs).half_area();
        auto root = std::make_unique<Node>();
        build(root.get(), refs, 1, threads);
        return root;
    }

  private:
    const float* tris_;
    const size_t leaf_max_;
    const float alpha_;
    float root_area_ = 0.0f;

    // Bounds of the triangle's parts below and above the plane x_axis = pl
    // (tri_split.h).
    void plane_split(uint32_t prim, int axis, float pl, Box& below, Box& above) const {
        tri_plane_bounds(tris_ + 9 * (size_t)prim, axis, pl, below.lo, below.hi, above.lo, above.hi);
    }

    static int bin_of(float x, float lo, float scale) {
        const float f = (x - lo) * scale;
        if (!(f >= 0.0f)) return 0;
        return f < (float)(kBins - 1) ? (int)f : kBins - 1;
    }

    // Splits refs (consumed) into left and right, both non-empty.
    void split(std::vector<Ref>& refs, int depth, std::vector<Ref>& L, std::vector<Ref>& R) {
        const size_t n = refs.size();
        const Box nb = bounds(refs);
        // object split: binned SAH over centroids
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (const Ref& r : refs)
            for (int k = 0; k < 3; ++k) {
                const float c = r.centroid(k);
                if (c > -INFINITY && c < INFINITY) {
                    clo[k] = std::min(clo[k], c);
                    chi[k] = std::max(chi[k], c);
                }
            }
        float best = INFINITY;
        int oax = -1, oplane = 0;
        Box obl, obr;
        float oscale = 0.0f;
        for (int k = 0; k < 3; ++k) {
            const float ext = chi[k] - clo[k];
            if (!(ext > 0.0f) || !(ext < INFINITY)) continue;
            const float scale = (float)kBins / ext;
            Box bins[kBins];
            size_t cnt[kBins] = {};
            for (Box& b : bins) b.reset();
            for (const Ref& r : refs) {
                const int j = bin_of(r.centroid(k), clo[k], scale);
                bins[j].grow(r.box);
                ++cnt[j];
            }
            Box right[kBins];
            float rcost[kBins];
            Box acc;
            acc.reset();
            size_t na = 0;
            for (int j = kBins - 1; j >= 1; --j) {
                acc.grow(bins[j]);
                na += cnt[j];
                right[j] = acc;
                rcost[j] = acc.half_area() * (float)na;
            }
            acc.reset();
            na = 0;
            for (int j = 1; j < kBins; ++j) {
                acc.grow(bins[j - 1]);
                na += cnt[j - 1];
                if (na == 0 || na == n) continue;
                const float c = acc.half_area() * (float)na + rcost[j];
                if (c < best) {
                    best = c;
                    oax = k;
                    oplane = j;
                    obl = acc;
                    obr = right[j];
                    oscale = scale;
                }
            }
        }
        // spatial split where the object split's children overlap much
        int sax = -1;
        float splane = 0.0f;
        if (tris_ && alpha_ > 0.0f && oax >= 0 && depth < kMaxSplitDepth &&
            intersect(obl, obr).half_area() > alpha_ * root_area_) {
            float sbest = best;
            for (int k = 0; k < 3; ++k) {
                const float ext = nb.hi[k] - nb.lo[k];
                if (!(ext > 0.0f) || !(ext < INFINITY)) continue;
                const float w = ext / (float)kBins, scale = (float)kBins / ext;
                float plane[kBins + 1];
                for (int j = 0; j <= kBins; ++j) plane[j] = j == kBins ? nb.hi[k] : nb.lo[k] + (float)j * w;
                Box bins[kBins];
                size_t enter[kBins] = {}, leave[kBins] = {};
                for (Box& b : bins) b.reset();
                for (const Ref& r : refs) {
                    const int b0 = bin_of(r.box.lo[k], nb.lo[k], scale), b1 = std::max(b0, bin_of(r.box.hi[k], nb.lo[k], scale));
                    ++enter[b0];
                    ++leave[b1];
                    if (b0 == b1) {
                        bins[b0].grow(r.box);
                        continue;
                    }
                    // bin j: the reference's box, cut to the triangle's part
                    // above bin j's lower plane and below its upper plane
                    Box above;
                    for (int j = b0; j <= b1; ++j) {
                        Box part = r.box;
                        if (j > b0) part = intersect(part, above);
                        if (j < b1) {
                            Box below;
                            plane_split(r.prim, k, plane[j + 1], below, above);
                            part = intersect(part, below);
                        }
                        if (!part.empty()) bins[j].grow(part);
                    }
                }
                float rcost[kBins];
                size_t rcnt[kBins];
                Box acc;
                acc.reset();
                size_t na = 0;
                for (int j = kBins - 1; j >= 1; --j) {
                    acc.grow(bins[j]);
                    na += leave[j];
                    rcost[j] = acc.half_area() * (float)na;
                    rcnt[j] = na;
                }
                acc.reset();
                na = 0;
                for (int j = 1; j < kBins; ++j) {
                    acc.grow(bins[j - 1]);
                    na += enter[j - 1];
                    if (na == 0 || rcnt[j] == 0) continue;
                    const float c = acc.half_area() * (float)na + rcost[j];
                    if (c < sbest) {
                        sbest = c;
                        sax = k;
                        splane = plane[j];
                    }
                }
            }
        }
        if (sax >= 0) {
            for (const Ref& r : refs) {
                if (r.box.hi[sax] <= splane) {
                    L.push_back(r);
                } else if (r.box.lo[sax] >= splane) {
                    R.push_back(r);
                } else {
                    Box below, above;
                    plane_split(r.prim, sax, splane, below, above);
                    const Box a = intersect(r.box, below), b = intersect(r.box, above);
                    if (!a.empty()) L.push_back(Ref{a, r.prim});
                    if (!b.empty()) R.push_back(Ref{b, r.prim});
                    if (a.empty() && b.empty()) L.push_back(r);  // cannot happen for a real triangle
                }
            }
            if (!L.empty() && !R.empty() && L.size() < n + n / 2 && R.size() < n + n / 2) {
                refs.clear();
                refs.shrink_to_fit();
                return;
            }
            L.clear();
            R.clear();
        }
        if (oax >= 0) {
            for (const Ref& r : refs) (bin_of(r.centroid(oax), clo[oax], oscale) < oplane ? L : R).push_back(r);
        }
        if (L.empty() || R.empty()) {  // no valid plane (coincident centroids): halve
            L.assign(refs.begin(), refs.begin() + n / 2);
            R.assign(refs.begin() + n / 2, refs.end());
        }
        refs.clear();
        refs.shrink_to_fit();
    }

    void side(Node* nd, int s, std::vector<Ref>& refs, int depth, unsigned threads) {
        nd->box[s] = bounds(refs);
        if (refs.size() <= leaf_max_) {
            for (const Ref& r : refs) nd->leaf[s].push_back(r.prim);
            refs.clear();
            return;
        }
        nd->child[s] = std::make_unique<Node>();
        build(nd->child[s].get(), refs, depth + 1, threads);
    }

    void build(Node* nd, std::vector<Ref>& refs, int depth, unsigned threads) {
        std::vector<Ref> L, R;
        split(refs, depth, L, R);
        if (threads > 1 && L.size() + R.size() >= kSpawnMin) {
            const unsigned tl = threads / 2, tr = threads - tl;
            std::thread worker;
            bool spawned = false;
            try {
                worker = std::thread([&, nd, depth, tl]() { side(nd, 0, L, depth, tl); });
                spawned = true;
            } catch (const std::system_error&) {
                spawned = false;
            }
            if (!spawned) side(nd, 0, L, depth, 1);
            side(nd, 1, R, depth, spawned ? tr : threads);
            if (spawned) worker.join();
        } else {
            side(nd, 0, L, depth, 1);
            side(nd, 1, R, depth, 1);
        }
    }
};

// Depth-first numbering of the temporary tree into nodes / order.
struct Writer {
    std::vector<BvhNode>& nodes;
    std::vector<uint32_t>& order;
    int node_base, prim_base;
    uint32_t depth = 0;

    int32_t leaf_ref(const std::vector<uint32_t>& prims) {
        const int32_t first = (int32_t)order.size();
        order.insert(order.end(), prims.begin(), prims.end());
        return ~(((first + prim_base) << 3) | ((int32_t)prims.size() - 1));
    }

    int32_t write(const Node* nd, uint32_t d) {
        depth = std::max(depth, d);
        const size_t me = nodes.size();
        nodes.emplace_back();
        int32_t ref[2];
        for (int s = 0; s < 2; ++s)
            ref[s] = nd->child[s] ? write(nd->child[s].get(), d + 1) : leaf_ref(nd->leaf[s]);
        Box b0 = nd->box[0], b1 = nd->box[1];
        enlarge_host(b0);
        enlarge_host(b1);
        BvhNode& out = nodes[me];
        out.a = make_float4(b0.lo[0], b0.hi[0], b0.lo[1], b0.hi[1]);
        out.b = make_float4(b1.lo[0], b1.hi[0], b1.lo[1], b1.hi[1]);
        out.c = make_float4(b0.lo[2], b0.hi[2], b1.lo[2], b1.hi[2]);
        out.d = make_int4(ref[0], ref[1], 0, 0);
        return node_base + (int32_t)me;
    }
};

}  // namespace

bool sbvh_build(const float* tris, uint32_t n, int leaf_max, float alpha, int node_base, int prim_base,
                std::vector<BvhNode>& nodes, std::vector<uint32_t>& order, uint32_t* depth, unsigned threads) {
    nodes.clear();
    order.clear();
    if (n == 0) return false;
    std::vector<Ref> refs(n);
    for (uint32_t i = 0; i < n; ++i) {
        const float* t = tris + 9 * (size_t)i;
        Box& b = refs[i].box;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = fminf(fminf(t[k], t[3 + k]), t[6 + k]);
            b.hi[k] = fmaxf(fmaxf(t[k], t[3 + k]), t[6 + k]);
        }
        refs[i].prim = i;
    }
    if (n == 1) {
        // one leaf on the left, an empty (never hit) box on the right
        Box b = refs[0].box;
        enlarge_host(b);
        const int32_t leaf = ~(prim_base << 3);
        BvhNode nd;
        nd.a = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
        nd.b = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
        nd.c = make_float4(b.lo[2], b.hi[2], INFINITY, -INFINITY);
        nd.d = make_int4(leaf, leaf, 0, 0);
        nodes.push_back(nd);
        order.push_back(0);
        *depth = 1;
        return true;
    }
    Sbvh builder(tris, leaf_max, alpha);
    std::unique_ptr<Node> root = builder.run(refs, std::max(threads, 1u));
    Writer w{nodes, order, node_base, prim_base};
    w.write(root.get(), 1);
    *depth = w.depth;
    return true;
}

}  // namespace ddgi

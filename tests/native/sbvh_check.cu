// Host-only check of the spatial-split tree builder (vulkanexp_gb300/csrc/sbvh.cu),
// run under AddressSanitizer / UndefinedBehaviorSanitizer by tests/test_native_host.py
// (and with the argument `threads`, inputs that build subtrees on other
// threads, under ThreadSanitizer).
// For overlapping box soups (also nearly axis-aligned ones, whose faces the
// split planes cut at grazing angles) and a height field: every triangle is referenced,
// references and leaf ranges stay in bounds, the depth is reported correctly,
// and the tree is conservative: for sample points of every triangle (vertices,
// edge midpoints, centroid, random interior points) a descent through the
// children whose stored boxes contain the point reaches a leaf holding it.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <array>
#include <random>
#include <vector>

#include "../../vulkanexp_gb300/csrc/sah.h"
#include "../../vulkanexp_gb300/csrc/traverse.cuh"

using namespace ddgi;

static int failures = 0;

static bool contains(const BvhNode& nd, int side, const float p[3]) {
    const float lo[3] = {side ? nd.b.x : nd.a.x, side ? nd.b.z : nd.a.z, side ? nd.c.z : nd.c.x};
    const float hi[3] = {side ? nd.b.y : nd.a.y, side ? nd.b.w : nd.a.w, side ? nd.c.w : nd.c.y};
    for (int k = 0; k < 3; ++k)
        if (!(lo[k] <= p[k] && p[k] <= hi[k])) return false;
    return true;
}

static bool reaches(const std::vector<BvhNode>& nodes, const std::vector<uint32_t>& order, int node_base,
                    int prim_base, int ref, const float p[3], uint32_t tri) {
    std::vector<int> stack{ref};
    while (!stack.empty()) {
        const int r = stack.back();
        stack.pop_back();
        const BvhNode& nd = nodes[(size_t)(r - node_base)];
        const int refs[2] = {nd.d.x, nd.d.y};
        for (int s = 0; s < 2; ++s) {
            if (!contains(nd, s, p)) continue;
            if (refs[s] >= 0) {
                stack.push_back(refs[s]);
            } else {
                const int code = ~refs[s], first = (code >> 3) - prim_base, cnt = (code & 7) + 1;
                for (int q = first; q < first + cnt; ++q)
                    if (order[(size_t)q] == tri) return true;
            }
        }
    }
    return false;
}

static void check(const char* name, const std::vector<float>& tris, int leaf_max, float alpha, int samples = 4) {
    const uint32_t n = (uint32_t)(tris.size() / 9);
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> order;
    uint32_t depth = 0;
    const int node_base = 5, prim_base = 3;
    if (!sbvh_build(tris.data(), n, leaf_max, alpha, node_base, prim_base, nodes, order, &depth, 4)) {
        std::printf("FAIL %s: build\n", name);
        ++failures;
        return;
    }
    std::vector<int> seen(n, 0);
    for (uint32_t t : order) {
        if (t >= n) {
            std::printf("FAIL %s: order entry %u\n", name, t);
            ++failures;
            return;
        }
        seen[t]++;
    }
    for (uint32_t t = 0; t < n; ++t)
        if (!seen[t]) {
            std::printf("FAIL %s: triangle %u unreferenced\n", name, t);
            ++failures;
            return;
        }
    // structure: refs in range, each node reached once, depth
    std::vector<int> reached(nodes.size(), 0);
    std::vector<std::pair<int, uint32_t>> st{{node_base, 1}};
    uint32_t maxd = 0;
    while (!st.empty()) {
        auto [r, d] = st.back();
        st.pop_back();
        const int k = r - node_base;
        if (k < 0 || (size_t)k >= nodes.size() || reached[(size_t)k]++) {
            std::printf("FAIL %s: bad or repeated node %d\n", name, r);
            ++failures;
            return;
        }
        maxd = std::max(maxd, d);
        const int refs[2] = {nodes[(size_t)k].d.x, nodes[(size_t)k].d.y};
        for (int s = 0; s < 2; ++s) {
            if (refs[s] >= 0) {
                st.push_back({refs[s], d + 1});
            } else {
                const int code = ~refs[s], first = (code >> 3) - prim_base, cnt = (code & 7) + 1;
                if (first < 0 || (size_t)(first + cnt) > order.size() || cnt > leaf_max) {
                    std::printf("FAIL %s: leaf range\n", name);
                    ++failures;
                    return;
                }
            }
        }
    }
    if (maxd != depth) {
        std::printf("FAIL %s: depth %u, longest chain %u\n", name, depth, maxd);
        ++failures;
        return;
    }
    // conservativeness at sample points of every triangle
    std::mt19937 rng(3);
    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    for (uint32_t t = 0; t < n; ++t) {
        const float* v = &tris[9 * (size_t)t];
        std::vector<std::array<float, 3>> pts;
        for (int i = 0; i < 3; ++i) pts.push_back({v[3 * i], v[3 * i + 1], v[3 * i + 2]});
        for (int i = 0; i < 3; ++i) {
            const int j = (i + 1) % 3;
            pts.push_back({0.5f * (v[3 * i] + v[3 * j]), 0.5f * (v[3 * i + 1] + v[3 * j + 1]),
                           0.5f * (v[3 * i + 2] + v[3 * j + 2])});
        }
        for (int s = 0; s < samples; ++s) {
            float a = U(rng), b = U(rng);
            if (a + b > 1.0f) a = 1.0f - a, b = 1.0f - b;
            const float c = 1.0f - a - b;
            pts.push_back({c * v[0] + a * v[3] + b * v[6], c * v[1] + a * v[4] + b * v[7], c * v[2] + a * v[5] + b * v[8]});
        }
        for (const auto& p : pts) {
            if (!reaches(nodes, order, node_base, prim_base, node_base, p.data(), t)) {
                std::printf("FAIL %s: point (%g %g %g) of triangle %u not reached\n", name, p[0], p[1], p[2], t);
                ++failures;
                return;
            }
        }
    }
    std::printf("ok %s: %u triangles, %zu references (+%.0f %%), %zu nodes, depth %u\n", name, n, order.size(),
                100.0 * ((double)order.size() - n) / n, nodes.size(), depth);
}

// Boxes with random centres, sizes and yaw; near_aligned: yaw within
// +-[1e-6, 1e-3] rad, so faces are nearly parallel to the split planes and
// clipping them is ill-conditioned.
static std::vector<float> box_soup(std::mt19937& rng, int boxes, float extent, bool near_aligned = false) {
    std::uniform_real_distribution<float> C(-extent, extent), S(0.05f, 0.6f), Y(0.0f, 6.2831853f);
    std::uniform_real_distribution<float> L(-6.0f, -3.0f);
    static const int f[12][3] = {{0, 2, 1}, {0, 3, 2}, {4, 5, 6}, {4, 6, 7}, {0, 1, 5}, {0, 5, 4},
                                 {2, 3, 7}, {2, 7, 6}, {1, 2, 6}, {1, 6, 5}, {0, 4, 7}, {0, 7, 3}};
    std::vector<float> out;
    for (int b = 0; b < boxes; ++b) {
        const float cx = C(rng), cy = C(rng) * 0.5f + extent * 0.5f, cz = C(rng);
        float yaw = Y(rng);
        if (near_aligned) yaw = (yaw < 3.14159265f ? 1.0f : -1.0f) * std::pow(10.0f, L(rng));
        const float sx = S(rng), sy = S(rng), sz = S(rng), cs = std::cos(yaw), sn = std::sin(yaw);
        float corner[8][3];
        for (int i = 0; i < 8; ++i) {
            const float x = (i & 1) ? sx : -sx, y = (i & 2) ? sy : -sy, z = (i & 4) ? sz : -sz;
            corner[i][0] = cx + cs * x + sn * z;
            corner[i][1] = cy + y;
            corner[i][2] = cz - sn * x + cs * z;
        }
        for (const auto& tri : f)
            for (int v = 0; v < 3; ++v)
                for (int k = 0; k < 3; ++k) out.push_back(corner[tri[v]][k]);
    }
    return out;
}

static std::vector<float> height_field(std::mt19937& rng, int cells, float size) {
    std::uniform_real_distribution<float> H(0.0f, 2.0f);
    std::vector<float> h((size_t)(cells + 1) * (cells + 1));
    for (float& x : h) x = H(rng);
    const float st = size / (float)cells;
    std::vector<float> out;
    auto P = [&](int i, int j, int k) { return k == 0 ? i * st : (k == 1 ? h[(size_t)i * (cells + 1) + j] : j * st); };
    for (int i = 0; i < cells; ++i)
        for (int j = 0; j < cells; ++j) {
            const int tri[2][3][2] = {{{i, j}, {i, j + 1}, {i + 1, j}}, {{i + 1, j}, {i, j + 1}, {i + 1, j + 1}}};
            for (const auto& t : tri)
                for (const auto& v : t)
                    for (int k = 0; k < 3; ++k) out.push_back(P(v[0], v[1], k));
        }
    return out;
}

// The clipped reference box against the exact geometry: triangles nearly
// parallel to a coordinate plane (thickness 1e-6 .. 1e-3 of their size along
// that axis) cut by a plane through them; every point of the triangle (in
// double) on either side of the plane lies in that side's clipped box.  (A
// sequential float polygon clipper was off by up to 1e-3 of an edge here.)
static void check_clip(std::mt19937& rng, int cases) {
    std::uniform_real_distribution<double> U(0.0, 1.0), C(-3.0, 3.0);
    std::uniform_real_distribution<double> L(-6.0, -3.0);
    double worst = 0.0;
    for (int c = 0; c < cases; ++c) {
        const int k = c % 3;
        const double thick = std::pow(10.0, L(rng)), base = C(rng);
        float tri[9];
        for (int v = 0; v < 3; ++v)
            for (int j = 0; j < 3; ++j) tri[3 * v + j] = (float)(j == k ? base + thick * U(rng) : C(rng));
        const double klo = std::min({(double)tri[k], (double)tri[3 + k], (double)tri[6 + k]});
        const double khi = std::max({(double)tri[k], (double)tri[3 + k], (double)tri[6 + k]});
        const float plane = (float)(klo + (khi - klo) * U(rng));
        // the node's slab also cuts the triangle in the other two axes (the
        // clipper's earlier planes: their rounded crossing points feed the
        // grazing cut)
        float nlo[3], nhi[3];
        for (int j = 0; j < 3; ++j) {
            const double tlo = std::min({(double)tri[j], (double)tri[3 + j], (double)tri[6 + j]});
            const double thi = std::max({(double)tri[j], (double)tri[3 + j], (double)tri[6 + j]});
            nlo[j] = j == k ? -1e30f : (float)(tlo + 0.3 * (thi - tlo) * U(rng));
            nhi[j] = j == k ? 1e30f : (float)(thi - 0.3 * (thi - tlo) * U(rng));
        }
        float lo[2][3], hi[2][3];
        for (int side = 0; side < 2; ++side) {
            float slo[3] = {nlo[0], nlo[1], nlo[2]}, shi[3] = {nhi[0], nhi[1], nhi[2]};
            if (side == 0) shi[k] = plane;
            else slo[k] = plane;
            sbvh_clip_box(tri, k, slo, shi, lo[side], hi[side]);
        }
        for (int s = 0; s < 2000; ++s) {
            double a = U(rng), b = U(rng);
            if (a + b > 1.0) a = 1.0 - a, b = 1.0 - b;
            double p[3];
            for (int j = 0; j < 3; ++j)
                p[j] = (1.0 - a - b) * tri[j] + a * (double)tri[3 + j] + b * (double)tri[6 + j];
            bool inside = true;
            for (int j = 0; j < 3; ++j)
                if (j != k && !(nlo[j] <= p[j] && p[j] <= nhi[j])) inside = false;
            if (!inside) continue;
            for (int side = 0; side < 2; ++side) {
                if (side == 0 ? !(p[k] <= plane) : !(p[k] >= plane)) continue;
                for (int j = 0; j < 3; ++j) {
                    const double out = std::max(lo[side][j] - p[j], p[j] - hi[side][j]);
                    worst = std::max(worst, out);
                    if (out > 1e-9) {
                        std::printf("FAIL clip: case %d axis %d, point outside the side-%d box by %g in axis %d\n",
                                    c, k, side, out, j);
                        ++failures;
                        return;
                    }
                }
            }
        }
    }
    std::printf("ok clip: %d grazing cuts, worst excursion %g\n", cases, worst);
}

int main(int argc, char** argv) {
    std::mt19937 rng(7);
    if (argc > 1 && std::strcmp(argv[1], "threads") == 0) {
        // inputs above the 8,192 references that send a subtree to another
        // thread, one sample point per triangle (for the race detector run)
        check("threaded box soup", box_soup(rng, 1200, 2.0f), 2, 1e-2f, 1);
        check("threaded height field", height_field(rng, 100, 30.0f), 2, 1e-2f, 1);
        std::printf(failures ? "FAILED %d\n" : "all ok\n", failures);
        return failures ? 1 : 0;
    }
    const int scale = argc > 1 ? std::atoi(argv[1]) : 1;
    for (float alpha : {1e-2f, 1e-5f, 0.0f}) {
        char name[64];
        std::snprintf(name, sizeof name, "box soup alpha=%g", alpha);
        check(name, box_soup(rng, 300 * scale, 2.0f), 2, alpha);
    }
    check("box soup leaf 1", box_soup(rng, 200 * scale, 1.0f), 1, 1e-2f);
    check("box soup leaf 4", box_soup(rng, 200 * scale, 1.0f), 4, 1e-2f);
    check("height field", height_field(rng, 40 * scale, 30.0f), 2, 1e-2f);
    // faces nearly parallel to the split planes, dense interior sampling
    check("near-aligned box soup", box_soup(rng, 600 * scale, 1.5f, true), 2, 1e-3f, 256);
    check("one triangle", box_soup(rng, 1, 1.0f), 2, 1e-2f);
    check_clip(rng, 3000 * scale);
    std::printf(failures ? "FAILED %d\n" : "all ok\n", failures);
    return failures ? 1 : 0;
}

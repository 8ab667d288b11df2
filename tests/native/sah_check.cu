// Host-only structural check of the SAH tree builder (vulkanexp_gb300/csrc/sah.cu),
// run under AddressSanitizer / UndefinedBehaviorSanitizer and under ThreadSanitizer
// (its 40,000-box case builds subtrees on other threads) by tests/test_native_host.py.
// For each case: every leaf position appears in exactly one leaf, `order` is a
// permutation, every child box contains the boxes of all primitives below it,
// references stay inside the node range, the reported depth is the longest
// root-to-leaf chain of inner nodes, and unused slots are never-hit fillers.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "../../vulkanexp_gb300/csrc/sah.h"
#include "../../vulkanexp_gb300/csrc/traverse.cuh"

using namespace ddgi;

static int failures = 0;
#define CHECK(c, ...)                          \
    do {                                       \
        if (!(c)) {                            \
            std::printf("FAIL: " __VA_ARGS__); \
            std::printf("\n");                 \
            ++failures;                        \
            return;                            \
        }                                      \
    } while (0)

static bool inside(float lo, float hi, float plo, float phi) {
    // a primitive box with a NaN coordinate on this axis constrains nothing
    // there (such a primitive can never be hit; the scene build refuses
    // non-finite vertices, this case only checks that the builder copes)
    if (!(plo == plo) || !(phi == phi)) return true;
    return lo <= plo && phi <= hi;
}

static void check_case(const char* name, const std::vector<float4>& lo, const std::vector<float4>& hi, int leaf_max,
                       int node_base, int prim_base) {
    const uint32_t n = (uint32_t)lo.size();
    std::vector<BvhNode> nodes(n > 1 ? n - 1 : 1);
    std::vector<uint32_t> order(n, 0xFFFFFFFFu);
    uint32_t depth = 0;
    CHECK(sah_build(lo.data(), hi.data(), n, leaf_max, node_base, prim_base, nodes.data(), order.data(), &depth, 4),
          "%s: build failed", name);
    std::vector<int> seen_prim(n, 0), seen_pos(n, 0), seen_node(nodes.size(), 0);
    for (uint32_t s = 0; s < n; ++s) {
        CHECK(order[s] < n, "%s: order[%u] out of range", name, s);
        seen_prim[order[s]]++;
    }
    for (uint32_t i = 0; i < n; ++i) CHECK(seen_prim[i] == 1, "%s: primitive %u placed %d times", name, i, seen_prim[i]);
    // walk: (node, depth)
    std::vector<std::pair<int, uint32_t>> stack{{0, 1}};
    uint32_t maxd = 0;
    while (!stack.empty()) {
        auto [k, d] = stack.back();
        stack.pop_back();
        CHECK(k >= 0 && (size_t)k < nodes.size(), "%s: node %d out of range", name, k);
        CHECK(seen_node[k]++ == 0, "%s: node %d reached twice", name, k);
        maxd = d > maxd ? d : maxd;
        const BvhNode& nd = nodes[k];
        const int refs[2] = {nd.d.x, nd.d.y};
        const float blo[2][3] = {{nd.a.x, nd.a.z, nd.c.x}, {nd.b.x, nd.b.z, nd.c.z}};
        const float bhi[2][3] = {{nd.a.y, nd.a.w, nd.c.y}, {nd.b.y, nd.b.w, nd.c.w}};
        for (int side = 0; side < 2; ++side) {
            if (n == 1 && side == 1) continue;  // the empty right side of a one-primitive tree
            // primitives below this child
            std::vector<int> st2{refs[side]};
            while (!st2.empty()) {
                int r = st2.back();
                st2.pop_back();
                if (r >= 0) {
                    const int c = r - node_base;
                    CHECK(c >= 0 && (size_t)c < nodes.size(), "%s: child %d out of range", name, r);
                    st2.push_back(nodes[c].d.x);
                    st2.push_back(nodes[c].d.y);
                } else {
                    const int code = ~r, first = (code >> 3) - prim_base, cnt = (code & 7) + 1;
                    CHECK(first >= 0 && (uint32_t)(first + cnt) <= n, "%s: leaf range out of bounds", name);
                    CHECK(cnt <= leaf_max || leaf_max < 1, "%s: leaf of %d > %d", name, cnt, leaf_max);
                    for (int q = first; q < first + cnt; ++q) {
                        const uint32_t p = order[q];
                        const float pl[3] = {lo[p].x, lo[p].y, lo[p].z}, ph[3] = {hi[p].x, hi[p].y, hi[p].z};
                        for (int a = 0; a < 3; ++a)
                            CHECK(inside(blo[side][a], bhi[side][a], pl[a], ph[a]),
                                  "%s: primitive %u outside its box on axis %d", name, p, a);
                    }
                }
            }
            if (refs[side] >= 0) stack.push_back({refs[side] - node_base, d + 1});
            else if (!(n == 1 && side == 1)) {
                const int code = ~refs[side], first = (code >> 3) - prim_base, cnt = (code & 7) + 1;
                for (int q = first; q < first + cnt; ++q) seen_pos[q]++;
            }
        }
    }
    for (uint32_t s = 0; s < n; ++s) CHECK(seen_pos[s] == 1, "%s: leaf position %u in %d leaves", name, s, seen_pos[s]);
    CHECK(depth == maxd, "%s: depth %u, longest chain %u", name, depth, maxd);
    for (size_t k = 0; k < nodes.size(); ++k)
        if (!seen_node[k]) CHECK(nodes[k].d.x == kNone && nodes[k].d.y == kNone, "%s: slot %zu not a filler", name, k);
    std::printf("ok %s: %u primitives, depth %u\n", name, n, depth);
}

int main() {
    std::mt19937 rng(5);
    std::uniform_real_distribution<float> U(-50.0f, 50.0f), S(0.0f, 2.0f);
    auto boxes = [&](uint32_t n, std::vector<float4>& lo, std::vector<float4>& hi) {
        lo.resize(n);
        hi.resize(n);
        for (uint32_t i = 0; i < n; ++i) {
            float c[3] = {U(rng), U(rng), U(rng)}, e[3] = {S(rng), S(rng), S(rng)};
            lo[i] = make_float4(c[0] - e[0], c[1] - e[1], c[2] - e[2], 0);
            hi[i] = make_float4(c[0] + e[0], c[1] + e[1], c[2] + e[2], 0);
        }
    };
    std::vector<float4> lo, hi;
    for (uint32_t n : {1u, 2u, 3u, 5u, 47u, 48u, 49u, 1000u, 40000u}) {
        for (int leaf : {1, 2, 4, 8}) {
            boxes(n, lo, hi);
            char name[64];
            std::snprintf(name, sizeof name, "random n=%u leaf=%d", n, leaf);
            check_case(name, lo, hi, leaf, 7, 11);
        }
    }
    // every centroid equal (no valid plane: halving), and a flat layer
    boxes(3000, lo, hi);
    for (auto& v : lo) v = make_float4(1, 2, 3, 0);
    for (auto& v : hi) v = make_float4(1, 2, 3, 0);
    check_case("identical boxes", lo, hi, 2, 0, 0);
    boxes(3000, lo, hi);
    for (size_t i = 0; i < lo.size(); ++i) lo[i].y = hi[i].y = 0.0f;
    check_case("flat layer", lo, hi, 2, 0, 0);
    // NaN and infinite coordinates must not break the build
    boxes(2000, lo, hi);
    for (size_t i = 0; i < lo.size(); i += 7) lo[i].x = NAN;
    for (size_t i = 3; i < lo.size(); i += 11) hi[i].z = INFINITY;
    check_case("nan and inf", lo, hi, 2, 0, 0);
    std::printf(failures ? "FAILED %d\n" : "all ok\n", failures);
    return failures ? 1 : 0;
}

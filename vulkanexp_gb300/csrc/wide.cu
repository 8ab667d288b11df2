// wide.cu — eight-wide quantised trees collapsed from the binary trees.
//
// A wide node starts from a binary node's two children; while it has fewer
// than eight, the inner child with the largest surface area is replaced by
// its two children (the greedy collapse of Wald, Benthin & Boulos 2008 /
// Ylitie, Karras & Laine 2017).  Leaf children keep their binary leaf
// references, inner children become wide nodes (laid out parent before
// children).  Empty boxes (the unused side of a one-primitive tree) are
// dropped.
//
// The children's boxes (the binary tree's enlarged boxes) are quantised per
// axis to 8 bits on a power-of-two grid anchored at the union's lower corner,
// lower bounds rounded down and upper bounds up, checked in double against
// the float boxes, so every quantised box contains the binary one: box tests
// stay at least as conservative as the binary tree's and the hit set is the
// same.  Slots are assigned by the octant the child's centre lies in
// relative to the node's centre (bit k set: low side of axis k), greedily
// by how far along that octant's diagonal the centre lies, so that visiting
// slots in decreasing (slot ^ ray octant) order approximates near-first.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/ddgi_exact.h"
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

double half_area(const Slot& s) {
    const double dx = (double)s.hi[0] - s.lo[0], dy = (double)s.hi[1] - s.lo[1], dz = (double)s.hi[2] - s.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

void set_byte(uint4& w, int idx, uint32_t v) {  // byte idx (0..15) of the 16-byte word
    uint32_t* p = &w.x + (idx >> 2);
    const int sh = 8 * (idx & 3);
    *p = (*p & ~(0xFFu << sh)) | (v << sh);
}

// Quantises the slots' boxes into n (grid and bounds); false if a box cannot
// be enclosed (non-finite bounds).
bool quantise(const Slot* slots, const int* slot_of, int ns, WideNode& n) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < ns; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], slots[i].lo[a]);
            hi[a] = std::max(hi[a], slots[i].hi[a]);
        }
    uint32_t ebits = 0;
    for (int a = 0; a < 3; ++a) {
        if (!std::isfinite(lo[a]) || !std::isfinite(hi[a])) return false;
        const double ext = (double)hi[a] - (double)lo[a];
        int e = -126;
        if (ext > 0.0) {
            e = (int)std::ceil(std::log2(ext / 255.0));
            e = std::max(-126, std::min(127, e));
            while (e < 127 && std::ldexp(255.0, e) < ext) ++e;
            while (e > -126 && std::ldexp(255.0, e - 1) >= ext) --e;
        }
        if (std::ldexp(255.0, e) < ext) return false;
        ebits |= (uint32_t)(e + 127) << (8 * a);
        const double step = std::ldexp(1.0, e), p = (double)lo[a];
        for (int k = 0; k < 16; ++k) set_byte(n.q[a], k, k < 8 ? 255u : 0u);  // empty slots: lo 255, hi 0
        for (int i = 0; i < ns; ++i) {
            const int s = slot_of[i];
            double ql = std::floor(((double)slots[i].lo[a] - p) / step);
            double qh = std::ceil(((double)slots[i].hi[a] - p) / step);
            ql = std::max(0.0, std::min(255.0, ql));
            qh = std::max(0.0, std::min(255.0, qh));
            while (ql > 0.0 && p + ql * step > (double)slots[i].lo[a]) ql -= 1.0;
            while (qh < 255.0 && p + qh * step < (double)slots[i].hi[a]) qh += 1.0;
            if (p + ql * step > (double)slots[i].lo[a] || p + qh * step < (double)slots[i].hi[a]) return false;
            set_byte(n.q[a], s, (uint32_t)ql);
            set_byte(n.q[a], 8 + s, (uint32_t)qh);
        }
    }
    n.org = make_float4(lo[0], lo[1], lo[2], ddgi_bits_float(ebits));
    return true;
}

// Slot of each child: octant of its centre around the node's centre (bit k:
// low side of axis k), greedily by the projection onto that octant's
// diagonal (most extreme first).
void assign_slots(const Slot* slots, int ns, int* slot_of) {
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < ns; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], (double)slots[i].lo[a]);
            hi[a] = std::max(hi[a], (double)slots[i].hi[a]);
        }
    struct Cand {
        double cost;
        int child, slot;
    };
    std::vector<Cand> cands;
    for (int i = 0; i < ns; ++i)
        for (int s = 0; s < 8; ++s) {
            double cost = 0.0;
            for (int a = 0; a < 3; ++a) {
                const double d = 0.5 * ((double)slots[i].lo[a] + (double)slots[i].hi[a]) - 0.5 * (lo[a] + hi[a]);
                cost += ((s >> a) & 1) ? d : -d;  // low side wanted: negative d is good
            }
            cands.push_back({cost, i, s});
        }
    std::stable_sort(cands.begin(), cands.end(), [](const Cand& x, const Cand& y) { return x.cost < y.cost; });
    bool child_done[8] = {}, slot_used[8] = {};
    for (int i = 0; i < ns; ++i) slot_of[i] = -1;
    for (const Cand& c : cands) {
        if (child_done[c.child] || slot_used[c.slot]) continue;
        child_done[c.child] = slot_used[c.slot] = true;
        slot_of[c.child] = c.slot;
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
        Slot slots[8];
        int ns = 0;
        for (int side = 0; side < 2; ++side) {
            Slot c;
            child_slot(bin[(size_t)w.bin], side, &c);
            if (!box_empty(c.lo, c.hi)) slots[ns++] = c;
        }
        for (;;) {  // open the largest inner child while a slot is free
            int best = -1;
            double area = -1.0;
            for (int i = 0; i < ns; ++i)
                if (slots[i].ref >= 0 && half_area(slots[i]) > area) {
                    area = half_area(slots[i]);
                    best = i;
                }
            if (best < 0) break;
            if ((size_t)slots[best].ref >= bin.size()) {
                *ok = false;
                return wroot;
            }
            Slot kids[2];
            int nk = 0;
            for (int side = 0; side < 2; ++side) {
                Slot g;
                child_slot(bin[(size_t)slots[best].ref], side, &g);
                if (!box_empty(g.lo, g.hi)) kids[nk++] = g;
            }
            if (ns - 1 + nk > 8) break;
            slots[best] = slots[ns - 1];
            --ns;
            for (int k = 0; k < nk; ++k) slots[ns++] = kids[k];
        }
        WideNode n;
        int slot_of[8];
        assign_slots(slots, ns, slot_of);
        if (!quantise(slots, slot_of, ns, n)) {
            *ok = false;
            return wroot;
        }
        int refs[8];
        for (int k = 0; k < 8; ++k) refs[k] = kNone;
        for (int i = 0; i < ns; ++i) {
            if (slots[i].ref >= 0) {
                const int nw = (int)out.size();
                out.emplace_back();
                work.push_back({slots[i].ref, nw, w.level + 1});
                refs[slot_of[i]] = nw;
            } else {
                refs[slot_of[i]] = slots[i].ref;
            }
        }
        n.ref[0] = make_int4(refs[0], refs[1], refs[2], refs[3]);
        n.ref[1] = make_int4(refs[4], refs[5], refs[6], refs[7]);
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
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        int r[4] = {w.ref[h].x, w.ref[h].y, w.ref[h].z, w.ref[h].w};
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
        w.ref[h] = make_int4(r[0], r[1], r[2], r[3]);
    }
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

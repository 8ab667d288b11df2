// traverse.cuh — two-level LBVH traversal (closest hit and any hit).
//
// The top-level tree is walked in world space; at an instance leaf an EXIT
// marker is pushed, the ray moves into object space through the instance's
// world-to-object transform and the mesh tree is walked; popping the marker
// restores the world ray.  Hits are accepted for t in [tmin, tmax]; among
// equal t the lowest (instance, primitive) wins, so the result does not
// depend on the visiting order.
#pragma once

#include "common.cuh"

namespace ddgi {

constexpr int kStack = 64;
constexpr int kExit = 0x7fffffff;
constexpr int kNone = (int)0x80000000;  // no node (never a valid reference)
constexpr uint32_t kNoHit = 0xFFFFFFFFu;
// Box tests use [tmin * kBoxLo, tcur * kBoxHi]: a relative margin far above
// the few-ulp error of slab and triangle distances, so that pruning never
// removes a box holding a hit the triangle test reports, at any ray length.
constexpr float kBoxLo = 0.99999f;
constexpr float kBoxHi = 1.00001f;

struct HitRec {
    float t, b1, b2;
    uint32_t inst, prim;
    bool back;
};

// Fetch counters of the measurement variant (COUNT = true): inner nodes
// visited, triangles tested, instances entered, rays traced (index 0 for
// closest-hit rays, 1 for any-hit rays), and shading bytes.
struct Fetches {
    uint32_t nodes[2] = {0, 0}, tris[2] = {0, 0}, insts[2] = {0, 0}, rays[2] = {0, 0}, shade_bytes = 0;
    uint32_t top_nodes[2] = {0, 0};  // the part of `nodes` in the top-level tree
};

// Closest hit (ANY = false) or any hit (ANY = true) with t in [tmin, tmax];
// ties on t go to the lowest (instance, primitive).
template <bool ANY, bool COUNT = false>
__device__ __forceinline__ bool traverse(const DeviceScene& sc, float3 wo, float3 wd, float tmin, float tmax,
                                         uint32_t mask, HitRec* best, uint32_t* err, Fetches* fc = nullptr) {
    if (COUNT) fc->rays[ANY]++;
    best->inst = kNoHit;
    best->prim = 0;
    best->t = tmax;
    best->b1 = best->b2 = 0.0f;
    best->back = false;
    if (sc.tlas_root < 0) return false;
    Ray r;
    ray_setup(r, wo, wd);
    int stack[kStack];
    int sp = 0;
    int ref = sc.tlas_root;
    bool in_blas = false;
    uint32_t inst_id = 0;
    float tcur = tmax;
    // A well-formed tree visits each node at most once per ray; the cap only
    // stops a malformed one from looping.
    for (uint32_t steps = 0;; ++steps) {
        if (steps > 4u * (sc.node_count + sc.tri_count + sc.instance_count) + 64u) {
            raise_error(err, DEV_BAD_INDEX);
            return best->inst != kNoHit;
        }
        if (ref >= 0) {
            if (COUNT) {
                fc->nodes[ANY]++;
                if (!in_blas) fc->top_nodes[ANY]++;
            }
            if ((uint32_t)ref >= sc.node_count) {
                raise_error(err, DEV_BAD_INDEX);
                return best->inst != kNoHit;
            }
            BvhNode n = load_node(sc.nodes, ref);
            bool h0, h1;
            float t0, t1;
            node_hit(r, n, tmin * kBoxLo, tcur * kBoxHi, &h0, &h1, &t0, &t1);
            if (h0 && h1) {
                int nearr = n.d.x, farr = n.d.y;
                if (t1 < t0) {
                    nearr = n.d.y;
                    farr = n.d.x;
                }
                if (sp >= kStack) {
                    raise_error(err, DEV_STACK_OVERFLOW);
                    return best->inst != kNoHit;
                }
                stack[sp++] = farr;
                ref = nearr;
                continue;
            }
            if (h0) {
                ref = n.d.x;
                continue;
            }
            if (h1) {
                ref = n.d.y;
                continue;
            }
        } else if (!in_blas) {
            // top-level leaf: one instance
            if ((uint32_t)((~ref) >> 3) >= sc.instance_count) {
                raise_error(err, DEV_BAD_INDEX);
                return best->inst != kNoHit;
            }
            const GpuInstance* gi = sc.instances + ((~ref) >> 3);
            int4 meta = __ldg(reinterpret_cast<const int4*>(gi) + 3);  // blas_root, custom, mask, id
            if (((uint32_t)meta.z & mask) != 0 && meta.x >= 0) {
                if (COUNT) fc->insts[ANY]++;
                if (sp >= kStack) {
                    raise_error(err, DEV_STACK_OVERFLOW);
                    return best->inst != kNoHit;
                }
                stack[sp++] = kExit;
                float4 w[3] = {__ldg(&gi->w2o[0]), __ldg(&gi->w2o[1]), __ldg(&gi->w2o[2])};
                float3 oo, od;
                xform_exact(w, wo, wd, &oo, &od);
                ray_setup(r, oo, od);
                inst_id = (uint32_t)meta.w;
                in_blas = true;
                ref = meta.x;
                continue;
            }
        } else {
            int first = (~ref) >> 3, count = ((~ref) & 7) + 1;
            if ((uint32_t)first + (uint32_t)count > sc.tri_count) {
                raise_error(err, DEV_BAD_INDEX);
                return best->inst != kNoHit;
            }
            if (COUNT) fc->tris[ANY] += count;
            for (int k = 0; k < count; ++k) {
                const float4* tp = reinterpret_cast<const float4*>(sc.tris + first + k);
                float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float t, b1, b2;
                bool back;
                if (tri_hit_exact(r, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), f3(c.x, c.y, c.z), tmin, tcur, &t, &b1, &b2,
                                  &back)) {
                    uint32_t prim = (uint32_t)__float_as_int(a.w);
                    bool better = ANY || best->inst == kNoHit || t < best->t ||
                                  (t == best->t && (inst_id < best->inst || (inst_id == best->inst && prim < best->prim)));
                    if (better) {
                        best->t = t;
                        best->inst = inst_id;
                        best->prim = prim;
                        best->b1 = b1;
                        best->b2 = b2;
                        best->back = back;
                        tcur = t;
                        if (ANY) return true;
                    }
                }
            }
        }
        // pop
        for (;;) {
            if (sp == 0) return best->inst != kNoHit;
            ref = stack[--sp];
            if (ref != kExit) break;
            in_blas = false;
            ray_setup(r, wo, wd);
        }
    }
}


// Warp-cooperative traversal for persistent kernels (Aila & Laine 2009,
// "while-while" with postponed leaves): every lane of the warp calls
// advance() together.  In phase 1 lanes walk inner nodes; a lane that meets a
// leaf keeps it and goes on walking until every lane holds a leaf (or has
// run out of nodes), so inner-node iterations stay busy.  Phase 2 processes
// the held leaves: an instance leaf moves the ray into the mesh tree, a
// triangle leaf runs the watertight tests.  The stack lives in shared memory
// (one column per thread).  Hit set, tie rule and results equal `traverse`.
// Threads of the blocks that run the walkers: a thread's stack entry i is
// at column i * kWalkerThreads of the block's shared array.
constexpr int kWalkerThreads = 128;
struct SmemStack {
    int* base;
    __device__ __forceinline__ int get(int i) const { return base[i * kWalkerThreads]; }
    __device__ __forceinline__ void set(int i, int v) { base[i * kWalkerThreads] = v; }
};

// The first `split` entries in shared memory, deeper ones in a per-thread
// local-memory array (L1-cached).  A smaller shared-memory part lets more
// warps reside per SM; traversals deeper than `split` pay local accesses.
// The local part is an array of the caller's (kSpillMax entries), kept out of
// the walker so that the walker's own fields stay in registers.
constexpr int kSpillMax = 96;
struct SplitStack {
    int* base;
    int split;
    int* spill;
    __device__ __forceinline__ int get(int i) const { return i < split ? base[i * kWalkerThreads] : spill[i - split]; }
    __device__ __forceinline__ void set(int i, int v) {
        if (i < split) base[i * kWalkerThreads] = v;
        else spill[i - split] = v;
    }
};

// World-space origin and direction of a walk: the top level needs only the
// slab reciprocals besides them (its leaves are instances, never triangles),
// recomputed when the walk leaves a mesh tree, which keeps nine values out of
// the registers of the persistent kernels.
struct WorldRay {
    float3 o, d;
};

template <bool ANY, class Stack = SmemStack>
struct WarpWalker {
    static constexpr bool kWide = false;
    // resident 128-thread blocks per SM the kernels are built for: with the
    // straggler exit of the search loop, 8 is 1.7 % faster than 10 (48
    // registers, spilling); the walker takes 56 registers, and 8 blocks of
    // its shared-memory stack fill an SM's shared memory
    static constexpr int kMinBlocks = 8;
    WorldRay wr;  // world ray
    Ray r;        // current ray (world or object space)
    Stack stk;
    int sp, cap, ref;
    bool in_blas;
    uint32_t inst_id, steps, mask;
    uint32_t wait_max;  // lanes still searching that no longer hold the warp in the search loop
    float tmin, tcur;
    HitRec best;

    __device__ __forceinline__ void clear() { ref = kNone; }  // no ray

    __device__ __forceinline__ bool start(const DeviceScene& sc, float3 o, float3 d, float tmin_, float tmax_,
                                          uint32_t mask_) {
        return start_at(sc, sc.tlas_root, o, d, tmin_, tmax_, mask_);
    }
    // Start at an explicit top-level root (several scenes in one node arena).
    __device__ __forceinline__ bool start_at(const DeviceScene& sc, int32_t root, float3 o, float3 d, float tmin_,
                                             float tmax_, uint32_t mask_) {
        wr.o = o;
        wr.d = d;
        ray_setup(r, o, d);
        tmin = tmin_;
        tcur = tmax_;
        mask = mask_;
        best.inst = kNoHit;
        best.prim = 0;
        best.t = tmax_;
        best.b1 = best.b2 = 0.0f;
        best.back = false;
        sp = 0;
        in_blas = false;
        inst_id = 0;
        steps = 0;
        ref = root >= 0 ? root : kNone;
        return ref != kNone;
    }

    __device__ __forceinline__ bool push(int v, uint32_t* err) {
        if (sp >= cap) {
            raise_error(err, DEV_STACK_OVERFLOW);
            return false;
        }
        stk.set(sp++, v);
        return true;
    }
    // pop within the current tree level (stops at an EXIT marker)
    __device__ __forceinline__ void pop_level() {
        if (sp == 0 || stk.get(sp - 1) == kExit) {
            ref = kNone;
            return;
        }
        ref = stk.get(--sp);
    }
    // pop across EXIT markers (restoring the world ray); false when empty
    __device__ __forceinline__ bool pop() {
        for (;;) {
            if (sp == 0) return false;
            ref = stk.get(--sp);
            if (ref != kExit) return true;
            in_blas = false;
            r.o = wr.o;  // back at the top level
            r.d = wr.d;
            r.inv = ray_inv(wr.d);
        }
    }

    // All lanes call this; returns true when an active lane's ray is finished.
    __device__ __forceinline__ bool advance(const DeviceScene& sc, uint32_t* err, bool active) {
        int leaf = kNone;
        bool failed = false;
        // every call counts as a step too: a ray that stopped making progress
        // (a malformed tree or a scheduling bug) ends with an error, not a hang
        if (active && ++steps > sc.max_steps) {
            raise_error(err, DEV_BAD_INDEX);
            failed = true;
        }
        bool searching = active && ref != kNone && !failed;
        const float blo = tmin * kBoxLo, bhi = tcur * kBoxHi;  // tcur is fixed until the leaf phase
        // step while more than `wait_max` lanes are still searching for their
        // first leaf (one vote per step; lanes already holding a leaf walk on
        // speculatively), but at least once when any is, so every searching
        // lane makes progress in every call; the stragglers carry on in the
        // next call instead of holding the whole warp in this loop
        for (uint32_t it = 0;; ++it) {
            const unsigned waiting = __ballot_sync(0xffffffffu, searching && leaf == kNone);
            if (waiting == 0u || (it > 0u && (uint32_t)__popc(waiting) <= wait_max)) break;
            if (searching) {
                if (ref >= 0) {
                    if (++steps > sc.max_steps || (uint32_t)ref >= sc.node_count) {
                        raise_error(err, DEV_BAD_INDEX);
                        failed = true;
                        searching = false;
                    } else {
                        BvhNode n = load_node(sc.nodes, ref);
                        bool h0, h1;
                        float t0, t1;
                        node_hit(r, n, blo, bhi, &h0, &h1, &t0, &t1);
                        if (h0 && h1) {
                            int nearr = n.d.x, farr = n.d.y;
                            if (t1 < t0) {
                                nearr = n.d.y;
                                farr = n.d.x;
                            }
                            if (!push(farr, err)) {
                                failed = true;
                                searching = false;
                            }
                            ref = nearr;
                        } else if (h0) {
                            ref = n.d.x;
                        } else if (h1) {
                            ref = n.d.y;
                        } else {
                            pop_level();
                        }
                    }
                } else if (leaf == kNone) {
                    leaf = ref;  // postpone it and keep walking
                    pop_level();
                } else {
                    searching = false;  // holding a leaf and at a second one
                }
                if (ref == kNone) searching = false;
            }
        }
        if (!active) return false;
        if (failed) return true;
        if (leaf != kNone) {
            if (!in_blas) {
                uint32_t slot = (uint32_t)((~leaf) >> 3);
                if (slot >= sc.instance_count) {
                    raise_error(err, DEV_BAD_INDEX);
                    return true;
                }
                const GpuInstance* gi = sc.instances + slot;
                int4 meta = __ldg(reinterpret_cast<const int4*>(gi) + 3);  // blas_root, custom, mask, id
                if (((uint32_t)meta.z & mask) != 0 && meta.x >= 0) {
                    if (ref != kNone && !push(ref, err)) return true;
                    if (!push(kExit, err)) return true;
                    float4 w[3] = {__ldg(&gi->w2o[0]), __ldg(&gi->w2o[1]), __ldg(&gi->w2o[2])};
                    float3 oo, od;
                    xform_exact(w, wr.o, wr.d, &oo, &od);
                    ray_setup(r, oo, od);
                    inst_id = (uint32_t)meta.w;
                    in_blas = true;
                    ref = meta.x;
                    return false;
                }
            } else {
                int first = (~leaf) >> 3, count = ((~leaf) & 7) + 1;
                if ((uint32_t)first + (uint32_t)count > sc.tri_count) {
                    raise_error(err, DEV_BAD_INDEX);
                    return true;
                }
                for (int k = 0; k < count; ++k) {
                    const float4* tp = reinterpret_cast<const float4*>(sc.tris + first + k);
                    float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                    float t, b1, b2;
                    bool back;
                    if (tri_hit_exact(r, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), f3(c.x, c.y, c.z), tmin, tcur, &t, &b1,
                                      &b2, &back)) {
                        uint32_t prim = (uint32_t)__float_as_int(a.w);
                        bool better = ANY || best.inst == kNoHit || t < best.t ||
                                      (t == best.t && (inst_id < best.inst || (inst_id == best.inst && prim < best.prim)));
                        if (better) {
                            best.t = t;
                            best.inst = inst_id;
                            best.prim = prim;
                            best.b1 = b1;
                            best.b2 = b2;
                            best.back = back;
                            tcur = t;
                            if (ANY) return true;
                        }
                    }
                }
            }
        }
        if (ref == kNone && !pop()) return true;
        return false;
    }
};

// ---------------------------------------------------------------------------
// Eight-wide traversal over quantised WideNode trees: the walker of
// WarpWalker (while-while, postponed leaves, shared-memory stack, straggler
// exit) with node groups in place of single references (Ylitie, Karras &
// Laine 2017): the current group is a node and the mask of its children
// still to visit, in the ray's octant order; visiting a child takes the
// highest bit; an inner child's own children are box-tested at once (all
// eight slots, one mask) and the rest of the current group is pushed as one
// stack entry (node index << 8 | mask).  The slab test of slot k along an
// axis is fma(q_k, 2^e * inv, (o_node - o_ray) * inv) with q_k the near or
// far bound byte, the same kind of rounding as the binary step's
// (lo - o) * inv; with the quantised boxes enclosing the binary tree's
// enlarged boxes and the same interval margins, pruning stays conservative.
// Hit set, tie rule and results equal the binary traversal's.
// ---------------------------------------------------------------------------
// Float of an 8-bit integer (exact): its bits under the exponent of 2^23.
__device__ __forceinline__ float byte_float(uint32_t b) { return __uint_as_float(0x4B000000u | b) - 8388608.0f; }
// The same for byte i of w, the float's bits assembled by one byte permute.
__device__ __forceinline__ float byte_float_at(uint32_t w, int i) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (uint32_t)i)) - 8388608.0f;
}

template <bool ANY, class Stack = SmemStack>
struct WideWalker {
    static constexpr bool kWide = true;
    static constexpr int kMinBlocks = 7;
    WorldRay wr;  // world ray
    Ray r;        // current ray (world or object space)
    Stack stk;
    int sp, cap;
    int node;       // node of the current group (kNone: none)
    uint32_t gmask;  // its children still to visit, bit (slot ^ oct)
    uint32_t oct;    // octant of r.d: bit k set when the direction's component k is negative
    bool in_blas;
    uint32_t inst_id, steps, mask;
    uint32_t wait_max;
    float tmin, tcur;
    HitRec best;

    __device__ __forceinline__ void clear() {  // no ray
        node = kNone;
        gmask = 0;
    }

    __device__ __forceinline__ static uint32_t octant_of(float3 d) {
        return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    }

    // Box tests of a node's eight slots; the mask bit of slot k is k ^ oct.
    __device__ __forceinline__ uint32_t test_children(const DeviceScene& sc, int n) const {
        const float4* p = reinterpret_cast<const float4*>(sc.wnodes + n);
        const float4 org = __ldg(p);
        const uint32_t eb = __float_as_uint(org.w);
        const float lo = tmin * kBoxLo, hi = tcur * kBoxHi;
        float tn[8], tf[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            tn[k] = lo;
            tf[k] = hi;
        }
#define DDGI_AXIS(A, O, INV, ORG)                                                                         \
    {                                                                                                     \
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(p + 1 + A));                                 \
        const float s = __uint_as_float(((eb >> (8 * A)) & 0xFFu) << 23) * INV;                           \
        const float b = (ORG - O) * INV;                                                                  \
        const bool pos = INV >= 0.0f;                                                                     \
        const uint32_t n0 = pos ? q.x : q.z, n1 = pos ? q.y : q.w, f0 = pos ? q.z : q.x, f1 = pos ? q.w : q.y; \
        _Pragma("unroll") for (int k = 0; k < 8; ++k) {                                                   \
            const uint32_t nw = k < 4 ? n0 : n1, fw = k < 4 ? f0 : f1;                                    \
            const float a = fmaf(byte_float_at(nw, k & 3), s, b);                                         \
            const float c = fmaf(byte_float_at(fw, k & 3), s, b);                                         \
            tn[k] = fmaxf(tn[k], a);                                                                      \
            tf[k] = fminf(tf[k], c);                                                                      \
        }                                                                                                 \
    }
        DDGI_AXIS(0, r.o.x, r.inv.x, org.x)
        DDGI_AXIS(1, r.o.y, r.inv.y, org.y)
        DDGI_AXIS(2, r.o.z, r.inv.z, org.z)
#undef DDGI_AXIS
        uint32_t m = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (tn[k] <= tf[k]) m |= 1u << ((uint32_t)k ^ oct);
        return m;
    }

    __device__ __forceinline__ bool start(const DeviceScene& sc, float3 o, float3 d, float tmin_, float tmax_,
                                          uint32_t mask_) {
        return start_at(sc, sc.wtlas_root, o, d, tmin_, tmax_, mask_);
    }
    __device__ __forceinline__ bool start_at(const DeviceScene& sc, int32_t root, float3 o, float3 d, float tmin_,
                                             float tmax_, uint32_t mask_) {
        wr.o = o;
        wr.d = d;
        ray_setup(r, o, d);
        oct = octant_of(d);
        tmin = tmin_;
        tcur = tmax_;
        mask = mask_;
        best.inst = kNoHit;
        best.prim = 0;
        best.t = tmax_;
        best.b1 = best.b2 = 0.0f;
        best.back = false;
        sp = 0;
        in_blas = false;
        inst_id = 0;
        steps = 0;
        node = kNone;
        gmask = 0;
        if (root < 0 || (uint32_t)root >= sc.wnode_count) return false;
        node = root;
        gmask = test_children(sc, root);
        return gmask != 0;
    }
    __device__ __forceinline__ bool push(int v, uint32_t* err) {
        if (sp >= cap) {
            raise_error(err, DEV_STACK_OVERFLOW);
            return false;
        }
        stk.set(sp++, v);
        return true;
    }
    // next group within the current tree level (stops at an EXIT marker)
    __device__ __forceinline__ void pop_level() {
        if (sp == 0 || stk.get(sp - 1) == kExit) {
            node = kNone;
            gmask = 0;
            return;
        }
        const int e = stk.get(--sp);
        node = e >> 8;
        gmask = (uint32_t)e & 0xFFu;
    }
    // next group across EXIT markers (restoring the world ray); false when empty
    __device__ __forceinline__ bool pop() {
        for (;;) {
            if (sp == 0) return false;
            const int e = stk.get(--sp);
            if (e != kExit) {
                node = e >> 8;
                gmask = (uint32_t)e & 0xFFu;
                return true;
            }
            in_blas = false;
            r.o = wr.o;  // back at the top level
            r.d = wr.d;
            r.inv = ray_inv(wr.d);
            oct = octant_of(wr.d);
        }
    }
    __device__ __forceinline__ int child_ref(const DeviceScene& sc, int n, uint32_t slot) const {
        return __ldg(reinterpret_cast<const int*>(sc.wnodes + n) + 16 + slot);
    }

    // All lanes call this; returns true when an active lane's ray is finished.
    __device__ __forceinline__ bool advance(const DeviceScene& sc, uint32_t* err, bool active) {
        int leaf = kNone;
        bool failed = false;
        if (active && ++steps > sc.wmax_steps) {  // as in WarpWalker::advance
            raise_error(err, DEV_BAD_INDEX);
            failed = true;
        }
        bool searching = active && node != kNone && !failed;
        for (uint32_t it = 0;; ++it) {  // as in WarpWalker::advance
            const unsigned waiting = __ballot_sync(0xffffffffu, searching && leaf == kNone);
            if (waiting == 0u || (it > 0u && (uint32_t)__popc(waiting) <= wait_max)) break;
            if (searching) {
                if (gmask != 0u) {
                    const uint32_t key = 31u - (uint32_t)__clz(gmask);
                    const int c = child_ref(sc, node, key ^ oct);
                    if (c >= 0) {
                        if (++steps > sc.wmax_steps || (uint32_t)c >= sc.wnode_count) {
                            raise_error(err, DEV_BAD_INDEX);
                            failed = true;
                            searching = false;
                        } else {
                            gmask &= ~(1u << key);
                            const uint32_t m = test_children(sc, c);
                            if (m != 0u) {
                                if (gmask != 0u && !push((node << 8) | (int)gmask, err)) {
                                    failed = true;
                                    searching = false;
                                }
                                node = c;
                                gmask = m;
                            }
                        }
                    } else if (leaf == kNone) {
                        gmask &= ~(1u << key);
                        leaf = c;  // postpone it and keep walking
                    } else {
                        searching = false;  // holding a leaf and at a second one (it stays in the mask)
                    }
                } else {
                    pop_level();
                }
                if (searching && node == kNone) searching = false;
            }
        }
        if (!active) return false;
        if (failed) return true;
        if (leaf != kNone) {
            if (!in_blas) {
                uint32_t slot = (uint32_t)((~leaf) >> 3);
                if (slot >= sc.instance_count) {
                    raise_error(err, DEV_BAD_INDEX);
                    return true;
                }
                const GpuInstance* gi = sc.winstances + slot;
                int4 meta = __ldg(reinterpret_cast<const int4*>(gi) + 3);  // blas_root (wide), custom, mask, id
                if (((uint32_t)meta.z & mask) != 0 && meta.x >= 0) {
                    if ((uint32_t)meta.x >= sc.wnode_count) {
                        raise_error(err, DEV_BAD_INDEX);
                        return true;
                    }
                    if (node != kNone && gmask != 0u && !push((node << 8) | (int)gmask, err)) return true;
                    if (!push(kExit, err)) return true;
                    float4 w[3] = {__ldg(&gi->w2o[0]), __ldg(&gi->w2o[1]), __ldg(&gi->w2o[2])};
                    float3 oo, od;
                    xform_exact(w, wr.o, wr.d, &oo, &od);
                    ray_setup(r, oo, od);
                    oct = octant_of(od);
                    inst_id = (uint32_t)meta.w;
                    in_blas = true;
                    node = meta.x;
                    gmask = test_children(sc, meta.x);
                    if (gmask != 0u) return false;
                    node = kNone;  // the mesh tree's root misses: back up
                }
            } else {
                int first = (~leaf) >> 3, count = ((~leaf) & 7) + 1;
                if ((uint32_t)first + (uint32_t)count > sc.tri_count) {
                    raise_error(err, DEV_BAD_INDEX);
                    return true;
                }
                for (int k = 0; k < count; ++k) {
                    const float4* tp = reinterpret_cast<const float4*>(sc.tris + first + k);
                    float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                    float t, b1, b2;
                    bool back;
                    if (tri_hit_exact(r, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), f3(c.x, c.y, c.z), tmin, tcur, &t, &b1,
                                      &b2, &back)) {
                        uint32_t prim = (uint32_t)__float_as_int(a.w);
                        bool better = ANY || best.inst == kNoHit || t < best.t ||
                                      (t == best.t && (inst_id < best.inst || (inst_id == best.inst && prim < best.prim)));
                        if (better) {
                            best.t = t;
                            best.inst = inst_id;
                            best.prim = prim;
                            best.b1 = b1;
                            best.b2 = b2;
                            best.back = back;
                            tcur = t;
                            if (ANY) return true;
                        }
                    }
                }
            }
        }
        if ((node == kNone || gmask == 0u) && !pop()) return true;
        return false;
    }
};

}  // namespace ddgi

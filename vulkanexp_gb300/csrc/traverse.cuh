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
struct SmemStack {
    int* base;
    int stride;
    __device__ __forceinline__ int get(int i) const { return base[i * stride]; }
    __device__ __forceinline__ void set(int i, int v) { base[i * stride] = v; }
};

// The first `split` entries in shared memory, deeper ones in a per-thread
// local-memory array (L1-cached).  A smaller shared-memory part lets more
// warps reside per SM; traversals deeper than `split` pay local accesses.
// The local part is an array of the caller's (kSpillMax entries), kept out of
// the walker so that the walker's own fields stay in registers.
constexpr int kSpillMax = 96;
struct SplitStack {
    int* base;
    int stride;
    int split;
    int* spill;
    __device__ __forceinline__ int get(int i) const { return i < split ? base[i * stride] : spill[i - split]; }
    __device__ __forceinline__ void set(int i, int v) {
        if (i < split) base[i * stride] = v;
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
// Four-wide traversal: the walker of WarpWalker (while-while, postponed
// leaves, shared-memory stack) over WideNode trees.  An inner step tests the
// four child boxes of a node (the same slab arithmetic and margins as the
// binary step), continues with the nearest hit child and pushes the others
// farthest first, so they pop nearest first.  Hit set, tie rule and results
// equal the binary traversal's.
// ---------------------------------------------------------------------------
__device__ __forceinline__ WideNode load_wide(const WideNode* nodes, int i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    WideNode n;
    n.lox = __ldg(p + 0);
    n.hix = __ldg(p + 1);
    n.loy = __ldg(p + 2);
    n.hiy = __ldg(p + 3);
    n.loz = __ldg(p + 4);
    n.hiz = __ldg(p + 5);
    float4 r = __ldg(p + 6);
    n.ref = make_int4(__float_as_int(r.x), __float_as_int(r.y), __float_as_int(r.z), __float_as_int(r.w));
    return n;
}

__device__ __forceinline__ float slab_near(float lx, float hx, float ly, float hy, float lz, float hz, const Ray& r,
                                           float tmin, float tmax, float* tfar) {
    float a0 = (lx - r.o.x) * r.inv.x, a1 = (hx - r.o.x) * r.inv.x;
    float a2 = (ly - r.o.y) * r.inv.y, a3 = (hy - r.o.y) * r.inv.y;
    float a4 = (lz - r.o.z) * r.inv.z, a5 = (hz - r.o.z) * r.inv.z;
    *tfar = fminf(fminf(fmaxf(a0, a1), fmaxf(a2, a3)), fminf(fmaxf(a4, a5), tmax));
    return fmaxf(fmaxf(fminf(a0, a1), fminf(a2, a3)), fmaxf(fminf(a4, a5), tmin));
}

template <bool ANY, class Stack = SmemStack>
struct WideWalker {
    static constexpr bool kWide = true;
    static constexpr int kMinBlocks = 7;
    Ray wr, r;
    Stack stk;
    int sp, cap, ref;
    bool in_blas;
    uint32_t inst_id, steps, mask;
    uint32_t wait_max;
    float tmin, tcur;
    HitRec best;

    __device__ __forceinline__ bool start(const DeviceScene& sc, float3 o, float3 d, float tmin_, float tmax_,
                                          uint32_t mask_) {
        return start_at(sc, sc.wtlas_root, o, d, tmin_, tmax_, mask_);
    }
    __device__ __forceinline__ bool start_at(const DeviceScene& sc, int32_t root, float3 o, float3 d, float tmin_,
                                             float tmax_, uint32_t mask_) {
        ray_setup(wr, o, d);
        r = wr;
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
    __device__ __forceinline__ void pop_level() {
        if (sp == 0 || stk.get(sp - 1) == kExit) {
            ref = kNone;
            return;
        }
        ref = stk.get(--sp);
    }
    __device__ __forceinline__ bool pop() {
        for (;;) {
            if (sp == 0) return false;
            ref = stk.get(--sp);
            if (ref != kExit) return true;
            in_blas = false;
            r = wr;
        }
    }

    // Inner step at node `ref`: false if the stack overflowed.  The slabs
    // are taken axis by axis over the four children (the same operations
    // per box as slab_near), so only one axis' bounds are live at a time.
    __device__ __forceinline__ bool inner_step(const DeviceScene& sc, uint32_t* err) {
        const float4* p = reinterpret_cast<const float4*>(sc.wnodes + ref);
        const float lo = tmin * kBoxLo, hi = tcur * kBoxHi;
        float t0 = lo, t1 = lo, t2 = lo, t3 = lo, f0 = hi, f1 = hi, f2 = hi, f3 = hi;
#define DDGI_AXIS(LO4, HI4, O, INV)                                                          \
    {                                                                                        \
        const float4 l = LO4, h = HI4;                                                       \
        float a, b;                                                                          \
        a = (l.x - O) * INV, b = (h.x - O) * INV;                                            \
        t0 = fmaxf(t0, fminf(a, b)), f0 = fminf(f0, fmaxf(a, b));                            \
        a = (l.y - O) * INV, b = (h.y - O) * INV;                                            \
        t1 = fmaxf(t1, fminf(a, b)), f1 = fminf(f1, fmaxf(a, b));                            \
        a = (l.z - O) * INV, b = (h.z - O) * INV;                                            \
        t2 = fmaxf(t2, fminf(a, b)), f2 = fminf(f2, fmaxf(a, b));                            \
        a = (l.w - O) * INV, b = (h.w - O) * INV;                                            \
        t3 = fmaxf(t3, fminf(a, b)), f3 = fminf(f3, fmaxf(a, b));                            \
    }
        DDGI_AXIS(__ldg(p + 0), __ldg(p + 1), r.o.x, r.inv.x)
        DDGI_AXIS(__ldg(p + 2), __ldg(p + 3), r.o.y, r.inv.y)
        DDGI_AXIS(__ldg(p + 4), __ldg(p + 5), r.o.z, r.inv.z)
#undef DDGI_AXIS
        const float4 rr = __ldg(p + 6);
        // misses sort last with key +inf
        int c0 = __float_as_int(rr.x), c1 = __float_as_int(rr.y), c2 = __float_as_int(rr.z), c3 = __float_as_int(rr.w);
        if (!(t0 <= f0) || c0 == kNone) t0 = INFINITY, c0 = kNone;
        if (!(t1 <= f1) || c1 == kNone) t1 = INFINITY, c1 = kNone;
        if (!(t2 <= f2) || c2 == kNone) t2 = INFINITY, c2 = kNone;
        if (!(t3 <= f3) || c3 == kNone) t3 = INFINITY, c3 = kNone;
#define DDGI_CSWAP(ta, ca, tb, cb)             \
    if (tb < ta) {                             \
        float tt = ta;                         \
        ta = tb;                               \
        tb = tt;                               \
        int cc = ca;                           \
        ca = cb;                               \
        cb = cc;                               \
    }
        DDGI_CSWAP(t0, c0, t1, c1)
        DDGI_CSWAP(t2, c2, t3, c3)
        DDGI_CSWAP(t0, c0, t2, c2)
        DDGI_CSWAP(t1, c1, t3, c3)
        DDGI_CSWAP(t1, c1, t2, c2)
#undef DDGI_CSWAP
        if (c3 != kNone && !push(c3, err)) return false;
        if (c2 != kNone && !push(c2, err)) return false;
        if (c1 != kNone && !push(c1, err)) return false;
        if (c0 != kNone) ref = c0;
        else pop_level();
        return true;
    }

    // All lanes call this; returns true when an active lane's ray is finished.
    __device__ __forceinline__ bool advance(const DeviceScene& sc, uint32_t* err, bool active) {
        int leaf = kNone;
        bool failed = false;
        if (active && ++steps > sc.wmax_steps) {  // as in WarpWalker::advance
            raise_error(err, DEV_BAD_INDEX);
            failed = true;
        }
        bool searching = active && ref != kNone && !failed;
        for (uint32_t it = 0;; ++it) {  // as in WarpWalker::advance
            const unsigned waiting = __ballot_sync(0xffffffffu, searching && leaf == kNone);
            if (waiting == 0u || (it > 0u && (uint32_t)__popc(waiting) <= wait_max)) break;
            if (searching) {
                if (ref >= 0) {
                    if (++steps > sc.wmax_steps || (uint32_t)ref >= sc.wnode_count) {
                        raise_error(err, DEV_BAD_INDEX);
                        failed = true;
                        searching = false;
                    } else if (!inner_step(sc, err)) {
                        failed = true;
                        searching = false;
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
                const GpuInstance* gi = sc.winstances + slot;
                int4 meta = __ldg(reinterpret_cast<const int4*>(gi) + 3);  // blas_root (wide), custom, mask, id
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

}  // namespace ddgi

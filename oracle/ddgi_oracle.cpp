/*
 * ddgi_oracle.cpp — CPU checker for the DDGI probe update.  TEST
 * INFRASTRUCTURE ONLY: it is loaded by the tests, by the package's smoke
 * check and by the CPU-baseline leg of the benchmark, never by the product.
 *
 * A scalar restatement of VulkanExp's probe-update shaders, templated on the
 * arithmetic type (float for the parity form, double for the error
 * reference), multithreaded over probes on a worker pool with the interface
 * of the reference's ThreadPool/TaskQueue (src/ThreadPool.hpp:10-75) and an
 * explicit worker count.
 *
 * Followed line by line:
 *   src/shaders/traceProbes.rgen:29-49        ray generation, tmin/tmax
 *   src/shaders/closesthit.glsl:133-289       NO_REFLECTION hit shading
 *   src/shaders/miss.rmiss:17-23              miss (constant sky radiance)
 *   src/shaders/shadow.rmiss:6-9              shadow query
 *   src/shaders/pbrMetallicRoughness.glsl:8-84
 *   src/shaders/irradiance.glsl:7-237         grid/octahedral math, sampleProbes
 *   src/shaders/common.glsl:4-8
 *   src/shaders/probesUpdate.glsl:29-121      colour/depth blend + state update
 *   src/shaders/probesCopyBorders.comp:21-245 border copy (generalised)
 *   src/shaders/probesInit.rgen:31-64         probe classification
 *   src/shaders/FinalGather.frag:39-80        final gather (the atlas consumer)
 *
 * Traversal is opaque in the reference (driver-built Vulkan acceleration
 * structures on RT cores).  Its closest-hit SEMANTICS are restated: the hit
 * with minimum t in [tmin, tmax], ties broken by the lowest (instance,
 * primitive), using the watertight ray/triangle test of Woop, Benthin and
 * Wald (JCGT 2(1), 2013) with every operation rounded separately
 * (compile with -ffp-contract=off).  The BVH here is an independent
 * median-split tree; only its pruning differs from the GPU's LBVH, and
 * pruning is conservative (boxes are enlarged), so hit sets are identical.
 *
 * Deliberate deviations from the reference, all in favour of the intended
 * behaviour (the CUDA path makes the same choices):
 *  - probesUpdate.glsl:63-68 fills the shared ray-direction array from only
 *    the 36 invocations of the colour workgroup, and traceProbes.rgen:46 only
 *    writes directions when probeCount >= raysPerProbe; here every ray uses
 *    the full direction table.
 *  - probesUpdate.glsl:106-110 reads the workgroup max-change after a memory
 *    barrier without an execution barrier (a race); here it is the max over
 *    all interior texels.
 *  - Texture filtering is exact bilinear (the hardware uses 8-bit weights).
 *  - pow(x, 3) and pow(x, 5) are evaluated as products.
 *
 * Pinned to the reference's own shader code: the files above, compiled as
 * C++ by oracle/build_ref_glsl.py and run on the host (every invocation a
 * thread, traceRayEXT through this file's traversal), give the same
 * reference-format atlases and probe states as this restatement's float
 * form, bit for bit, on the update passes and on a whole room update
 * (tests/test_reference_shaders.py, fixtures in tests/golden/).
 *
 * Atlas storage: the plain form keeps FP32 texels.  The reference-format form
 * (grid precision DDGI_PRECISION_REFERENCE_FORMAT) rounds every stored texel
 * to the formats of the reference's atlas images (B10G11R11 unsigned floats
 * for irradiance, RG16F for depth: src/IrradianceProbes.cpp:41, 63) with
 * ddgi_round_r11/b10/half of include/ddgi_exact.h, so its bounce lookup reads
 * the same rounded values the reference's does.
 */
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <functional>
#include <future>
#include <mutex>
#include <thread>
#include <vector>

#include "../include/ddgi.h"
#include "../include/ddgi_exact.h"

namespace {

// ---------------------------------------------------------------------------
// Small GLSL-like vector type
// ---------------------------------------------------------------------------
template <class T>
struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit V3(T s) : x(s), y(s), z(s) {}
    template <class U>
    explicit V3(const V3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> V3<T> normalize(V3<T> a) {
    T inv = T(1) / length(a);
    return a * inv;
}
template <class T> V3<T> vabs(V3<T> a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
template <class T> T clampT(T v, T lo, T hi) { return std::min(std::max(v, lo), hi); }
template <class T> V3<T> mix3(V3<T> a, V3<T> b, T t) { return a * (T(1) - t) + b * t; }
template <class T> T mixT(T a, T b, T t) { return a * (T(1) - t) + b * t; }
template <class T> T glsl_sign(T v) { return v > T(0) ? T(1) : (v < T(0) ? T(-1) : T(0)); }
template <class T> T sign_not_zero(T v) { return v >= T(0) ? T(1) : T(-1); }

using F3 = V3<float>;

// Constant of src/shaders/common.glsl:4
template <class T> constexpr T kPi() { return T(3.1415926538); }

// ---------------------------------------------------------------------------
// Worker pool with the interface of the reference's ThreadPool
// (src/ThreadPool.hpp:10-75, ThreadPool.cpp:5-28): `threadCount` workers fed
// from one task queue, queue() returning the task's future, and a TaskQueue
// that collects the futures of a batch and waits for them.  The reference
// keeps one global pool of hardware_concurrency() - 1 workers
// (ThreadPool.hpp:31, 37-40); the checker's pools take an explicit worker
// count instead (the caller's, normally every host core), one pool per
// count, made on first use in each process.
// ---------------------------------------------------------------------------
thread_local bool t_pool_worker = false;  // the current thread is a pool worker

class ThreadPool {
  public:
    class TaskQueue {
      public:
        explicit TaskQueue(ThreadPool& pool) : pool_(pool) {}
        TaskQueue(const TaskQueue&) = delete;
        TaskQueue& operator=(const TaskQueue&) = delete;
        ~TaskQueue() { wait(); }
        void start(std::function<void()>&& fn) { futures_.push_back(pool_.queue(std::move(fn))); }
        void wait() {
            for (auto& f : futures_) f.wait();
            futures_.clear();
        }

      private:
        ThreadPool& pool_;
        std::vector<std::future<void>> futures_;
    };

    explicit ThreadPool(uint32_t threadCount) { startThreads(threadCount); }
    ThreadPool(const ThreadPool&) = delete;
    ThreadPool& operator=(const ThreadPool&) = delete;
    ~ThreadPool() {
        {
            std::lock_guard<std::mutex> lock(mutex_);
            closing_ = true;
        }
        ready_.notify_all();
        for (auto& t : workers_) t.join();
    }

    void startThreads(uint32_t threadCount) {
        for (uint32_t i = 0; i < threadCount; ++i) workers_.emplace_back([this] { work(); });
    }
    uint32_t threadCount() const { return (uint32_t)workers_.size(); }

    std::future<void> queue(std::function<void()>&& fn) {
        std::packaged_task<void()> task(std::move(fn));
        std::future<void> done = task.get_future();
        {
            std::lock_guard<std::mutex> lock(mutex_);
            pending_.push_back(std::move(task));
        }
        ready_.notify_one();
        return done;
    }

    // The pool of `threadCount` workers of this process.  Pools are kept
    // until the process ends; a process forked after a pool was made has no
    // workers behind the inherited object, so it makes its own.
    static ThreadPool& withThreads(uint32_t threadCount) {
        static std::mutex registry_mutex;
        static std::vector<ThreadPool*> registry;
        std::lock_guard<std::mutex> lock(registry_mutex);
        const pid_t self = getpid();
        for (ThreadPool* p : registry)
            if (p->owner_ == self && p->threadCount() == threadCount) return *p;
        registry.push_back(new ThreadPool(threadCount));  // never freed: workers live as long as the process
        return *registry.back();
    }

  private:
    void work() {
        t_pool_worker = true;
        for (;;) {
            std::packaged_task<void()> task;
            {
                std::unique_lock<std::mutex> lock(mutex_);
                ready_.wait(lock, [this] { return closing_ || !pending_.empty(); });
                if (pending_.empty()) return;  // closing, nothing left to run
                task = std::move(pending_.front());
                pending_.pop_front();
            }
            task();
        }
    }

    const pid_t owner_ = getpid();
    std::vector<std::thread> workers_;
    std::deque<std::packaged_task<void()>> pending_;
    std::mutex mutex_;
    std::condition_variable ready_;
    bool closing_ = false;
};

// fn(begin, end) over [0, n) in chunks of `grain`, on a pool of `nthreads`
// workers (each takes chunks from a shared counter until none is left); the
// calling thread waits.  Serial for one thread, a small n, or a call made from
// inside a pool task (a worker waiting on its own pool could starve it).
void parallel_for(size_t n, int nthreads, const std::function<void(size_t, size_t)>& fn, size_t grain = 1) {
    if (nthreads <= 1 || n <= grain || t_pool_worker) {
        fn(0, n);
        return;
    }
    std::atomic<size_t> next{0};
    ThreadPool::TaskQueue batch(ThreadPool::withThreads((uint32_t)nthreads));
    for (int i = 0; i < nthreads; ++i)
        batch.start([&]() {
            for (;;) {
                const size_t b = next.fetch_add(grain);
                if (b >= n) break;
                fn(b, std::min(n, b + grain));
            }
        });
    batch.wait();
}

// ---------------------------------------------------------------------------
// Scene + CPU BVH
// ---------------------------------------------------------------------------
struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const float p[3]) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    void grow(const Box& b) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    // Conservative enlargement so that float slab tests never prune a box
    // containing a hit that the triangle test would report.
    void enlarge() {
        for (int k = 0; k < 3; ++k) {
            float e = (hi[k] - lo[k]) * 1e-5f + (std::fabs(lo[k]) + std::fabs(hi[k])) * 1e-6f + 1e-7f;
            lo[k] -= e;
            hi[k] += e;
        }
    }
};

struct Node {
    Box box;
    uint32_t first = 0;  // leaf: first index into order[]; inner: left child
    uint32_t count = 0;  // leaf: primitive count; inner: 0 (right child = first + 1 ... stored in `right`)
    uint32_t right = 0;
};

struct Bvh {
    std::vector<Node> nodes;
    std::vector<uint32_t> order;  // leaf primitive ids
};

void build_bvh(Bvh& bvh, const std::vector<Box>& boxes) {
    const uint32_t n = (uint32_t)boxes.size();
    bvh.nodes.clear();
    bvh.order.resize(n);
    for (uint32_t i = 0; i < n; ++i) bvh.order[i] = i;
    if (n == 0) return;
    std::vector<float> cent(3 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) cent[3 * (size_t)i + k] = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);
    bvh.nodes.reserve(2 * (size_t)n);
    struct Item { uint32_t node, b, e; };
    std::vector<Item> stack;
    bvh.nodes.push_back(Node{});
    stack.push_back({0, 0, n});
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        Box bb, cb;
        for (uint32_t i = it.b; i < it.e; ++i) {
            bb.grow(boxes[bvh.order[i]]);
            cb.grow(&cent[3 * (size_t)bvh.order[i]]);
        }
        bb.enlarge();
        Node& nd = bvh.nodes[it.node];
        nd.box = bb;
        uint32_t cnt = it.e - it.b;
        int axis = 0;
        float ext = cb.hi[0] - cb.lo[0];
        for (int k = 1; k < 3; ++k)
            if (cb.hi[k] - cb.lo[k] > ext) { ext = cb.hi[k] - cb.lo[k]; axis = k; }
        if (cnt <= 4 || !(ext > 0.0f)) {
            if (cnt > 4 && !(ext > 0.0f)) {
                // coincident centroids: split by index
            } else {
                nd.first = it.b;
                nd.count = cnt;
                continue;
            }
        }
        uint32_t mid = it.b + cnt / 2;
        std::nth_element(bvh.order.begin() + it.b, bvh.order.begin() + mid, bvh.order.begin() + it.e,
                         [&](uint32_t a, uint32_t b) {
                             float ca = cent[3 * (size_t)a + axis], cbv = cent[3 * (size_t)b + axis];
                             return ca < cbv || (ca == cbv && a < b);
                         });
        uint32_t l = (uint32_t)bvh.nodes.size();
        bvh.nodes.push_back(Node{});
        bvh.nodes.push_back(Node{});
        bvh.nodes[it.node].first = l;
        bvh.nodes[it.node].right = l + 1;
        bvh.nodes[it.node].count = 0;
        stack.push_back({l, it.b, mid});
        stack.push_back({l + 1, mid, it.e});
    }
}

struct MeshData {
    std::vector<F3> v0, v1, v2;  // object-space triangle vertices, in primitive order
    Bvh bvh;
    Box bounds;
};

struct InstanceData {
    float o2w[12], w2o[12];
    uint32_t custom, mask, mesh;
};

struct Scene {
    std::vector<MeshData> meshes;
    std::vector<InstanceData> instances;
    Bvh tlas;
    std::vector<F3> normals;  // per vertex (global vertex array)
    std::vector<uint32_t> indices;
    std::vector<ddgi_offset_entry> offsets;
    std::vector<ddgi_material> materials;
};

// ---------------------------------------------------------------------------
// Exact ray/box and ray/triangle tests
// ---------------------------------------------------------------------------
struct RayPre {
    F3 o, d;
    float inv[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

RayPre make_ray(F3 o, F3 d) {
    RayPre r;
    r.o = o;
    r.d = d;
    for (int k = 0; k < 3; ++k) {
        float dk = d[k];
        r.inv[k] = 1.0f / (dk != 0.0f ? dk : 1e-30f);
    }
    int kz = 0;
    if (std::fabs(d.y) > std::fabs(d[kz])) kz = 1;
    if (std::fabs(d.z) > std::fabs(d[kz])) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
    return r;
}

// Box tests use [tmin * kBoxLo, tcur * kBoxHi]: a relative margin far above
// the few-ulp error of slab and triangle distances, so that pruning never
// removes a box holding a hit the triangle test reports.
constexpr float kBoxLo = 0.99999f;
constexpr float kBoxHi = 1.00001f;

inline bool box_hit(const RayPre& r, const Box& b, float tmin, float tmax, float* tnear) {
    float t0 = tmin, t1 = tmax;
    for (int k = 0; k < 3; ++k) {
        float a = (b.lo[k] - r.o[k]) * r.inv[k];
        float c = (b.hi[k] - r.o[k]) * r.inv[k];
        float n = std::min(a, c), f = std::max(a, c);
        t0 = std::max(t0, n);
        t1 = std::min(t1, f);
    }
    *tnear = t0;
    return t0 <= t1;
}

struct TriHit {
    float t, b1, b2;
    bool backface;
};

// Watertight test; returns true for t in [tmin, tmax].
inline bool tri_hit(const RayPre& r, F3 v0, F3 v1, F3 v2, float tmin, float tmax, TriHit* h) {
    F3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float Ax = A[r.kx] - r.Sx * A[r.kz];
    float Ay = A[r.ky] - r.Sy * A[r.kz];
    float Bx = B[r.kx] - r.Sx * B[r.kz];
    float By = B[r.ky] - r.Sy * B[r.kz];
    float Cx = C[r.kx] - r.Sx * C[r.kz];
    float Cy = C[r.ky] - r.Sy * C[r.kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = (U + V) + W;
    if (det == 0.0f) return false;
    float Az = r.Sz * A[r.kz];
    float Bz = r.Sz * B[r.kz];
    float Cz = r.Sz * C[r.kz];
    float T = (U * Az + V * Bz) + W * Cz;
    float t = T / det;
    if (!(t >= tmin && t <= tmax)) return false;
    h->t = t;
    h->b1 = V / det;
    h->b2 = W / det;
    h->backface = det < 0.0f;
    return true;
}

inline void xform_ray(const float w[12], F3 o, F3 d, F3* oo, F3* od) {
    for (int r = 0; r < 3; ++r) {
        float a = w[4 * r + 0] * o.x;
        float b = w[4 * r + 1] * o.y;
        float c = w[4 * r + 2] * o.z;
        (*oo)[r] = ((a + b) + c) + w[4 * r + 3];
        float e = w[4 * r + 0] * d.x;
        float f = w[4 * r + 1] * d.y;
        float g = w[4 * r + 2] * d.z;
        (*od)[r] = (e + f) + g;
    }
}

struct Hit {
    uint32_t inst = 0xFFFFFFFFu, prim = 0;
    float t = 0, b1 = 0, b2 = 0;
    bool backface = false;
    bool valid() const { return inst != 0xFFFFFFFFu; }
};

inline bool better(float t, uint32_t inst, uint32_t prim, const Hit& best) {
    if (!best.valid()) return true;
    if (t < best.t) return true;
    if (t > best.t) return false;
    if (inst != best.inst) return inst < best.inst;
    return prim < best.prim;
}

// Closest hit (any_hit=false) or first hit found (any_hit=true).
bool trace(const Scene& sc, F3 o, F3 d, float tmin, float tmax, uint32_t mask, bool any_hit, Hit* out) {
    Hit best;
    if (sc.tlas.nodes.empty()) { *out = best; return false; }
    float tcur = tmax;
    RayPre wr = make_ray(o, d);
    uint32_t stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const Node& nd = sc.tlas.nodes[stack[--sp]];
        float tn;
        if (!box_hit(wr, nd.box, tmin * kBoxLo, tcur * kBoxHi, &tn)) continue;
        if (nd.count == 0) {
            stack[sp++] = nd.right;
            stack[sp++] = nd.first;
            continue;
        }
        for (uint32_t k = 0; k < nd.count; ++k) {
            uint32_t ii = sc.tlas.order[nd.first + k];
            const InstanceData& inst = sc.instances[ii];
            if ((inst.mask & mask) == 0) continue;
            const MeshData& m = sc.meshes[inst.mesh];
            if (m.bvh.nodes.empty()) continue;
            F3 oo, od;
            xform_ray(inst.w2o, o, d, &oo, &od);
            RayPre r = make_ray(oo, od);
            uint32_t bst[64];
            int bsp = 0;
            bst[bsp++] = 0;
            while (bsp > 0) {
                const Node& bn = m.bvh.nodes[bst[--bsp]];
                float t2;
                if (!box_hit(r, bn.box, tmin * kBoxLo, tcur * kBoxHi, &t2)) continue;
                if (bn.count == 0) {
                    bst[bsp++] = bn.right;
                    bst[bsp++] = bn.first;
                    continue;
                }
                for (uint32_t q = 0; q < bn.count; ++q) {
                    uint32_t p = m.bvh.order[bn.first + q];
                    TriHit th;
                    if (!tri_hit(r, m.v0[p], m.v1[p], m.v2[p], tmin, tcur, &th)) continue;
                    if (any_hit) {
                        best.inst = ii; best.prim = p; best.t = th.t; best.b1 = th.b1; best.b2 = th.b2;
                        best.backface = th.backface;
                        *out = best;
                        return true;
                    }
                    if (better(th.t, ii, p, best)) {
                        best.inst = ii; best.prim = p; best.t = th.t; best.b1 = th.b1; best.b2 = th.b2;
                        best.backface = th.backface;
                        tcur = th.t;
                    }
                }
            }
        }
    }
    *out = best;
    return best.valid();
}

// ---------------------------------------------------------------------------
// Grid and octahedral math (irradiance.glsl:7-138)
// ---------------------------------------------------------------------------
struct Grid {
    F3 mn, mx;
    int res[3];
    uint32_t rays, colorRes, depthRes;
    float sharp, hyst, bias;
    bool quant;  // reference-format atlas: stores rounded to R11G11B10F / RG16F
    uint32_t count() const { return (uint32_t)res[0] * res[1] * res[2]; }
};

Grid make_grid(const ddgi_grid_desc* g) {
    Grid o;
    o.mn = F3(g->extent_min[0], g->extent_min[1], g->extent_min[2]);
    o.mx = F3(g->extent_max[0], g->extent_max[1], g->extent_max[2]);
    for (int k = 0; k < 3; ++k) o.res[k] = g->resolution[k];
    o.rays = g->rays_per_probe;
    o.colorRes = g->color_res;
    o.depthRes = g->depth_res;
    o.sharp = g->depth_sharpness;
    o.hyst = g->hysteresis;
    o.bias = g->shadow_bias;
    o.quant = g->precision == DDGI_PRECISION_REFERENCE_FORMAT;
    return o;
}

// A stored atlas value of the reference-format form (IrradianceProbes.cpp:41,
// 63): colour channel c rounded to the B10G11R11 unsigned float it becomes
// in the reference's irradiance image, a depth channel to a half.  Double
// values are first rounded to float, as a float32 shader value would be.
template <class T> T round_color_store(T v, int c) {
    float f = (float)v;
    return T(c == 2 ? ddgi_round_b10(f) : ddgi_round_r11(f));
}
template <class T> T round_depth_store(T v) { return T(ddgi_round_half((float)v)); }

inline void grid_index(uint32_t index, const Grid& g, int idx[3]) {  // :7-13
    idx[0] = (int)(index % (uint32_t)g.res[0]);
    idx[1] = (int)((index % (uint32_t)(g.res[0] * g.res[1])) / (uint32_t)g.res[0]);
    idx[2] = (int)(index / (uint32_t)(g.res[0] * g.res[1]));
}
inline uint32_t linear_index(const int idx[3], const Grid& g) {  // :15-17
    return (uint32_t)(idx[0] + g.res[0] * idx[1] + g.res[0] * g.res[1] * idx[2]);
}
template <class T> V3<T> cell_size(const Grid& g) {  // :19-21
    return {(T(g.mx.x) - T(g.mn.x)) / T(g.res[0] - 1), (T(g.mx.y) - T(g.mn.y)) / T(g.res[1] - 1),
            (T(g.mx.z) - T(g.mn.z)) / T(g.res[2] - 1)};
}
template <class T> V3<T> probe_pos(const int idx[3], const Grid& g) {  // :23-26
    V3<T> c = cell_size<T>(g);
    return {T(idx[0]) * c.x + T(g.mn.x), T(idx[1]) * c.y + T(g.mn.y), T(idx[2]) * c.z + T(g.mn.z)};
}

template <class T> void oct_decode(T ox, T oy, V3<T>* out) {  // :107-112
    V3<T> v(ox, oy, T(1) - std::fabs(ox) - std::fabs(oy));
    if (v.z < T(0)) {
        T nx = (T(1) - std::fabs(v.y)) * sign_not_zero(v.x);
        T ny = (T(1) - std::fabs(v.x)) * sign_not_zero(v.y);
        v.x = nx;
        v.y = ny;
    }
    *out = normalize(v);
}

template <class T> void sphere_to_oct_uv(V3<T> d, T* u, T* v) {  // :119-138
    V3<T> oct(glsl_sign(d.x), glsl_sign(d.y), glsl_sign(d.z));
    T sum = dot(d, oct);
    V3<T> o(d.x / sum, d.y / sum, d.z / sum);
    if (o.z < T(0)) {
        V3<T> a = vabs(o);
        T nx = oct.x * (T(1) - a.y);
        T ny = oct.y * (T(1) - a.x);
        o.x = nx;
        o.y = ny;
    }
    *u = o.x * T(0.5) + T(0.5);
    *v = o.y * T(0.5) + T(0.5);
}

// Texel-centre scale of probesUpdate.glsl:33-42 for an interior side n:
// the reference's truncated constants for n = 6 and n = 14, 2/n otherwise.
inline float texel_scale(uint32_t n) {
    if (n == 6) return 0.33333f;
    if (n == 14) return 0.142857f;
    return (float)(2.0 / (double)n);
}

// ---------------------------------------------------------------------------
// Atlas views
// ---------------------------------------------------------------------------
template <class T>
struct Atlas {
    T* color;  // RGBA
    T* depth;  // RG
    uint32_t cw, ch, dw, dh;
};

template <class T>
void bilinear(const T* img, uint32_t w, uint32_t h, int ch, int nc, T u, T v, T* out) {
    // LINEAR filter, REPEAT addressing (src/RaytracingDescriptors.hpp:63, 70)
    T x = u * T(w) - T(0.5);
    T y = v * T(h) - T(0.5);
    T fx0 = std::floor(x), fy0 = std::floor(y);
    T ax = x - fx0, ay = y - fy0;
    long i0 = (long)fx0, j0 = (long)fy0;
    auto wrap = [](long i, long n) { long r = i % n; return r < 0 ? r + n : r; };
    long i1 = wrap(i0 + 1, w), j1 = wrap(j0 + 1, h);
    i0 = wrap(i0, w);
    j0 = wrap(j0, h);
    for (int c = 0; c < nc; ++c) {
        T t00 = img[((size_t)j0 * w + i0) * ch + c];
        T t10 = img[((size_t)j0 * w + i1) * ch + c];
        T t01 = img[((size_t)j1 * w + i0) * ch + c];
        T t11 = img[((size_t)j1 * w + i1) * ch + c];
        T top = t00 * (T(1) - ax) + t10 * ax;
        T bot = t01 * (T(1) - ax) + t11 * ax;
        out[c] = top * (T(1) - ay) + bot * ay;
    }
}

// sampleProbes (irradiance.glsl:145-237)
template <class T>
V3<T> sample_probes(V3<T> position, V3<T> normal, V3<T> toCamera, const Grid& g, const uint32_t* states,
                    const Atlas<T>& at) {
    V3<T> cs = cell_size<T>(g);
    V3<T> gridCoords = (position - V3<T>(g.mn)) / vabs(cs);
    if (!(gridCoords.x >= T(0) && gridCoords.y >= T(0) && gridCoords.z >= T(0))) return V3<T>();
    V3<T> biasVector = (normal + toCamera) * T(g.bias);
    V3<T> biasedPosition = position + biasVector;
    const T lim = T(16777216);
    int first[3] = {(int)std::min(gridCoords.x, lim), (int)std::min(gridCoords.y, lim), (int)std::min(gridCoords.z, lim)};
    V3<T> fp = probe_pos<T>(first, g);
    V3<T> alpha = (position - fp) / vabs(cs);
    alpha = V3<T>(clampT(alpha.x, T(0), T(1)), clampT(alpha.y, T(0), T(1)), clampT(alpha.z, T(0), T(1)));

    V3<T> finalColor;
    T totalWeight = 0;
    V3<T> fallbackColor;
    T totalFallbackWeight = 0;
    T uvsx = T(g.res[0] * g.res[1]), uvsy = T(g.res[2]);
    T cr = T(g.colorRes), dr = T(g.depthRes);

    for (int i = 0; i < 8; ++i) {
        int off[3] = {i & 1, (i >> 1) & 1, (i >> 2) & 1};
        int pc[3] = {first[0] + off[0], first[1] + off[1], first[2] + off[2]};
        if (pc[0] > g.res[0] - 1 || pc[1] > g.res[1] - 1 || pc[2] > g.res[2] - 1) continue;
        if (states[linear_index(pc, g)] == 0) continue;
        V3<T> probePosition = probe_pos<T>(pc, g);
        V3<T> directionToProbe = normalize(probePosition - position);
        V3<T> biasedDirectionToProbe = probePosition - biasedPosition;
        T su, sv;
        sphere_to_oct_uv(normal, &su, &sv);
        T cscale = T(g.colorRes - 2) / T(g.colorRes);
        T dscale = T(g.depthRes - 2) / T(g.depthRes);
        T lcu = cscale * su, lcv = cscale * sv;
        T du, dv;
        sphere_to_oct_uv(-normalize(biasedDirectionToProbe), &du, &dv);
        T ldu = dscale * du, ldv = dscale * dv;
        int tile = pc[1] * g.res[0] + pc[0];
        T cu = (T((int)g.colorRes * tile + 1) / cr + lcu) / uvsx;
        T cv = (T((int)g.colorRes * pc[2] + 1) / cr + lcv) / uvsy;
        T du2 = (T((int)g.depthRes * tile + 1) / dr + ldu) / uvsx;
        T dv2 = (T((int)g.depthRes * pc[2] + 1) / dr + ldv) / uvsy;
        V3<T> tri(off[0] ? alpha.x : T(1) - alpha.x, off[1] ? alpha.y : T(1) - alpha.y,
                  off[2] ? alpha.z : T(1) - alpha.z);
        T weight = 1;
        T bfw = std::max(T(0.0001), (dot(directionToProbe, normal) + T(1)) * T(0.5));
        weight *= bfw * bfw + T(0.2);
        T fallbackWeight = weight;
        T depth[2];
        bilinear(at.depth, at.dw, at.dh, 2, 2, du2, dv2, depth);
        T mean = depth[0];
        T variance = std::fabs(depth[0] * depth[0] - depth[1]);
        T dist = length(probePosition - biasedPosition);
        T dm = std::max(dist - mean, T(0.0001));
        T cheb = variance / (variance + dm * dm);
        cheb = std::max(cheb * cheb * cheb, T(0));
        weight *= (dist <= mean) ? T(1) : cheb;
        weight = std::max(T(0.000001), weight);
        const T crush = T(0.2);
        if (weight < crush) weight *= weight * weight * (T(1) / (crush * crush));
        T triw = tri.x * tri.y * tri.z + T(0.001);
        weight *= triw;
        fallbackWeight *= triw;
        T col[3];
        bilinear(at.color, at.cw, at.ch, 4, 3, cu, cv, col);
        V3<T> color(std::sqrt(col[0]), std::sqrt(col[1]), std::sqrt(col[2]));
        finalColor = finalColor + color * weight;
        totalWeight += weight;
        fallbackColor = fallbackColor + color * fallbackWeight;
        totalFallbackWeight += fallbackWeight;
    }
    if (totalWeight > T(1e-3)) finalColor = finalColor * (T(1) / totalWeight);
    if (totalFallbackWeight > T(1e-3)) fallbackColor = fallbackColor * (T(1) / totalFallbackWeight);
    finalColor = finalColor * finalColor;
    fallbackColor = fallbackColor * fallbackColor;
    T a = T(8) * clampT(totalWeight, T(0), T(1) / T(8));
    return mix3(fallbackColor, finalColor, a);
}

// pbrMetallicRoughness (pbrMetallicRoughness.glsl:43-84)
template <class T>
V3<T> pbr(V3<T> n, V3<T> v, V3<T> lightColor, V3<T> lightDir, V3<T> albedo, T metal, T rough) {
    const T pi = kPi<T>();
    V3<T> f0(T(0.04));
    V3<T> diffuseColor = albedo * (V3<T>(T(1)) - f0);
    diffuseColor = diffuseColor * (T(1) - metal);
    T alphaRoughness = rough * rough;
    V3<T> specularColor = mix3(f0, albedo, metal);
    T reflectance = std::max(std::max(specularColor.x, specularColor.y), specularColor.z);
    T reflectance90 = clampT(reflectance * T(25), T(0), T(1));
    V3<T> R0 = specularColor;
    V3<T> R90 = V3<T>(T(1)) * reflectance90;
    V3<T> l = normalize(lightDir);
    V3<T> h = normalize(l + v);
    T NdotL = clampT(dot(n, l), T(0.001), T(1));
    T NdotV = clampT(std::fabs(dot(n, v)), T(0.001), T(1));
    T NdotH = clampT(dot(n, h), T(0), T(1));
    T VdotH = clampT(dot(v, h), T(0), T(1));
    T x = clampT(T(1) - VdotH, T(0), T(1));
    T x2 = x * x;
    T p5 = x2 * x2 * x;
    V3<T> F = R0 + (R90 - R0) * p5;
    T a2 = alphaRoughness * alphaRoughness;
    T attL = T(2) * NdotL / (NdotL + std::sqrt(a2 + (T(1) - a2) * (NdotL * NdotL)));
    T attV = T(2) * NdotV / (NdotV + std::sqrt(a2 + (T(1) - a2) * (NdotV * NdotV)));
    T G = attL * attV;
    T a = NdotH * alphaRoughness;
    T k = alphaRoughness / ((T(1) - NdotH * NdotH) + a * a);
    T D = clampT(k * k * (T(1) / pi), T(0), T(4));
    V3<T> diffuseContrib = (V3<T>(T(1)) - F) * diffuseColor * (T(1) / pi);
    V3<T> specContrib = F * (G * D / (T(4) * NdotL * NdotV));
    return lightColor * (diffuseContrib + specContrib) * NdotL;
}

struct Light {
    F3 dir, color, sky;
    float brightness = 1.0f;  // LightBuffer.color.a
};

// Miss radiance mode (oracle_set_sky_mode): 0 the constant sky radiance,
// 1 the atmospheric sky of src/shaders/sky.glsl:60-127 (miss.rmiss:22).
std::atomic<int> g_sky_mode{0};

// sky() of src/shaders/sky.glsl:60-127 with showSun = true, in T; the
// operation order follows the shader expression by expression.
template <class T>
V3<T> atmosphere(V3<T> rayOrigin, V3<T> rayDirection, V3<T> sunPosition, V3<T> sunColor, T brightness) {
    const T inner = T(100000.0f), outer = T(2500.0f) + inner, avg = T(0.25f);
    const T scale = T(1) / (outer - inner);
    const V3<T> invWl(T(1) / T(std::pow(0.650f, 4.0f)), T(1) / T(std::pow(0.570f, 4.0f)),
                      T(1) / T(std::pow(0.475f, 4.0f)));
    const T pi = kPi<T>(), Kr = T(0.0025f), Km = T(0.0010f), g = T(-0.990f);
    const T Kr4PI = Kr * T(4) * pi, Km4PI = Km * T(4) * pi;
    auto scale_fn = [&](T c) {
        T x = T(1) - c;
        return avg * std::exp(T(-0.00287f) + x * (T(0.459f) + x * (T(3.83f) + x * (T(-6.80f) + x * T(5.25f)))));
    };
    auto outside = [&](T radius, V3<T> o, V3<T> d) {
        T a = dot(d, d), b = dot(d, o), c = dot(o, o) - radius * radius;
        T gg = b * b - a * c;
        if (gg > T(0)) {
            T dis = (-std::sqrt(gg) - b) / a;
            if (dis > T(0)) return dis;
        }
        return T(-1);
    };
    auto inside = [&](T radius, V3<T> o, V3<T> d) {
        V3<T> oc = -o;
        T docdir = dot(oc, d);
        V3<T> pc = o + d * docdir;
        T lc = length(pc);
        T dist = std::sqrt(radius * radius - lc * lc);
        T lo = length(pc - o);
        return docdir > T(0) ? dist - lo : dist + lo;
    };
    sunColor = sunColor * brightness;
    V3<T> position = rayOrigin - V3<T>(T(0), -inner - T(100), T(0));
    T height = length(position);
    V3<T> lightDir = normalize(sunPosition);
    if (std::fabs(height - inner) < T(1e-3f)) {
        position = position + normalize(position) * T(1e-2f);
        height = length(position);
    }
    const V3<T> zero(T(0), T(0), T(0));
    if (height < outer) {
        if (height > inner) {
            T pd = outside(inner, position, rayDirection);
            if (pd >= T(0)) {
                T l = std::max(T(0.1f), dot(lightDir, normalize(position + rayDirection * pd)));
                return V3<T>(l * T(0.05f), l * T(0.05f), l * T(0.05f));
            }
        } else {
            return zero;
        }
        T rayDepth = inside(outer, position, rayDirection);
        if (std::isinf(rayDepth) || std::isnan(rayDepth)) return zero;
        const T k = scale / avg;
        T depth = std::exp(k * (inner - height));
        T startAngle = dot(rayDirection, position) / height;
        T startOffset = depth * scale_fn(startAngle);
        T sampleLength = rayDepth / T(64);
        T scaledLength = sampleLength * scale;
        V3<T> sampleRay = rayDirection * sampleLength;
        V3<T> samplePoint = position + sampleRay * T(0.5f);
        V3<T> color = zero;
        for (int i = 0; i < 64; ++i) {
            T h = length(samplePoint);
            T dep = std::exp(k * (inner - h));
            T lightAngle = dot(lightDir, samplePoint) / h;
            T cameraAngle = dot(rayDirection, samplePoint) / h;
            T scatter = startOffset + dep * (scale_fn(lightAngle) - scale_fn(cameraAngle));
            V3<T> att(std::exp(-scatter * (invWl.x * Kr4PI + Km4PI)), std::exp(-scatter * (invWl.y * Kr4PI + Km4PI)),
                      std::exp(-scatter * (invWl.z * Kr4PI + Km4PI)));
            if (std::isinf(att.x) || std::isinf(att.y) || std::isinf(att.z) || std::isnan(att.x) ||
                std::isnan(att.y) || std::isnan(att.z))
                continue;
            color = color + att * (dep * scaledLength);
            samplePoint = samplePoint + sampleRay;
        }
        V3<T> secondary(color.x * Km * sunColor.x, color.y * Km * sunColor.y, color.z * Km * sunColor.z);
        color = V3<T>(color.x * (invWl.x * Kr * sunColor.x), color.y * (invWl.y * Kr * sunColor.y),
                      color.z * (invWl.z * Kr * sunColor.z));
        T miecos = dot(lightDir, -rayDirection);
        T g2 = g * g;
        T phase = T(1.5f) * ((T(1) - g2) / (T(2) + g2)) * (T(1) + miecos * miecos) /
                  std::pow(std::max(T(1e-3f), T(1) + g2 - T(2) * g * miecos), T(1.5f));
        color = color + secondary * phase;
        if (!(std::isinf(color.x) || std::isinf(color.y) || std::isinf(color.z))) return color;
    } else {
        T d = outside(outer, position, rayDirection);
        if (d > T(0)) {
            T l = dot(lightDir, normalize(position + rayDirection * d)) * T(0.5f);
            return V3<T>(l * T(0.5294117647f), l * T(0.80784313725f), l * T(0.92156862745f));
        }
    }
    return zero;
}

// The differentiable parameters of an update: per-material albedo (NULL =
// the materials' base colour), sun radiance and sky radiance, in T.
template <class T>
struct ShadeParams {
    const T* albedo;  // material_count x 3
    V3<T> sun, sky;
};

template <class T>
ShadeParams<T> default_params(const Light& L) {
    return ShadeParams<T>{nullptr, V3<T>(L.color), V3<T>(L.sky)};
}

// Shading of one probe ray given its closest hit (closesthit.glsl
// NO_REFLECTION + miss).  shadow: -1 traces the shadow query, 0/1 uses a
// recorded result; *shadowed_out receives it.
template <class T>
void shade_hit(const Scene& sc, const Grid& g, const Light& L, const ShadeParams<T>& P, const uint32_t* states,
               const Atlas<T>& prev, F3 origin, F3 dir, const Hit& h, int shadow, bool* shadowed_out, T out[4]);

// Hit shading of one probe ray (traceProbes.rgen + closesthit.glsl NO_REFLECTION + miss + shadow).
template <class T>
void shade_ray(const Scene& sc, const Grid& g, const Light& L, const uint32_t* states, const Atlas<T>& prev,
               F3 origin, F3 dir, float tmax, T out[4], Hit* hit_out, bool* shadowed_out = nullptr) {
    Hit h;
    trace(sc, origin, dir, 0.01f, tmax, 0x3u, false, &h);
    if (hit_out) *hit_out = h;
    shade_hit<T>(sc, g, L, default_params<T>(L), states, prev, origin, dir, h, -1, shadowed_out, out);
}

template <class T>
void shade_hit(const Scene& sc, const Grid& g, const Light& L, const ShadeParams<T>& P, const uint32_t* states,
               const Atlas<T>& prev, F3 origin, F3 dir, const Hit& h, int shadow, bool* shadowed_out, T out[4]) {
    if (shadowed_out) *shadowed_out = false;
    if (!h.valid()) {  // miss.rmiss:17-23: constant sky, or sky() (sky.glsl:60-127)
        V3<T> sky = P.sky;
        if (g_sky_mode.load())
            sky = atmosphere<T>(V3<T>(T(origin.x), T(origin.y), T(origin.z)), V3<T>(T(dir.x), T(dir.y), T(dir.z)),
                                V3<T>(T(L.dir.x), T(L.dir.y), T(L.dir.z)),
                                V3<T>(T(L.color.x), T(L.color.y), T(L.color.z)), T(L.brightness));
        out[0] = sky.x;
        out[1] = sky.y;
        out[2] = sky.z;
        out[3] = T(-1);
        return;
    }
    if (h.backface) {  // closesthit.glsl:137-141
        out[0] = out[1] = out[2] = 0;
        out[3] = T(h.t) * T(0.80);
        return;
    }
    const InstanceData& inst = sc.instances[h.inst];
    // Hit position in float, product then sum rounded separately (the CUDA
    // path computes it the same way); it is also the shadow-ray origin, so
    // both forms share it.
    F3 posf(dir.x * h.t + origin.x, dir.y * h.t + origin.y, dir.z * h.t + origin.z);
    const ddgi_offset_entry& oe = sc.offsets[inst.custom];
    uint32_t io = oe.index_offset + 3 * h.prim;
    uint32_t i0 = sc.indices[io], i1 = sc.indices[io + 1], i2 = sc.indices[io + 2];
    V3<T> n0(sc.normals[oe.vertex_offset + i0]), n1(sc.normals[oe.vertex_offset + i1]),
        n2(sc.normals[oe.vertex_offset + i2]);
    const ddgi_material& m = sc.materials[oe.material_index];
    T b1 = T(h.b1), b2 = T(h.b2);
    T b0 = T(1) - b1 - b2;
    V3<T> tsn = normalize(n0 * b0 + n1 * b1 + n2 * b2);
    const float* w = inst.w2o;
    V3<T> nw(tsn.x * T(w[0]) + tsn.y * T(w[4]) + tsn.z * T(w[8]),
             tsn.x * T(w[1]) + tsn.y * T(w[5]) + tsn.z * T(w[9]),
             tsn.x * T(w[2]) + tsn.y * T(w[6]) + tsn.z * T(w[10]));
    V3<T> normal = normalize(nw);
    V3<T> albedo(T(m.base_color[0]), T(m.base_color[1]), T(m.base_color[2]));
    if (P.albedo) {
        const T* a = P.albedo + 3 * (size_t)oe.material_index;
        albedo = V3<T>(a[0], a[1], a[2]);
    }
    T metal = T(m.metallic), rough = T(m.roughness);
    V3<T> color(T(m.emissive[0]), T(m.emissive[1]), T(m.emissive[2]));
    V3<T> f0(T(0.04));
    V3<T> diffuseColor = albedo * (V3<T>(T(1)) - f0);
    diffuseColor = diffuseColor * (T(1) - metal);
    V3<T> specularColor = mix3(f0, albedo, metal);
    V3<T> D(dir);
    V3<T> reflectDir = D - normal * (T(2) * dot(normal, D));
    V3<T> position(posf);
    V3<T> reflection = sample_probes<T>(position, reflectDir, -D, g, states, prev);
    color = color + specularColor * reflection;
    V3<T> indirect = sample_probes<T>(position, normal, -D, g, states, prev);
    color = color + indirect * diffuseColor;
    bool shadowed;
    if (shadow < 0) {
        Hit sh;
        shadowed = trace(sc, posf, L.dir, 0.1f, 10000.0f, 0xFFu, true, &sh);
    } else {
        shadowed = shadow != 0;
    }
    if (shadowed_out) *shadowed_out = shadowed;
    if (!shadowed) {
        color = color + pbr<T>(normal, normalize(-D), P.sun, V3<T>(L.dir), albedo, metal, rough);
        if (L.dir.y < 0.0f) {
            T f = T(1) - clampT(-T(L.dir.y), T(0), T(0.1)) / T(0.1);
            color = color * f;
        }
    }
    out[0] = color.x;
    out[1] = color.y;
    out[2] = color.z;
    out[3] = T(h.t);
}

inline F3 exact_probe_origin(const Grid& g, uint32_t linear) {
    int idx[3];
    grid_index(linear, g, idx);
    F3 cell((g.mx.x - g.mn.x) / (float)(g.res[0] - 1), (g.mx.y - g.mn.y) / (float)(g.res[1] - 1),
            (g.mx.z - g.mn.z) / (float)(g.res[2] - 1));
    F3 o;
    for (int k = 0; k < 3; ++k) {
        float p = (float)idx[k] * cell[k];
        o[k] = p + g.mn[k];
    }
    return o;
}

inline float exact_tmax(const Grid& g) {
    float dx = g.mx.x - g.mn.x, dy = g.mx.y - g.mn.y, dz = g.mx.z - g.mn.z;
    float a = dx * dx, b = dy * dy, c = dz * dz;
    return std::sqrt((a + b) + c);
}

// Blend of one probe (probesUpdate.glsl:49-121) + border copy (probesCopyBorders.comp).
template <class T>
void blend_probe(const Grid& g, uint32_t linear, const T* rays /* R x 4 */, const float* dirs /* R x 4 */,
                 Atlas<T>& at, uint32_t* states, bool update_state, bool do_depth = true) {
    int idx[3];
    grid_index(linear, g, idx);
    V3<T> cs = cell_size<T>(g);
    T gridCellSize = length(cs);
    int tile = idx[1] * g.res[0] + idx[0];
    // ---- colour ----
    {
        uint32_t n = g.colorRes - 2;
        T scale = T(texel_scale(n));
        T centre = T(0.5) * T(n - 1);
        int ox = (int)g.colorRes * tile, oy = (int)g.colorRes * idx[2];
        uint32_t outOfRange = 0;
        for (uint32_t r = 0; r < g.rays; ++r) {
            T dpt = rays[4 * r + 3];
            if (dpt < T(0) || dpt > gridCellSize) ++outOfRange;
        }
        T maxChange = 0;
        for (uint32_t ty = 0; ty < n; ++ty)
            for (uint32_t tx = 0; tx < n; ++tx) {
                V3<T> td;
                oct_decode(scale * (T(tx) - centre), scale * (T(ty) - centre), &td);
                T acc[4] = {0, 0, 0, 0};
                for (uint32_t r = 0; r < g.rays; ++r) {
                    V3<T> d(T(dirs[4 * r]), T(dirs[4 * r + 1]), T(dirs[4 * r + 2]));
                    T w = std::max(T(0), dot(td, d));
                    acc[0] += w * rays[4 * r + 0];
                    acc[1] += w * rays[4 * r + 1];
                    acc[2] += w * rays[4 * r + 2];
                    acc[3] += w;
                }
                if (acc[3] > T(1e-3)) {
                    acc[0] /= acc[3];
                    acc[1] /= acc[3];
                    acc[2] /= acc[3];
                }
                size_t px = (size_t)(ox + 1 + tx), py = (size_t)(oy + 1 + ty);
                T* texel = at.color + (py * at.cw + px) * 4;
                for (int c = 0; c < 3; ++c) maxChange = std::max(maxChange, (T)std::fabs(acc[c] - texel[c]));
                T h = T(g.hyst);
                for (int c = 0; c < 3; ++c) texel[c] = acc[c] * (T(1) - h) + texel[c] * h;
                if (g.quant)  // imageStore into the r11f_g11f_b10f image (probesUpdate.glsl:17, 103)
                    for (int c = 0; c < 3; ++c) texel[c] = round_color_store(texel[c], c);
                texel[3] = T(1);
            }
        if (update_state) {  // probesUpdate.glsl:110-119
            uint32_t& s = states[linear];
            if (outOfRange >= g.rays) {
                s = 8;
            } else {
                float mc = (float)maxChange;
                float sf = (float)s;
                if (mc < 0.02f / sf) s = std::min(s + 1u, 8u);
                else if (mc > 0.04f / sf) s = std::max(s - 1u, 1u);
                else if (mc > 0.25f) s = 1;
            }
        }
    }
    // ---- depth ----
    if (do_depth) {
        uint32_t n = g.depthRes - 2;
        T scale = T(texel_scale(n));
        T centre = T(0.5) * T(n - 1);
        int ox = (int)g.depthRes * tile, oy = (int)g.depthRes * idx[2];
        for (uint32_t ty = 0; ty < n; ++ty)
            for (uint32_t tx = 0; tx < n; ++tx) {
                V3<T> td;
                oct_decode(scale * (T(tx) - centre), scale * (T(ty) - centre), &td);
                T acc[3] = {0, 0, 0};
                for (uint32_t r = 0; r < g.rays; ++r) {
                    V3<T> d(T(dirs[4 * r]), T(dirs[4 * r + 1]), T(dirs[4 * r + 2]));
                    T depth = std::min(gridCellSize, rays[4 * r + 3]);
                    if (depth < T(0)) depth = gridCellSize;
                    T w = std::pow(std::max(T(0), dot(td, d)), T(g.sharp));
                    acc[0] += w * depth;
                    acc[1] += w * depth * depth;
                    acc[2] += w;
                }
                if (acc[2] > T(1e-3)) {
                    acc[0] /= acc[2];
                    acc[1] /= acc[2];
                }
                size_t px = (size_t)(ox + 1 + tx), py = (size_t)(oy + 1 + ty);
                T* texel = at.depth + (py * at.dw + px) * 2;
                T h = T(g.hyst);
                for (int c = 0; c < 2; ++c) texel[c] = acc[c] * (T(1) - h) + texel[c] * h;
                if (g.quant)  // imageStore into the rg16f image (probesUpdate.glsl:19)
                    for (int c = 0; c < 2; ++c) texel[c] = round_depth_store(texel[c]);
            }
    }
}

// Border copy for one tile of side n (probesCopyBorders.comp:21-245, generalised).
template <class T>
void copy_borders(T* img, uint32_t w, int ch, int ox, int oy, int n) {
    auto at = [&](int x, int y) { return img + ((size_t)(oy + y) * w + (size_t)(ox + x)) * ch; };
    auto cp = [&](int dx, int dy, int sx, int sy) {
        const T* s = at(sx, sy);
        T* d = at(dx, dy);
        for (int c = 0; c < ch; ++c) d[c] = s[c];
    };
    cp(0, 0, n - 2, n - 2);
    cp(0, n - 1, n - 2, 1);
    cp(n - 1, 0, 1, n - 2);
    cp(n - 1, n - 1, 1, 1);
    for (int j = 1; j <= n - 2; ++j) {
        cp(0, j, 1, n - 1 - j);
        cp(n - 1, j, n - 2, n - 1 - j);
        cp(j, 0, n - 1 - j, 1);
        cp(j, n - 1, n - 1 - j, n - 2);
    }
}

template <class T>
int run_update(const Scene& sc, const ddgi_grid_desc* gd, const ddgi_light* ld, const float orientation[9],
               const uint32_t* list, uint32_t nlist, uint32_t* states, T* color, T* depth, float* ray_out,
               ddgi_hit* hit_out, int nthreads) {
    Grid g = make_grid(gd);
    Light L;
    L.dir = F3(ld->direction[0], ld->direction[1], ld->direction[2]);
    L.color = F3(ld->color[0], ld->color[1], ld->color[2]);
    L.sky = F3(ld->sky[0], ld->sky[1], ld->sky[2]);
    L.brightness = ld->color[3];
    const uint32_t R = g.rays;
    std::vector<float> dirs(4 * (size_t)R);
    ddgi_ray_direction_table(orientation, R, dirs.data());
    Atlas<T> at;
    at.color = color;
    at.depth = depth;
    at.cw = g.colorRes * g.res[0] * g.res[1];
    at.ch = g.colorRes * g.res[2];
    at.dw = g.depthRes * g.res[0] * g.res[1];
    at.dh = g.depthRes * g.res[2];
    std::vector<uint32_t> probes;
    if (list) probes.assign(list, list + nlist);
    else {
        probes.resize(g.count());
        for (uint32_t i = 0; i < g.count(); ++i) probes[i] = i;
    }
    const size_t np = probes.size();
    std::vector<T> rays(np * R * 4);
    float tmax = exact_tmax(g);
    // Phase 1: trace + shade against the previous atlas (read-only).
    parallel_for(np, nthreads, [&](size_t b, size_t e) {
        for (size_t s = b; s < e; ++s) {
            F3 o = exact_probe_origin(g, probes[s]);
            for (uint32_t r = 0; r < R; ++r) {
                F3 d(dirs[4 * r], dirs[4 * r + 1], dirs[4 * r + 2]);
                Hit h;
                shade_ray<T>(sc, g, L, states, at, o, d, tmax, &rays[(s * R + r) * 4], &h);
                if (hit_out) {
                    ddgi_hit& ho = hit_out[s * R + r];
                    ho.instance = h.inst;
                    ho.primitive = h.valid() ? h.prim : 0;
                    ho.t = h.valid() ? h.t : 0.0f;
                    ho.backface = h.valid() && h.backface ? 1 : 0;
                }
            }
        }
    });
    if (ray_out)
        for (size_t i = 0; i < rays.size(); ++i) ray_out[i] = (float)rays[i];
    // Phase 2: blend + border copy per probe (disjoint tiles).
    std::vector<uint32_t> new_states(states, states + g.count());
    parallel_for(np, nthreads, [&](size_t b, size_t e) {
        for (size_t s = b; s < e; ++s) {
            uint32_t p = probes[s];
            blend_probe<T>(g, p, &rays[s * R * 4], dirs.data(), at, new_states.data(), true);
            int idx[3];
            grid_index(p, g, idx);
            int tile = idx[1] * g.res[0] + idx[0];
            copy_borders<T>(at.color, at.cw, 4, (int)g.colorRes * tile, (int)g.colorRes * idx[2], (int)g.colorRes);
            copy_borders<T>(at.depth, at.dw, 2, (int)g.depthRes * tile, (int)g.depthRes * idx[2], (int)g.depthRes);
        }
    });
    std::memcpy(states, new_states.data(), sizeof(uint32_t) * g.count());
    return 0;
}

// A recorded probe ray: closest hit and shadow result, so that later
// forward passes can replay shading + blend with other parameters while the
// hit set stays fixed (the differentiation workload's assumption).
struct RecHit {
    uint32_t inst, prim;
    float t, b1, b2;
    uint32_t flags;  // bit 0 backface, bit 1 shadowed
};

// K successive updates of every probe.  replay = false traces (and records
// into `rec` when given); replay = true shades the recorded hits instead.
// depth_snap (K depth atlases) receives the depth atlas after every update
// when recording; replays copy it back instead of re-blending depth, which
// does not depend on the parameters once the hits are fixed.
template <class T>
int run_chain(const Scene& sc, const ddgi_grid_desc* gd, const ddgi_light* ld, const ShadeParams<T>* Pover,
              const float* orientations, uint32_t K, uint32_t* states, T* color, T* depth, RecHit* rec, bool replay,
              T* depth_snap, int nthreads) {
    Grid g = make_grid(gd);
    Light L;
    L.dir = F3(ld->direction[0], ld->direction[1], ld->direction[2]);
    L.color = F3(ld->color[0], ld->color[1], ld->color[2]);
    L.sky = F3(ld->sky[0], ld->sky[1], ld->sky[2]);
    L.brightness = ld->color[3];
    ShadeParams<T> P = Pover ? *Pover : default_params<T>(L);
    const uint32_t R = g.rays, NP = g.count();
    Atlas<T> at;
    at.color = color;
    at.depth = depth;
    at.cw = g.colorRes * g.res[0] * g.res[1];
    at.ch = g.colorRes * g.res[2];
    at.dw = g.depthRes * g.res[0] * g.res[1];
    at.dh = g.depthRes * g.res[2];
    const float tmax = exact_tmax(g);
    std::vector<float> dirs(4 * (size_t)R);
    std::vector<T> rays((size_t)NP * R * 4);
    for (uint32_t k = 0; k < K; ++k) {
        ddgi_ray_direction_table(orientations + 9 * (size_t)k, R, dirs.data());
        RecHit* rk = rec ? rec + (size_t)k * NP * R : nullptr;
        parallel_for(NP, nthreads, [&](size_t b, size_t e) {
            for (size_t p = b; p < e; ++p) {
                F3 o = exact_probe_origin(g, (uint32_t)p);
                for (uint32_t r = 0; r < R; ++r) {
                    F3 d(dirs[4 * r], dirs[4 * r + 1], dirs[4 * r + 2]);
                    T* out = &rays[(p * R + r) * 4];
                    size_t ri = p * R + r;
                    if (replay) {
                        const RecHit& q = rk[ri];
                        Hit h;
                        h.inst = q.inst;
                        h.prim = q.prim;
                        h.t = q.t;
                        h.b1 = q.b1;
                        h.b2 = q.b2;
                        h.backface = (q.flags & 1u) != 0;
                        shade_hit<T>(sc, g, L, P, states, at, o, d, h, (q.flags & 2u) ? 1 : 0, nullptr, out);
                    } else {
                        Hit h;
                        trace(sc, o, d, 0.01f, tmax, 0x3u, false, &h);
                        bool sh = false;
                        shade_hit<T>(sc, g, L, P, states, at, o, d, h, -1, &sh, out);
                        if (rk) {
                            RecHit& q = rk[ri];
                            q.inst = h.inst;
                            q.prim = h.valid() ? h.prim : 0;
                            q.t = h.valid() ? h.t : 0.0f;
                            q.b1 = h.b1;
                            q.b2 = h.b2;
                            q.flags = (h.valid() && h.backface ? 1u : 0u) | (sh ? 2u : 0u);
                        }
                    }
                }
            }
        });
        std::vector<uint32_t> ns(states, states + NP);
        const bool depth_from_snap = replay && depth_snap;
        parallel_for(NP, nthreads, [&](size_t b, size_t e) {
            for (size_t p = b; p < e; ++p) {
                blend_probe<T>(g, (uint32_t)p, &rays[p * R * 4], dirs.data(), at, ns.data(), true, !depth_from_snap);
                int idx[3];
                grid_index((uint32_t)p, g, idx);
                int tile = idx[1] * g.res[0] + idx[0];
                copy_borders<T>(at.color, at.cw, 4, (int)g.colorRes * tile, (int)g.colorRes * idx[2], (int)g.colorRes);
                if (!depth_from_snap)
                    copy_borders<T>(at.depth, at.dw, 2, (int)g.depthRes * tile, (int)g.depthRes * idx[2],
                                    (int)g.depthRes);
            }
        });
        std::memcpy(states, ns.data(), sizeof(uint32_t) * NP);
        const size_t dn = (size_t)at.dw * at.dh * 2;
        if (depth_snap) {
            if (depth_from_snap) std::memcpy(depth, depth_snap + (size_t)k * dn, dn * sizeof(T));
            else std::memcpy(depth_snap + (size_t)k * dn, depth, dn * sizeof(T));
        }
    }
    return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// C API (loaded with ctypes by the tests and the benchmark's CPU leg)
// ---------------------------------------------------------------------------
extern "C" {

struct oracle_scene {
    Scene s;
};

oracle_scene* oracle_scene_create(const ddgi_scene_desc* d, int nthreads) {
    auto* os = new oracle_scene();
    Scene& sc = os->s;
    sc.normals.resize(d->vertex_count);
    for (uint32_t i = 0; i < d->vertex_count; ++i)
        sc.normals[i] = F3(d->vertices[i].normal[0], d->vertices[i].normal[1], d->vertices[i].normal[2]);
    sc.indices.assign(d->indices, d->indices + d->index_count);
    sc.offsets.assign(d->offsets, d->offsets + d->offset_count);
    sc.materials.assign(d->materials, d->materials + d->material_count);
    sc.meshes.resize(d->mesh_count);
    parallel_for(d->mesh_count, nthreads, [&](size_t b, size_t e) {
        for (size_t mi = b; mi < e; ++mi) {
            const ddgi_mesh& m = d->meshes[mi];
            MeshData& md = sc.meshes[mi];
            uint32_t nt = m.index_count / 3;
            md.v0.resize(nt);
            md.v1.resize(nt);
            md.v2.resize(nt);
            std::vector<Box> boxes(nt);
            for (uint32_t t = 0; t < nt; ++t) {
                const float* p[3];
                for (int k = 0; k < 3; ++k) {
                    uint32_t vi = m.vertex_offset + d->indices[m.index_offset + 3 * t + k];
                    p[k] = d->vertices[vi].pos;
                }
                md.v0[t] = F3(p[0][0], p[0][1], p[0][2]);
                md.v1[t] = F3(p[1][0], p[1][1], p[1][2]);
                md.v2[t] = F3(p[2][0], p[2][1], p[2][2]);
                for (int k = 0; k < 3; ++k) boxes[t].grow(p[k]);
                md.bounds.grow(boxes[t]);
            }
            build_bvh(md.bvh, boxes);
        }
    });
    sc.instances.resize(d->instance_count);
    std::vector<Box> iboxes(d->instance_count);
    for (uint32_t i = 0; i < d->instance_count; ++i) {
        const ddgi_instance& in = d->instances[i];
        InstanceData& id = sc.instances[i];
        std::memcpy(id.o2w, in.transform, sizeof(id.o2w));
        if (!ddgi_affine_inverse(in.transform, id.w2o)) std::memset(id.w2o, 0, sizeof(id.w2o));
        id.custom = in.custom_index & 0xFFFFFFu;
        id.mask = in.mask & 0xFFu;
        id.mesh = in.mesh_index;
        const Box& mb = sc.meshes[in.mesh_index].bounds;
        Box wb;
        for (int c = 0; c < 8; ++c) {
            double p[3] = {(c & 1) ? mb.hi[0] : mb.lo[0], (c & 2) ? mb.hi[1] : mb.lo[1], (c & 4) ? mb.hi[2] : mb.lo[2]};
            float q[3];
            for (int r = 0; r < 3; ++r)
                q[r] = (float)(in.transform[4 * r] * p[0] + in.transform[4 * r + 1] * p[1] + in.transform[4 * r + 2] * p[2] +
                               in.transform[4 * r + 3]);
            wb.grow(q);
        }
        wb.enlarge();
        iboxes[i] = wb;
    }
    build_bvh(sc.tlas, iboxes);
    return os;
}

void oracle_scene_destroy(oracle_scene* s) { delete s; }

// Closest hit (any_hit = 0) or shadow query (any_hit = 1) for n rays.
void oracle_trace(const oracle_scene* s, const float* origins, const float* dirs, uint32_t n, float tmin, float tmax,
                  uint32_t mask, int any_hit, ddgi_hit* out, float* bary, int nthreads) {
    parallel_for(n, nthreads, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            Hit h;
            trace(s->s, F3(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]),
                  F3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]), tmin, tmax, mask, any_hit != 0, &h);
            out[i].instance = h.inst;
            out[i].primitive = h.valid() ? h.prim : 0;
            out[i].t = h.valid() ? h.t : 0.0f;
            out[i].backface = h.valid() && h.backface ? 1 : 0;
            if (bary) {
                bary[2 * i] = h.b1;
                bary[2 * i + 1] = h.b2;
            }
        }
    }, 64);
}

// One probe update.  fp64 != 0: atlases are double arrays, else float.
// states: probe states (in/out).  ray_out (np*R*4 floats) and hit_out may be NULL.
int oracle_update(const oracle_scene* s, const ddgi_grid_desc* g, const ddgi_light* l, const float orientation[9],
                  const uint32_t* list, uint32_t nlist, uint32_t* states, void* color, void* depth, int fp64,
                  float* ray_out, ddgi_hit* hit_out, int nthreads) {
    if (fp64)
        return run_update<double>(s->s, g, l, orientation, list, nlist, states, (double*)color, (double*)depth, ray_out,
                                  hit_out, nthreads);
    return run_update<float>(s->s, g, l, orientation, list, nlist, states, (float*)color, (float*)depth, ray_out,
                             hit_out, nthreads);
}

// Trace + shade (float) of n given probe rays against a previous atlas:
// rays[8 k ...] = origin, direction, tmin, tmax; out[4 k ...] = radiance and
// hit distance as the probe update records them.  For checking the shading
// against the reference's own stages on the same rays.
void oracle_shade_rays(const oracle_scene* s, const ddgi_grid_desc* gd, const ddgi_light* ld, const uint32_t* states,
                       const float* color, const float* depth, const float* rays, uint32_t n, float* out, int nthreads) {
    Grid g = make_grid(gd);
    Light L;
    L.dir = F3(ld->direction[0], ld->direction[1], ld->direction[2]);
    L.color = F3(ld->color[0], ld->color[1], ld->color[2]);
    L.sky = F3(ld->sky[0], ld->sky[1], ld->sky[2]);
    L.brightness = ld->color[3];
    Atlas<float> at;
    at.color = const_cast<float*>(color);
    at.depth = const_cast<float*>(depth);
    at.cw = g.colorRes * g.res[0] * g.res[1];
    at.ch = g.colorRes * g.res[2];
    at.dw = g.depthRes * g.res[0] * g.res[1];
    at.dh = g.depthRes * g.res[2];
    parallel_for(n, nthreads, [&](size_t b, size_t e) {
        for (size_t k = b; k < e; ++k) {
            const float* r = rays + 8 * k;
            const F3 o(r[0], r[1], r[2]), d(r[3], r[4], r[5]);
            Hit h;
            trace(s->s, o, d, r[6], r[7], 0x3u, false, &h);
            shade_hit<float>(s->s, g, L, default_params<float>(L), states, at, o, d, h, -1, nullptr, out + 4 * k);
        }
    }, 64);
}

// Blend + border only, from given ray records (R x 4 per listed probe) — for
// checking the blend kernel in isolation.
int oracle_blend(const ddgi_grid_desc* gd, const float orientation[9], const uint32_t* list, uint32_t nlist,
                 const float* rays, uint32_t* states, float* color, float* depth, int nthreads);

// FP64 form of oracle_blend (float ray records, double atlases).
int oracle_blend64(const ddgi_grid_desc* gd, const float orientation[9], const uint32_t* list, uint32_t nlist,
                   const float* rays, uint32_t* states, double* color, double* depth, int nthreads) {
    Grid g = make_grid(gd);
    std::vector<float> dirs(4 * (size_t)g.rays);
    ddgi_ray_direction_table(orientation, g.rays, dirs.data());
    Atlas<double> at;
    at.color = color;
    at.depth = depth;
    at.cw = g.colorRes * g.res[0] * g.res[1];
    at.ch = g.colorRes * g.res[2];
    at.dw = g.depthRes * g.res[0] * g.res[1];
    at.dh = g.depthRes * g.res[2];
    std::vector<uint32_t> probes;
    if (list) probes.assign(list, list + nlist);
    else {
        probes.resize(g.count());
        for (uint32_t i = 0; i < g.count(); ++i) probes[i] = i;
    }
    std::vector<uint32_t> ns(states, states + g.count());
    parallel_for(probes.size(), nthreads, [&](size_t b, size_t e) {
        std::vector<double> rd(4 * (size_t)g.rays);
        for (size_t s2 = b; s2 < e; ++s2) {
            uint32_t p = probes[s2];
            for (size_t i = 0; i < rd.size(); ++i) rd[i] = rays[s2 * g.rays * 4 + i];
            blend_probe<double>(g, p, rd.data(), dirs.data(), at, ns.data(), true);
            int idx[3];
            grid_index(p, g, idx);
            int tile = idx[1] * g.res[0] + idx[0];
            copy_borders<double>(at.color, at.cw, 4, (int)g.colorRes * tile, (int)g.colorRes * idx[2], (int)g.colorRes);
            copy_borders<double>(at.depth, at.dw, 2, (int)g.depthRes * tile, (int)g.depthRes * idx[2], (int)g.depthRes);
        }
    });
    std::memcpy(states, ns.data(), sizeof(uint32_t) * g.count());
    return 0;
}

int oracle_blend(const ddgi_grid_desc* gd, const float orientation[9], const uint32_t* list, uint32_t nlist,
                 const float* rays, uint32_t* states, float* color, float* depth, int nthreads) {
    Grid g = make_grid(gd);
    std::vector<float> dirs(4 * (size_t)g.rays);
    ddgi_ray_direction_table(orientation, g.rays, dirs.data());
    Atlas<float> at;
    at.color = color;
    at.depth = depth;
    at.cw = g.colorRes * g.res[0] * g.res[1];
    at.ch = g.colorRes * g.res[2];
    at.dw = g.depthRes * g.res[0] * g.res[1];
    at.dh = g.depthRes * g.res[2];
    std::vector<uint32_t> probes;
    if (list) probes.assign(list, list + nlist);
    else {
        probes.resize(g.count());
        for (uint32_t i = 0; i < g.count(); ++i) probes[i] = i;
    }
    std::vector<uint32_t> ns(states, states + g.count());
    parallel_for(probes.size(), nthreads, [&](size_t b, size_t e) {
        for (size_t s2 = b; s2 < e; ++s2) {
            uint32_t p = probes[s2];
            blend_probe<float>(g, p, rays + s2 * g.rays * 4, dirs.data(), at, ns.data(), true);
            int idx[3];
            grid_index(p, g, idx);
            int tile = idx[1] * g.res[0] + idx[0];
            copy_borders<float>(at.color, at.cw, 4, (int)g.colorRes * tile, (int)g.colorRes * idx[2], (int)g.colorRes);
            copy_borders<float>(at.depth, at.dw, 2, (int)g.depthRes * tile, (int)g.depthRes * idx[2], (int)g.depthRes);
        }
    });
    std::memcpy(states, ns.data(), sizeof(uint32_t) * g.count());
    return 0;
}

// Border-copy table for a tile of side n: (dst x, dst y, src x, src y) per
// entry, in the order corners, x = 0 / x = n-1 columns, y = 0 / y = n-1 rows.
uint32_t oracle_border_table(int n, int* out) {
    std::vector<int> v;
    auto cp = [&](int dx, int dy, int sx, int sy) { v.insert(v.end(), {dx, dy, sx, sy}); };
    cp(0, 0, n - 2, n - 2);
    cp(0, n - 1, n - 2, 1);
    cp(n - 1, 0, 1, n - 2);
    cp(n - 1, n - 1, 1, 1);
    for (int j = 1; j <= n - 2; ++j) cp(0, j, 1, n - 1 - j);
    for (int j = 1; j <= n - 2; ++j) cp(n - 1, j, n - 2, n - 1 - j);
    for (int j = 1; j <= n - 2; ++j) cp(j, 0, n - 1 - j, 1);
    for (int j = 1; j <= n - 2; ++j) cp(j, n - 1, n - 1 - j, n - 2);
    if (out) std::memcpy(out, v.data(), v.size() * sizeof(int));
    return (uint32_t)(v.size() / 4);
}

// Single math entry points for known-answer tests.
void oracle_oct_decode(float x, float y, float* out3) {
    V3<float> v;
    oct_decode(x, y, &v);
    out3[0] = v.x; out3[1] = v.y; out3[2] = v.z;
}
void oracle_sphere_to_oct_uv(const float* d3, float* uv) {
    sphere_to_oct_uv(F3(d3[0], d3[1], d3[2]), &uv[0], &uv[1]);
}
float oracle_texel_scale(uint32_t n) { return texel_scale(n); }
void oracle_probe_world_position(const ddgi_grid_desc* gd, uint32_t index, float* out3) {
    const Grid g = make_grid(gd);
    int idx[3];
    grid_index(index, g, idx);
    const F3 p = probe_pos<float>(idx, g);
    out3[0] = p.x; out3[1] = p.y; out3[2] = p.z;
}
// Miss radiance of later calls: 0 constant sky radiance, 1 atmospheric sky.
void oracle_set_sky_mode(int mode) { g_sky_mode.store(mode); }
// The atmospheric sky in float (sky.glsl's sky() with showSun = true).
void oracle_sky(const float* origin, const float* dir, const float* sun_pos, const float* sun_color, float brightness,
                float* out3) {
    const F3 c = atmosphere<float>(F3(origin[0], origin[1], origin[2]), F3(dir[0], dir[1], dir[2]),
                                   F3(sun_pos[0], sun_pos[1], sun_pos[2]), F3(sun_color[0], sun_color[1], sun_color[2]),
                                   brightness);
    out3[0] = c.x; out3[1] = c.y; out3[2] = c.z;
}

// Reference-format storage rounding of n values: kind 0 = 11-bit unsigned
// float (red, green), 1 = 10-bit unsigned float (blue), 2 = half.
void oracle_round_store(int kind, const float* in, float* out, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i)
        out[i] = kind == 0 ? ddgi_round_r11(in[i]) : (kind == 1 ? ddgi_round_b10(in[i]) : ddgi_round_half(in[i]));
}
void oracle_direction_table(const float orientation[9], uint32_t n, float* out4) {
    ddgi_ray_direction_table(orientation, n, out4);
}
void oracle_pbr(const float* n, const float* v, const float* lc, const float* ldir, const float* albedo, float metal,
                float rough, float* out3) {
    F3 r = pbr<float>(F3(n[0], n[1], n[2]), F3(v[0], v[1], v[2]), F3(lc[0], lc[1], lc[2]), F3(ldir[0], ldir[1], ldir[2]),
                      F3(albedo[0], albedo[1], albedo[2]), metal, rough);
    out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
}
// sampleProbes on a float atlas with all-ON (or given) states.
void oracle_sample_probes(const ddgi_grid_desc* gd, const uint32_t* states, const float* color, const float* depth,
                          const float* pos, const float* nrm, const float* view, float* out3) {
    Grid g = make_grid(gd);
    Atlas<float> at;
    at.color = const_cast<float*>(color);
    at.depth = const_cast<float*>(depth);
    at.cw = g.colorRes * g.res[0] * g.res[1];
    at.ch = g.colorRes * g.res[2];
    at.dw = g.depthRes * g.res[0] * g.res[1];
    at.dh = g.depthRes * g.res[2];
    F3 r = sample_probes<float>(F3(pos[0], pos[1], pos[2]), F3(nrm[0], nrm[1], nrm[2]), F3(view[0], view[1], view[2]), g,
                                states, at);
    out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Differentiation support: K-update chains in FP64 with a recorded hit set.
// ---------------------------------------------------------------------------
extern "C" {

uint32_t oracle_rec_hit_bytes(void) { return (uint32_t)sizeof(RecHit); }

// FP64 forward over all probes for K updates (orientations: K x 9), tracing
// and recording every ray's hit and shadow result into rec (K * P * R).
int oracle_record(const oracle_scene* s, const ddgi_grid_desc* g, const ddgi_light* l, const float* orientations,
                  uint32_t K, uint32_t* states, double* color, double* depth, void* rec, double* depth_snap,
                  int nthreads) {
    return run_chain<double>(s->s, g, l, nullptr, orientations, K, states, color, depth, static_cast<RecHit*>(rec),
                             false, depth_snap, nthreads);
}

// FP64 forward replaying a recorded hit set with the given parameters:
// albedo (material_count x 3, NULL = the materials' base colour), sun and
// sky radiance (3 doubles each).
// Probe classification, probesInit.rgen:31-64 with probeInitMiss.rmiss:11-14
// and backfaceTest.rchit:11-15: 512 closest-hit rays per probe (mask
// INSTANCE_STATIC = 1, InstanceMasks.glsl:1), direction i = orientation *
// sphericalFibonacci(i, raysPerProbe) (for i >= raysPerProbe the formula
// gives the degenerate (0, 0, cos) directions, kept as the shader has them),
// t in [0.01, 1.5 |cell|].  Hits closer than |cell| (:44): back faces are
// counted (:45); a hit position within one cell of the probe on every axis
// (:46-48, position rounded as product then sum) marks the probe near
// geometry.  State (:52-59): 0 if back-face hits > raysPerProbe / 2, else 1
// near geometry, else 8.
void oracle_init_probes(const oracle_scene* s, const ddgi_grid_desc* gd, const float orientation[9], uint32_t* states,
                        int nthreads) {
    const Grid g = make_grid(gd);
    const F3 cell = cell_size<float>(g);
    const float max_distance = length(cell);
    const float tmax = 1.5f * max_distance;
    std::vector<F3> dirs(512);
    for (uint32_t i = 0; i < 512; ++i) {
        float d[4];
        ddgi_ray_direction(orientation, i, g.rays, d);
        dirs[i] = F3(d[0], d[1], d[2]);
    }
    parallel_for(g.count(), nthreads, [&](size_t b, size_t e) {
        for (size_t p = b; p < e; ++p) {
            const F3 o = exact_probe_origin(g, (uint32_t)p);
            uint32_t back = 0;
            bool near = false;
            for (uint32_t i = 0; i < 512; ++i) {
                Hit h;
                trace(s->s, o, dirs[i], 0.01f, tmax, 0x1u, false, &h);
                if (!h.valid() || !(h.t < max_distance)) continue;
                if (h.backface) ++back;
                F3 pos;
                for (int k = 0; k < 3; ++k) pos[k] = dirs[i][k] * h.t + o[k];
                F3 dist = vabs(pos - o);
                if (dist.x < cell.x && dist.y < cell.y && dist.z < cell.z) near = true;
            }
            states[p] = (float)back > 0.5f * (float)g.rays ? 0u : (near ? 1u : 8u);
        }
    }, 1);
}

// Final gather, src/shaders/FinalGather.frag:39-80 per pixel: sky radiance
// where depth <= 0 (the constant sky replacing sky.glsl), else
// direct * pbrMetallicRoughness(sun) + mix(0.004, albedo, metal) * reflection
// + sampleProbes(position, normal, view) * albedo * (1 - 0.004) * (1 - metal)
// + emissive, view = normalize(camera - position), normal normalised.
void oracle_final_gather(const ddgi_grid_desc* gd, const ddgi_light* ld, const uint32_t* states, const float* color,
                         const float* depth, uint32_t pixels, const float* position_depth,
                         const float* normal_metalness, const float* albedo_roughness, const float* emissive,
                         const float* direct_light, const float* reflection, const float* origin, float* out,
                         int nthreads) {
    const Grid g = make_grid(gd);
    Atlas<float> at;
    at.color = const_cast<float*>(color);
    at.depth = const_cast<float*>(depth);
    at.cw = g.colorRes * g.res[0] * g.res[1];
    at.ch = g.colorRes * g.res[2];
    at.dw = g.depthRes * g.res[0] * g.res[1];
    at.dh = g.depthRes * g.res[2];
    const F3 cam(origin[0], origin[1], origin[2]);
    const F3 lc(ld->color[0], ld->color[1], ld->color[2]), ldir(ld->direction[0], ld->direction[1], ld->direction[2]);
    parallel_for(pixels, nthreads, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            const float* pd = position_depth + 4 * i;
            float* o = out + 4 * i;
            if (!(pd[3] > 0.0f)) {  // FinalGather.frag:55-57
                F3 sky(ld->sky[0], ld->sky[1], ld->sky[2]);
                if (g_sky_mode.load())  // view direction in position.xyz, brightness 1
                    sky = atmosphere<float>(cam, normalize(F3(pd[0], pd[1], pd[2])), ldir, lc, 1.0f);
                o[0] = sky.x;
                o[1] = sky.y;
                o[2] = sky.z;
                o[3] = 1.0f;
                continue;
            }
            const float* nm = normal_metalness + 4 * i;
            const float* ar = albedo_roughness + 4 * i;
            const F3 position(pd[0], pd[1], pd[2]);
            const F3 normal = normalize(F3(nm[0], nm[1], nm[2]));
            const F3 albedo(ar[0], ar[1], ar[2]);
            const float metal = nm[3], rough = ar[3];
            const F3 view = normalize(cam - position);
            F3 c = pbr<float>(normal, view, lc, ldir, albedo, metal, rough) * direct_light[i];
            const float f0 = 0.004f;
            const F3 diffuse = albedo * (1.0f - f0) * (1.0f - metal);
            const F3 specular = mix3(F3(f0, f0, f0), albedo, metal);
            const F3 refl = reflection ? F3(reflection[4 * i], reflection[4 * i + 1], reflection[4 * i + 2])
                                       : F3(0.0f, 0.0f, 0.0f);
            c = c + specular * refl;
            c = c + sample_probes<float>(position, normal, view, g, states, at) * diffuse;
            c = c + F3(emissive[4 * i], emissive[4 * i + 1], emissive[4 * i + 2]);
            o[0] = c.x;
            o[1] = c.y;
            o[2] = c.z;
            o[3] = 1.0f;
        }
    }, 256);
}

int oracle_replay(const oracle_scene* s, const ddgi_grid_desc* g, const ddgi_light* l, const double* albedo,
                  const double* sun, const double* sky, const float* orientations, uint32_t K, uint32_t* states,
                  double* color, double* depth, const void* rec, const double* depth_snap, int nthreads) {
    ShadeParams<double> P;
    P.albedo = albedo;
    P.sun = V3<double>(sun[0], sun[1], sun[2]);
    P.sky = V3<double>(sky[0], sky[1], sky[2]);
    return run_chain<double>(s->s, g, l, &P, orientations, K, states, color, depth,
                             const_cast<RecHit*>(static_cast<const RecHit*>(rec)), true,
                             const_cast<double*>(depth_snap), nthreads);
}

}  // extern "C"

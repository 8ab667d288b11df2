// glsl_compute.hpp — what the reference's compute shaders
// (src/shaders/probesUpdate.glsl through probesUpdateIrradiance.comp and
// probesUpdateDepth.comp, and probesCopyBorders.comp) need beyond
// glsl_shim.hpp to run on the host: unsigned vectors, matrices, the built-in
// invocation IDs, storage images with their formats' rounding on store,
// workgroup barriers and shared-memory atomics, and a dispatch that runs
// every invocation of a workgroup as its own thread; and what
// FinalGather.frag adds: subpass inputs read at the current fragment and
// inverse(mat4).  Test infrastructure: built by oracle/build_ref_glsl.py
// into oracle/_ref/, loaded only by tests and the fixture generator.
//
// Execution model: workgroups run one after the other (the shaders'
// workgroups touch disjoint texels and probe states); inside a workgroup all
// invocations run concurrently as threads, so barrier() is a real execution
// barrier and `shared` variables (file-scope statics in the translated
// source) are shared by exactly the invocations of one workgroup.  A
// shader's private globals are thread_local.
//
// One departure, stated where the shader needs it: groupMemoryBarrier()
// also waits for the whole workgroup.  probesUpdate.glsl reads the
// workgroup's shared maximum after an atomicMax and only a memory barrier;
// on a GPU that read races with the other invocations' atomics, and the
// barrier here gives the value the code is written to compute (the maximum
// over all texels).
#pragma once

#include <string.h>

#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "glsl_shim.hpp"

namespace glsl {

template <int A, int B>
struct uswz2 {
    uint e[3];
    operator uvec2() const { return uvec2{e[A], e[B]}; }
};
struct uvec3;
struct uswz3 {
    uint e[3];
    operator uvec3() const;
};
struct uvec3 {
    union {
        struct {
            uint x, y, z;
        };
        uswz2<0, 1> xy;
        uswz2<1, 2> yz;
        uswz3 xyz;
    };
    uvec3() { x = y = z = 0u; }
    uvec3(uint a, uint b, uint c) {
        x = a;
        y = b;
        z = c;
    }
    uvec3(const uvec3& o) {
        x = o.x;
        y = o.y;
        z = o.z;
    }
    uvec3& operator=(const uvec3& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        return *this;
    }
};
inline uswz3::operator uvec3() const { return uvec3(e[0], e[1], e[2]); }
inline ivec3::ivec3(const uvec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}

// Matrices are arrays of columns, as in GLSL.
struct mat4 {
    vec4 c[4];
};
struct mat4x3 {  // 4 columns of 3 rows
    vec3 c[4];
};
struct mat3 {
    vec3 c[3];
    mat3(const vec3& a, const vec3& b, const vec3& d) {
        c[0] = a;
        c[1] = b;
        c[2] = d;
    }
    explicit mat3(const mat4& m) {
        for (int i = 0; i < 3; ++i) c[i] = vec3(m.c[i]);
    }
    explicit mat3(const mat4x3& m) {
        for (int i = 0; i < 3; ++i) c[i] = m.c[i];
    }
};
inline vec3 operator*(const mat3& m, const vec3& v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z; }
inline vec4 operator*(const mat4& m, const vec4& v) {
    return ((m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z) + m.c[3] * v.w;
}
// inverse(mat4): the adjugate over the determinant, by 2x2 minors, in float.
inline mat4 inverse(const mat4& M) {
    float a[4][4];  // a[row][col]
    for (int c = 0; c < 4; ++c) {
        a[0][c] = M.c[c].x, a[1][c] = M.c[c].y, a[2][c] = M.c[c].z, a[3][c] = M.c[c].w;
    }
    const float s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1], s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2];
    const float s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3], s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2];
    const float s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3], s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3];
    const float c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3], c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3];
    const float c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2], c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3];
    const float c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2], c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1];
    const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    const float r = 1.0f / det;
    float b[4][4];
    b[0][0] = (a[1][1] * c5 - a[1][2] * c4 + a[1][3] * c3) * r;
    b[0][1] = (-a[0][1] * c5 + a[0][2] * c4 - a[0][3] * c3) * r;
    b[0][2] = (a[3][1] * s5 - a[3][2] * s4 + a[3][3] * s3) * r;
    b[0][3] = (-a[2][1] * s5 + a[2][2] * s4 - a[2][3] * s3) * r;
    b[1][0] = (-a[1][0] * c5 + a[1][2] * c2 - a[1][3] * c1) * r;
    b[1][1] = (a[0][0] * c5 - a[0][2] * c2 + a[0][3] * c1) * r;
    b[1][2] = (-a[3][0] * s5 + a[3][2] * s2 - a[3][3] * s1) * r;
    b[1][3] = (a[2][0] * s5 - a[2][2] * s2 + a[2][3] * s1) * r;
    b[2][0] = (a[1][0] * c4 - a[1][1] * c2 + a[1][3] * c0) * r;
    b[2][1] = (-a[0][0] * c4 + a[0][1] * c2 - a[0][3] * c0) * r;
    b[2][2] = (a[3][0] * s4 - a[3][1] * s2 + a[3][3] * s0) * r;
    b[2][3] = (-a[2][0] * s4 + a[2][1] * s2 - a[2][3] * s0) * r;
    b[3][0] = (-a[1][0] * c3 + a[1][1] * c1 - a[1][2] * c0) * r;
    b[3][1] = (a[0][0] * c3 - a[0][1] * c1 + a[0][2] * c0) * r;
    b[3][2] = (-a[3][0] * s3 + a[3][1] * s1 - a[3][2] * s0) * r;
    b[3][3] = (a[2][0] * s3 - a[2][1] * s1 + a[2][2] * s0) * r;
    mat4 out;
    for (int c = 0; c < 4; ++c) out.c[c] = vec4(b[0][c], b[1][c], b[2][c], b[3][c]);
    return out;
}

// Fragment-stage inputs: one value per pixel of the current fragment.
struct subpassInput {
    const float* texels = nullptr;  // 4 floats per pixel
};
inline thread_local size_t gl_current_pixel = 0;
inline vec4 subpassLoad(const subpassInput& s) {
    const float* t = s.texels + 4 * gl_current_pixel;
    return vec4(t[0], t[1], t[2], t[3]);
}
// row vector times matrix: one dot product per column
inline vec4 operator*(const vec3& v, const mat4x3& m) {
    return vec4(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2]), dot(v, m.c[3]));
}

// int vectors convert to float in mixed arithmetic
inline vec2 operator-(const ivec2& a, float s) { return vec2(a) - s; }
inline ivec2 operator-(const ivec2& a, const ivec2& b) { return ivec2(a.x - b.x, a.y - b.y); }
inline bool operator==(const ivec2& a, const ivec2& b) { return a.x == b.x && a.y == b.y; }
inline vec4& operator+=(vec4& a, const vec4& b) {
    a.x += b.x, a.y += b.y, a.z += b.z, a.w += b.w;
    return a;
}
template <int N, int A, int B, int C>
inline swz3<N, A, B, C>& operator/=(swz3<N, A, B, C>& s, float d) {
    s.e[A] /= d, s.e[B] /= d, s.e[C] /= d;
    return s;
}
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline uint floatBitsToUint(float f) {
    uint u;
    memcpy(&u, &f, 4);
    return u;
}
inline float uintBitsToFloat(uint u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// ---- storage images ----
enum ImageFormat { IMG_rgba32f, IMG_r11f_g11f_b10f, IMG_rg16f };

// A float rounded to nearest (ties to even) to a float of `mbits` mantissa
// bits and a 5-bit exponent (bias 15), as the 16-bit and the unsigned
// 11-/10-bit formats store it: below 2^-14 in steps of 2^-(14 + mbits)
// (denormals), above in steps of 2^(e - mbits) for 2^e <= |x| < 2^(e + 1),
// to infinity from 2^16 on.  Unsigned formats take negatives to 0.
inline float round_5bit_exponent_float(float x, int mbits, bool is_unsigned) {
    if (__builtin_isnan(x)) return x;
    if (is_unsigned && x < 0.0f) return 0.0f;
    if (__builtin_isinf(x)) return x;
    const float ax = fabsf(x);
    int e2;
    frexpf(ax, &e2);  // ax in [2^(e2 - 1), 2^e2)
    int e = e2 - 1;
    if (e < -14) e = -14;
    const float step = ldexpf(1.0f, e - mbits);
    const float r = nearbyintf(ax / step) * step;  // ax / step is exact
    const float out = r >= 65536.0f ? INFINITY : r;
    return x < 0.0f ? -out : out;
}

struct image2D {
    ImageFormat format;
    float* texels = nullptr;  // row-major, `channels` floats per texel
    int width = 0, height = 0, channels = 4;
    explicit image2D(ImageFormat f) : format(f) {}
};
// Out-of-range loads read 0 and stores are dropped (robust buffer access).
inline vec4 imageLoad(const image2D& im, const ivec2& p) {
    float v[4] = {0.0f, 0.0f, 0.0f, 1.0f};
    if (p.x < 0 || p.y < 0 || p.x >= im.width || p.y >= im.height) return vec4(0.0f);
    const float* t = im.texels + ((size_t)p.y * im.width + p.x) * im.channels;
    const int n = im.format == IMG_rgba32f ? 4 : (im.format == IMG_r11f_g11f_b10f ? 3 : 2);
    for (int c = 0; c < n && c < im.channels; ++c) v[c] = t[c];
    return vec4(v[0], v[1], v[2], v[3]);
}
inline void imageStore(const image2D& im, const ivec2& p, const vec4& v) {
    if (p.x < 0 || p.y < 0 || p.x >= im.width || p.y >= im.height) return;
    float* t = im.texels + ((size_t)p.y * im.width + p.x) * im.channels;
    const float in[4] = {v.x, v.y, v.z, v.w};
    for (int c = 0; c < im.channels; ++c) {
        if (im.format == IMG_rgba32f) t[c] = in[c];
        else if (im.format == IMG_r11f_g11f_b10f)
            t[c] = c < 2 ? round_5bit_exponent_float(in[c], 6, true)
                         : (c == 2 ? round_5bit_exponent_float(in[c], 5, true) : 1.0f);
        else t[c] = c < 2 ? round_5bit_exponent_float(in[c], 10, false) : 0.0f;
    }
}

// ---- invocations, barriers, atomics ----
class WorkgroupBarrier {
  public:
    explicit WorkgroupBarrier(int n) : n_(n) {}
    void wait() {
        std::unique_lock<std::mutex> lk(m_);
        const unsigned long gen = gen_;
        if (++arrived_ == n_) {
            arrived_ = 0;
            ++gen_;
            cv_.notify_all();
        } else {
            cv_.wait(lk, [&] { return gen_ != gen; });
        }
    }
    std::mutex atomics;

  private:
    std::mutex m_;
    std::condition_variable cv_;
    int n_, arrived_ = 0;
    unsigned long gen_ = 0;
};

inline thread_local uvec3 gl_WorkGroupID, gl_LocalInvocationID, gl_GlobalInvocationID;
inline thread_local uint gl_LocalInvocationIndex;
inline thread_local WorkgroupBarrier* gl_current_workgroup = nullptr;

inline void barrier() { gl_current_workgroup->wait(); }
inline void memoryBarrierShared() {}  // threads of one process see each other's stores after barrier()
inline void groupMemoryBarrier() { gl_current_workgroup->wait(); }
inline uint atomicMax(uint& mem, uint v) {
    std::lock_guard<std::mutex> g(gl_current_workgroup->atomics);
    const uint old = mem;
    if (v > old) mem = v;
    return old;
}

// Runs `main` for workgroups 0 .. groups-1 of a one-dimensional dispatch
// with the workgroup size `size`.
inline void dispatch(uint groups, const uvec3& size, void (*main)()) {
    const uint n = size.x * size.y * size.z;
    for (uint g = 0; g < groups; ++g) {
        WorkgroupBarrier wg((int)n);
        std::vector<std::thread> th;
        th.reserve(n);
        for (uint i = 0; i < n; ++i)
            th.emplace_back([&, i] {
                gl_current_workgroup = &wg;
                gl_LocalInvocationIndex = i;
                gl_LocalInvocationID = uvec3(i % size.x, (i / size.x) % size.y, i / (size.x * size.y));
                gl_WorkGroupID = uvec3(g, 0u, 0u);
                gl_GlobalInvocationID = uvec3(g * size.x + gl_LocalInvocationID.x, gl_LocalInvocationID.y,
                                              gl_LocalInvocationID.z);
                main();
            });
        for (auto& t : th) t.join();
    }
}


// ---- resources of the probe-update shaders ----
// ProbeGrid (src/shaders/ProbeGrid.glsl) from the C ABI's grid description;
// G is the shader's ProbeGrid, declared by the shader source.
template <class G, class D>
inline G make_probe_grid(const D* d) {
    G g;
    g.extentMin = vec3(d->extent_min[0], d->extent_min[1], d->extent_min[2]);
    g.depthSharpness = d->depth_sharpness;
    g.extentMax = vec3(d->extent_max[0], d->extent_max[1], d->extent_max[2]);
    g.hysteresis = d->hysteresis;
    g.resolution = ivec3((int)d->resolution[0], (int)d->resolution[1], (int)d->resolution[2]);
    g.raysPerProbe = d->rays_per_probe;
    g.colorRes = d->color_res;
    g.depthRes = d->depth_res;
    g.shadowBias = d->shadow_bias;
    g.padding[0] = 0;
    return g;
}

inline void bind_image(image2D& im, float* texels, int width, int height, int channels) {
    im.texels = texels;
    im.width = width;
    im.height = height;
    im.channels = channels;
}

}  // namespace glsl
